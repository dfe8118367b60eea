"""GB300Backend: the reference's backend contract (src/backends.jl:4-14) implemented over
libgbca.so. Method names follow the contract with Julia's `!` dropped:

    supports(backend, scheme)                    src/backends.jl:89-95
    check_problem(backend, prob, scheme)         src/backends.jl:97-105
    allocate_state(backend, prob, scheme)        src/backends.jl:107-119
    advance(backend, state, prob, scheme, p, t)  src/backends.jl:121-130  (advance!)
    current_state(backend, state)                src/backends.jl:132-139
    set_state(backend, state, u)                 src/backends.jl:141-148  (set_state!)
    read_cell / write_cell                       src/backends.jl:380-383  (write_cell!)

`advance` is one step from t to t + 1, as the integrator calls it (src/problem.jl:455).
The backend queues consecutive steps and hands them to the library as one call when
anything reads or replaces the state, or when the parameters change, so the device runs
them temporally blocked. Results are those of ReferenceBackend, bit for bit for the Int8
rules (draws keyed as src/random.jl:102-107)."""
from __future__ import annotations

import ctypes
import hashlib

import numpy as np

from . import capi
from .errors import ArgumentError, IncompatibleSpaceError, StateShapeError, UnsupportedCombinationError
from .model import (Checkerboard, Constant, ForestFire, Generations, KernelSI, Lattice, Lenia, Life, Moore,
                    Stochastic, Synchronous, VonNeumann)


class GB300Backend:
    """Run the sweep on the GPU through libgbca.so (hand-written sm_103a kernels).
    Needs a CUDA device; there is no CPU fallback.

    `background` switches on active-tile sweeps, the GPU form of
    SparseBackend(background; tilesize) (src/sparse.jl): only tiles holding a non-background
    cell, and tiles within reach of them, are swept. The rule must be quiescent."""

    def __init__(self, background=None, tilesize: int = 64):
        self.background, self.tilesize = background, int(tilesize)

    def __repr__(self):
        if self.background is None:
            return "GB300Backend()"
        return f"GB300Backend(background={self.background}, tilesize={self.tilesize})"

    def __eq__(self, other):
        return isinstance(other, GB300Backend) and (self.background, self.tilesize) == \
            (other.background, other.tilesize)

    def __hash__(self):
        return hash(("GB300Backend", self.background, self.tilesize))


def supports(backend, scheme) -> bool:
    """src/backends.jl:153: the gated synchronous schemes; active-tile sweeps run
    Synchronous and Stochastic, as SparseBackend (src/sparse.jl:40)."""
    if not isinstance(backend, GB300Backend):
        return False
    if backend.background is not None:
        return isinstance(scheme, (Synchronous, Stochastic))
    return isinstance(scheme, (Synchronous, Stochastic, Checkerboard))


def _params_tuple(rule, p):
    """The rule's numbers from the integrator's p: forest fire reads p.p and p.f, the
    kernel-field SI rule p.β (or p.beta)."""
    if isinstance(rule, KernelSI):
        if p is None:
            raise ArgumentError("the kernel-field SI rule needs its parameter β")
        if isinstance(p, dict):
            beta = p["β"] if "β" in p else p["beta"]
        else:
            beta = getattr(p, "β", None)
            beta = getattr(p, "beta") if beta is None else beta
        return (float(np.float32(beta)) if rule.float32 else float(beta),)
    if not isinstance(rule, ForestFire):
        return ()
    if p is None:
        raise ArgumentError("the forest-fire rule needs parameters (p=..., f=...)")
    get = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    vals = (float(get("p")), float(get("f")))
    if rule.float32:
        vals = tuple(float(np.float32(v)) for v in vals)
    return vals


def make_desc(prob, scheme) -> capi.Desc:
    """The gbca_desc of a problem; raises the reference's errors for what the backend
    cannot run (the checks of check_problem)."""
    space, rule = prob.space, prob.rule
    if not isinstance(space, Lattice):
        raise IncompatibleSpaceError("GB300Backend needs a lattice")
    d = capi.Desc()
    d.n1, d.n2 = space.dims
    for a, b in enumerate(space.boundaries):
        d.boundary[a] = b.kind
        d.constant[a] = float(b.value) if isinstance(b, Constant) else 0.0
    d.seed = int(prob.seed) % (1 << 64)
    if isinstance(scheme, Stochastic):
        d.scheme, d.scheme_p, d.scheme_p_f32 = capi.STOCHASTIC, scheme.p, int(scheme.float32)
    elif isinstance(scheme, Checkerboard):
        d.scheme = capi.CHECKERBOARD
    else:
        d.scheme = capi.SYNCHRONOUS
    if isinstance(rule, Lenia):
        d.rule = capi.RULE_LENIA
        d.lenia_method = capi.FFT if rule.method == "fft" else capi.DIRECT
        d.lenia_R, d.lenia_npeaks = rule.R, len(rule.peaks)
        if len(rule.peaks) > capi.MAX_PEAKS:
            raise ArgumentError(f"GB300Backend runs Lenia with at most {capi.MAX_PEAKS} peaks")
        for k, v in enumerate(rule.peaks):
            d.lenia_peaks[k] = v
        d.lenia_mu, d.lenia_sigma, d.lenia_dt = rule.mu, rule.sigma, rule.dt
        d.lenia_f64 = int(rule.precision == "Float64")
        want = np.float64 if d.lenia_f64 else np.float32
        if np.asarray(prob.u0).dtype != want:
            raise ArgumentError(f"Lenia(precision={rule.precision}) needs a {rule.precision} state")
        return d
    nb = prob.neighbours
    if not isinstance(nb, (Moore, VonNeumann)):
        raise ArgumentError("GB300Backend runs Moore(r) and VonNeumann(r) neighbourhoods")
    d.nbhd, d.radius = nb.kind, nb.radius
    if np.asarray(prob.u0).dtype != np.int8:
        raise ArgumentError("GB300Backend runs Life, Generations and forest-fire rules on Int8 states")
    if isinstance(rule, Life):
        d.rule, d.birth, d.survive, d.states = capi.RULE_LIFE, rule.birth, rule.survive, 2
    elif isinstance(rule, Generations):
        d.rule, d.birth, d.survive, d.states = capi.RULE_GENERATIONS, rule.birth, rule.survive, rule.states
    elif isinstance(rule, ForestFire):
        d.rule, d.params_f32 = capi.RULE_FOREST_FIRE, int(rule.float32)
    elif isinstance(rule, KernelSI):
        d.rule, d.params_f32 = capi.RULE_SI_FIELD, int(rule.float32)
        if rule.field not in prob.fields:
            raise ArgumentError(f"the rule reads field :{rule.field}, which the problem does not define")
        if rule.covariate is not None and rule.covariate not in prob.covariates:
            raise ArgumentError(f"the rule reads covariate :{rule.covariate}, which the problem does not define")
    else:
        raise ArgumentError(f"GB300Backend cannot run {type(rule).__name__}: arbitrary LocalRules cannot cross "
                            "the C ABI; use Life, Generations, ForestFire or Lenia")
    return d


def check_problem(backend, prob, scheme) -> None:
    d = make_desc(prob, scheme)
    capi.check(capi.lib().gbca_check(ctypes.byref(d)))


class GB300State:
    """The backend's state: a library handle plus the queue of steps not yet run."""

    def __init__(self, desc: capi.Desc, dtype):
        self.desc, self.dtype = desc, np.dtype(dtype)
        self.dims = (int(desc.n1), int(desc.n2))
        self.handle = ctypes.c_void_p()
        capi.check(capi.lib().gbca_create(ctypes.byref(desc), ctypes.byref(self.handle)))
        self.pending, self.pending_t0, self.pending_params = 0, 0, ()

    def flush(self):
        if self.pending:
            vals = self.pending_params
            arr = (ctypes.c_double * max(1, len(vals)))(*vals)
            n, self.pending = self.pending, 0
            capi.check(capi.lib().gbca_advance(self.handle, self.pending_t0, n, arr, len(vals)))

    def close(self):
        if self.handle:
            capi.lib().gbca_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def nbytes(self):
        return self.dims[0] * self.dims[1] * self.dtype.itemsize


def _attach_environment(st: GB300State, prob) -> None:
    """The problem's mask, the SI rule's kernel field and covariate, on the device."""
    L = capi.lib()
    if prob.mask is not None:
        if st.desc.rule == capi.RULE_LENIA:
            raise ArgumentError("GB300Backend runs masks with Int8 rules only")
        m = np.asfortranarray(np.asarray(prob.mask, dtype=np.uint8))
        capi.check(L.gbca_set_mask(st.handle, m.ctypes.data, m.nbytes))
    rule = prob.rule
    if isinstance(rule, KernelSI):
        f = prob.fields[rule.field]
        taps, weights, _ = f.resolve(prob.space, rule.field)
        t = np.ascontiguousarray(np.asarray(taps, dtype=np.int32).reshape(-1))
        w = np.ascontiguousarray(weights, dtype=np.float64)
        capi.check(L.gbca_set_field(st.handle, len(w), t.ctypes.data, w.ctypes.data, int(f.precision == "Float32"),
                                    capi.SOURCE_INDICATOR if f.source == "x == 1" else capi.SOURCE_IDENTITY,
                                    capi.FFT if f.method == "fft" else capi.DIRECT))
        if rule.covariate is not None:
            c = np.asarray(prob.covariates[rule.covariate])
            f32 = c.dtype == np.float32
            c = np.asfortranarray(c.astype(np.float32 if f32 else np.float64, copy=False))
            nt = c.shape[2] if c.ndim == 3 else 1
            capi.check(L.gbca_set_covariate(st.handle, c.ctypes.data, nt, int(f32)))


def allocate_state(backend, prob, scheme) -> GB300State:
    d = make_desc(prob, scheme)
    dtype = (np.float64 if d.lenia_f64 else np.float32) if d.rule == capi.RULE_LENIA else np.int8
    st = GB300State(d, dtype)
    _attach_environment(st, prob)
    if getattr(backend, "background", None) is not None:
        if not supports(backend, scheme):
            raise UnsupportedCombinationError(repr(backend), repr(scheme))
        capi.check(capi.lib().gbca_set_sparse(st.handle, 1, int(backend.background), backend.tilesize))
    set_state(backend, st, prob.u0)
    return st


def advance(backend, st: GB300State, prob, scheme, p, t: int) -> None:
    """One step t -> t + 1 (queued)."""
    params = _params_tuple(prob.rule, p)
    if st.pending and st.pending_t0 + st.pending == t and params == st.pending_params:
        st.pending += 1
        return
    st.flush()
    st.pending_t0, st.pending, st.pending_params = int(t), 1, params


def current_state(backend, st: GB300State) -> np.ndarray:
    """A host copy in the layout of u0 (column-major)."""
    st.flush()
    out = np.empty(st.dims, dtype=st.dtype, order="F")
    capi.check(capi.lib().gbca_get_state(st.handle, out.ctypes.data, out.nbytes))
    return out


def set_state(backend, st: GB300State, u) -> None:
    st.flush()
    a = np.asarray(u)
    if a.shape != st.dims:
        raise StateShapeError(f"the state has size {a.shape}, the space {st.dims}")
    a = np.asfortranarray(a.astype(st.dtype, copy=False))
    capi.check(capi.lib().gbca_set_state(st.handle, a.ctypes.data, a.nbytes))


def read_cell(backend, st: GB300State, I):
    st.flush()
    i, j = I
    out = np.zeros(1, dtype=st.dtype)
    capi.check(capi.lib().gbca_read_cell(st.handle, int(i), int(j), out.ctypes.data))
    return out[0]


def write_cell(backend, st: GB300State, I, v) -> None:
    st.flush()
    i, j = I
    val = np.array([v], dtype=st.dtype)
    capi.check(capi.lib().gbca_write_cell(st.handle, int(i), int(j), val.ctypes.data))


# the last lattice update_cell stepped: (problem, time, parameters, digest of the state) and
# the stepped state, so a loop over every cell of one state costs one sweep
_UPDATE_CELL_CACHE: dict = {}


def update_cell(prob, u, I, t: int, p=None):
    """The new state of cell I when the whole state u (in the layout of prob.u0) is updated
    synchronously at time t with parameters p (default prob.p), without changing u: the rule
    applied to the cell and its neighbours under the space's boundaries, with the problem's
    mask and the draws every backend makes (src/backends.jl:281-307). I is a 1-based (i, j)
    or a 1-based column-major linear index.

    Computed on the GPU: u goes through one Synchronous sweep of this backend's kernels and
    cell I is read back. The stepped lattice is kept for the next call with the same problem,
    time, parameters and state, so asking for every cell costs one sweep. As in the
    reference, problems with kernel fields (the SI rule, Lenia) are refused."""
    if prob.fields or isinstance(prob.rule, (KernelSI, Lenia)):
        raise ArgumentError("update_cell does not compute kernel fields; use GB300Backend's sweep")
    a = np.asarray(u)
    n1, n2 = prob.space.dims
    if a.shape != (n1, n2):
        raise StateShapeError(f"the state has size {a.shape}, the space {(n1, n2)}")
    if isinstance(I, (int, np.integer)):
        if not 1 <= int(I) <= n1 * n2:
            raise ArgumentError(f"cell index {I} is outside 1:{n1 * n2}")
        i, j = (int(I) - 1) % n1 + 1, (int(I) - 1) // n1 + 1
    else:
        i, j = (int(x) for x in I)
        if not (1 <= i <= n1 and 1 <= j <= n2):
            raise ArgumentError(f"cell index ({i}, {j}) is outside the {n1} x {n2} lattice")
    params = prob.p if p is None else p
    a8 = np.asfortranarray(a.astype(np.int8, copy=False))
    key = (id(prob), int(t), _params_tuple(prob.rule, params), hashlib.blake2b(a8.tobytes(order="F")).hexdigest())
    hit = _UPDATE_CELL_CACHE.get("key")
    if hit != key:
        st = allocate_state(GB300Backend(), prob, Synchronous())
        try:
            set_state(None, st, a8)
            advance(None, st, prob, Synchronous(), params, int(t))
            stepped = current_state(None, st)
        finally:
            st.close()
        _UPDATE_CELL_CACHE.clear()
        _UPDATE_CELL_CACHE.update(key=key, state=stepped, prob=prob)  # prob kept alive: its id stays unique
    return _UPDATE_CELL_CACHE["state"][i - 1, j - 1]


def snapshot(st: GB300State) -> int:
    """Queues a copy of the state after the queued steps (device staging, asynchronous copy
    to pinned memory); returns a ticket for snapshot_fetch."""
    st.flush()
    ticket = ctypes.c_int64()
    capi.check(capi.lib().gbca_snapshot(st.handle, ctypes.byref(ticket)))
    return int(ticket.value)


def snapshot_fetch(st: GB300State, ticket: int) -> np.ndarray:
    """The state a snapshot captured (column-major, as u0)."""
    out = np.empty(st.dims, dtype=st.dtype, order="F")
    capi.check(capi.lib().gbca_snapshot_fetch(st.handle, int(ticket), out.ctypes.data, out.nbytes))
    return out


def device_summaries(st: GB300State, nvals: int = 3):
    """state_counts (src/measures.jl:14-20) and Moran's I (src/measures.jl:91-107) of the
    current state, computed on the device: (counts[0:nvals], cells outside, morans)."""
    st.flush()
    counts = (ctypes.c_int64 * max(1, nvals))()
    other = ctypes.c_int64()
    mi = ctypes.c_double()
    capi.check(capi.lib().gbca_summaries(st.handle, counts, nvals, ctypes.byref(other), ctypes.byref(mi)))
    return [int(counts[k]) for k in range(nvals)], int(other.value), float(mi.value)


def tune(st: GB300State, prob=None, p=None):
    """Times the candidate sweep geometries of the state's fast kernel on its current state
    (restored afterwards) and caches the fastest for the problem's shape; returns
    (steps per pass, tile rows, staging), (0, 0, 0) when the problem runs on the general kernel."""
    st.flush()
    vals = _params_tuple(prob.rule, p if p is not None else prob.p) if prob is not None else ()
    arr = (ctypes.c_double * max(1, len(vals)))(*vals)
    k, rows, staging = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    capi.check(capi.lib().gbca_tune(st.handle, arr, len(vals), ctypes.byref(k), ctypes.byref(rows),
                                    ctypes.byref(staging)))
    return int(k.value), int(rows.value), int(staging.value)


def set_geometry(st: GB300State, steps_per_pass: int = 0, tile_rows: int = 0, staging: int = 0) -> None:
    """Pins the state's sweep geometry (staging 1: the forest fire's tiles by TMA); (0, 0, 0)
    returns it to the tuned or default one."""
    st.flush()
    capi.check(capi.lib().gbca_set_geometry(st.handle, int(steps_per_pass), int(tile_rows), int(staging)))
