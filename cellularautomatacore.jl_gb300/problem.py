"""Problems, integrators and solutions with the reference's SciML-style interface
(src/problem.jl): CAProblem, init / step / solve, saveat and save_start / save_end,
discrete callbacks that read and modify `integ.u`, remake, seed_trajectory and
EnsembleProblem. The integrator drives any backend through the contract functions; with
GB300Backend the steps between two reads of the state run as one temporally blocked
device call."""
from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import Any, Callable, Optional

import numpy as np

from . import backend as B
from .errors import ArgumentError, StateShapeError, UnsupportedCombinationError
from .model import Constant, Lattice, Moore, Synchronous, Torus


@dataclass(frozen=True)
class CAProblem:
    """CAProblem(rule, u0, tspan, p=None; space, seed, kwargs) (src/problem.jl:67-92)."""
    rule: Any
    u0: Any
    tspan: tuple
    p: Any = None
    space: Any = None
    seed: int = 0
    kwargs: dict = field(default_factory=dict)
    neighbours: Any = None
    covariates: dict = field(default_factory=dict)
    fields: dict = field(default_factory=dict)
    mask: Any = None

    @staticmethod
    def new(rule, u0, tspan, p=None, space=None, seed=0, covariates=None, fields=None, mask=None, **kwargs):
        for k in kwargs:
            if k not in ("callback", "saveat", "save_everystep", "save_start", "save_end", "backend"):
                raise ArgumentError(f"unknown keyword {k}")
        u0 = np.asarray(u0)
        space = Torus(*u0.shape) if space is None else space
        ts = (0, int(tspan)) if np.isscalar(tspan) else (int(tspan[0]), int(tspan[1]))
        if ts[1] < ts[0]:
            raise ArgumentError(f"tspan must not run backwards, got {ts}")
        if tuple(u0.shape) != tuple(space.dims):
            raise StateShapeError(f"the initial state has size {u0.shape}, the space {space.dims}")
        for b in space.boundaries:  # src/state.jl:53-103
            if isinstance(b, Constant) and np.issubdtype(u0.dtype, np.integer):
                info = np.iinfo(u0.dtype)
                if not (float(b.value).is_integer() and info.min <= b.value <= info.max):
                    from .errors import IncompatibleSpaceError
                    raise IncompatibleSpaceError(f"the boundary Constant({b.value}): a state of {u0.dtype} cannot hold it")
        nb = getattr(rule, "neighbourhood", None)
        nb = Moore(1) if nb is None else nb  # default_neighbourhood on a square lattice
        rule.validate_state(u0)
        covariates = dict(covariates or {})
        for k, a in covariates.items():  # src/environment.jl:73-84
            a = np.asarray(a)
            if a.ndim not in (2, 3) or tuple(a.shape[:2]) != tuple(space.dims):
                raise StateShapeError(f"covariate :{k} has size {a.shape}, the space {space.dims}")
        if mask is not None:  # src/environment.jl:123-130
            m = np.asarray(mask)
            if m.dtype != np.bool_:
                raise ArgumentError("mask must be an array of Bools")
            if tuple(m.shape) != tuple(space.dims):
                raise StateShapeError(f"the mask has size {m.shape}, the space {space.dims}")
        fields = dict(fields or {})
        for k, f in fields.items():  # src/environment.jl:53-69
            from .model import KernelField
            if not isinstance(f, KernelField):
                raise ArgumentError(f"field :{k} must be a KernelField, got {type(f).__name__}")
            f.resolve(space, k)
        return CAProblem(rule, u0, ts, p, space, int(seed) % (1 << 64), dict(kwargs), nb, covariates, fields, mask)

    def remake(self, **changes):
        """src/problem.jl:103-113."""
        args = dict(rule=self.rule, u0=self.u0, tspan=self.tspan, p=self.p, space=self.space, seed=self.seed,
                    covariates=self.covariates, fields=self.fields, mask=self.mask)
        kwargs = changes.pop("kwargs", self.kwargs)
        args.update(changes)
        return CAProblem.new(args["rule"], args["u0"], args["tspan"], args["p"], space=args["space"],
                             seed=args["seed"], covariates=args["covariates"], fields=args["fields"],
                             mask=args["mask"], **kwargs)


def remake(prob: CAProblem, **changes) -> CAProblem:
    return prob.remake(**changes)


@dataclass
class CASolution:
    """Saved states u at times t (src/problem.jl:132-139)."""
    u: list
    t: list
    prob: CAProblem
    alg: Any
    backend: Any
    retcode: str


def final_state(sol: CASolution):
    return sol.u[-1]


@dataclass
class DiscreteCallback:
    """condition(u, t, integ) -> bool, then affect(integ) may change integ.u / integ.p."""
    condition: Callable
    affect: Callable
    initialize: Optional[Callable] = None


class CAIntegrator:
    """src/problem.jl:196-236: `u` is fetched from the backend when read."""

    def __init__(self, prob, alg, backend, state, t, saveat, save_everystep, save_end, callbacks):
        self.prob, self.alg, self.backend, self.state = prob, alg, backend, state
        self.t, self.p = t, prob.p
        self.saveat, self.save_everystep, self.save_end = saveat, save_everystep, save_end
        self._sol_u, self._pending = [], []  # saves, and the indices still held as snapshot tickets
        self.sol_t, self.callbacks = [], callbacks
        self.retcode = "Default"
        self._u, self._fresh, self._modified = None, False, False

    @property
    def sol_u(self):
        _fetch_saves(self, 0)
        return self._sol_u

    @sol_u.setter
    def sol_u(self, v):
        _fetch_saves(self, 0)
        self._sol_u = v

    @property
    def u(self):
        if not self._fresh:
            self._u = B.current_state(self.backend, self.state) if isinstance(self.backend, B.GB300Backend) \
                else self.backend.current_state(self.state)
            self._fresh = True
        return self._u

    @u.setter
    def u(self, v):
        v = np.asarray(v)
        if v.shape != tuple(self.prob.space.dims):
            raise StateShapeError(f"state of size {v.shape}, space {self.prob.space.dims}")
        self._u, self._fresh, self._modified = v, True, True

    def u_modified(self, modified: bool):
        self._modified = modified

    def terminate(self):
        self.retcode = "Terminated"


def _b(backend, name):
    return getattr(B, name) if isinstance(backend, B.GB300Backend) else getattr(backend, name)


def _sync(integ):
    """src/problem.jl:292-298."""
    if integ._modified and integ._fresh:
        _b(integ.backend, "set_state")(integ.backend, integ.state, integ._u)
    integ._modified = False


def _should_save(integ):
    """src/problem.jl:336-342."""
    t, (t0, t1) = integ.t, integ.prob.tspan
    if integ.save_end and t == t1:
        return True
    s = integ.saveat
    if s is None:
        return integ.save_everystep
    return (t - t0) % s == 0 if np.isscalar(s) else t in s


class _Snapshot:
    """A saved state still on its way from the device (a gbca_snapshot ticket)."""
    __slots__ = ("ticket",)

    def __init__(self, ticket):
        self.ticket = ticket


def _fetch_saves(integ, keep: int):
    """Collects the oldest pending snapshots until at most `keep` remain."""
    while len(integ._pending) > keep:
        k = integ._pending.pop(0)
        integ._sol_u[k] = B.snapshot_fetch(integ.state, integ._sol_u[k].ticket)


def _save(integ):
    """A save. On the GB300 backend, a state not yet fetched is saved through the device-side
    path: staged on the device and copied out while the sweep goes on (fetched later, at most
    eight in flight); otherwise the integrator's state is copied."""
    if isinstance(integ.backend, B.GB300Backend) and not integ._fresh:
        integ._sol_u.append(_Snapshot(B.snapshot(integ.state)))
        integ._pending.append(len(integ._sol_u) - 1)
        _fetch_saves(integ, 8)
    else:
        integ._sol_u.append(np.array(integ.u, copy=True, order="F"))
    integ.sol_t.append(integ.t)


def init(prob: CAProblem, alg=None, backend=None, saveat=None, save_everystep=None, save_start=True, save_end=True,
         callback=None, seed=None) -> CAIntegrator:
    """src/problem.jl:395-434."""
    alg = Synchronous() if alg is None else alg
    if seed is not None:
        prob = prob.remake(seed=seed)
    kw = dict(prob.kwargs)
    backend = kw.pop("backend", None) if backend is None else backend
    backend = B.GB300Backend() if backend is None else backend
    saveat = kw.get("saveat") if saveat is None else saveat
    if save_everystep is None:
        save_everystep = kw.get("save_everystep", saveat is None)
    if not _b(backend, "supports")(backend, alg):
        raise UnsupportedCombinationError(repr(backend), repr(alg))
    _b(backend, "check_problem")(backend, prob, alg)
    if saveat is not None and np.isscalar(saveat) and saveat <= 0:
        raise ArgumentError(f"saveat must be positive, got {saveat}")
    cbs = []
    for c in (kw.get("callback"), callback):
        if c is None:
            continue
        cbs.extend(c if isinstance(c, (list, tuple)) else [c])
    st = _b(backend, "allocate_state")(backend, prob, alg)
    integ = CAIntegrator(prob, alg, backend, st, prob.tspan[0], saveat, save_everystep, save_end, cbs)
    for cb in cbs:
        if cb.initialize is not None:
            cb.initialize(cb, integ.u, integ.t, integ)
    _sync(integ)
    if save_start:
        _save(integ)
    return integ


def _finished(integ):
    return integ.t >= integ.prob.tspan[1] or integ.retcode == "Terminated"


def step(integ: CAIntegrator, n: int = 1) -> CAIntegrator:
    """src/problem.jl:451-462."""
    adv = _b(integ.backend, "advance")
    for _ in range(n):
        if _finished(integ):
            break
        _sync(integ)
        adv(integ.backend, integ.state, integ.prob, integ.alg, integ.p, integ.t)
        integ.t += 1
        integ._fresh = False
        for cb in integ.callbacks:  # src/problem.jl:440-449
            if cb.condition(integ.u, integ.t, integ):
                integ._modified = True
                cb.affect(integ)
                _sync(integ)
        if _should_save(integ) or integ.retcode == "Terminated":
            _save(integ)
    return integ


def solve_integrator(integ: CAIntegrator) -> CASolution:
    step(integ, integ.prob.tspan[1] - integ.t)
    if integ.retcode == "Default":
        integ.retcode = "Success"
    return CASolution(integ.sol_u, integ.sol_t, integ.prob, integ.alg, integ.backend, integ.retcode)


def reinit(integ: CAIntegrator, u0=None, t0=None) -> CAIntegrator:
    """src/problem.jl:508-531: restart from u0 at t0; the draws restart too."""
    u0 = integ.prob.u0 if u0 is None else u0
    _b(integ.backend, "set_state")(integ.backend, integ.state, u0)
    integ.t = integ.prob.tspan[0] if t0 is None else int(t0)
    integ._fresh = integ._modified = False
    integ.retcode = "Default"
    integ.sol_u, integ.sol_t = [], []
    _save(integ)
    return integ


def solve(prob: CAProblem, alg=None, **kwargs) -> CASolution:
    """src/problem.jl:557-559."""
    return solve_integrator(init(prob, alg, **kwargs))


# ---------------------------------------------------------------- ensembles


def seed_trajectory(prob: CAProblem, sim_id: int, sim_seed=None) -> CAProblem:
    """src/problem.jl:571-574: trajectory i runs with seed prob.seed + i."""
    seed = (prob.seed + int(sim_id)) % (1 << 64) if sim_seed is None else int(sim_seed)
    return prob.remake(seed=seed)


@dataclass
class EnsembleProblem:
    """SciMLBase's EnsembleProblem with prob_func = seed_trajectory by default
    (src/problem.jl:585-589). prob_func(prob, i) and output_func(sol, i) -> value."""
    prob: CAProblem
    prob_func: Callable = lambda prob, i: seed_trajectory(prob, i)
    output_func: Callable = lambda sol, i: sol


def solve_ensemble_serial(eprob: EnsembleProblem, alg=None, trajectories: int = 1, **kwargs):
    """One full solve per trajectory (i = 1..trajectories), as EnsembleSerial does: the
    plain one-solve-per-launch path that the batched ensemble is measured against."""
    out = []
    for i in range(1, trajectories + 1):
        pr = eprob.prob_func(eprob.prob, i)
        out.append(eprob.output_func(solve(pr, alg, **kwargs), i))
    return out
