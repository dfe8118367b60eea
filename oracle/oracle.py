"""CPU oracle for the stencil sweep — TEST INFRASTRUCTURE ONLY.

A ctypes front end over ``gbca_oracle.c`` (a C restatement of
CellularAutomataCore.jl's ReferenceBackend / ArrayBackend per-cell arithmetic)
plus a numpy restatement of the FFTW kernel-field extension. Only the tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm may
import this module, and only as the checker. The product path never does.

Parity pins (the reference, Julia, cannot run here): the Philox4x32-10
known-answer vectors of ``test/test_random.jl:4-14``, the naive Life /
Generations definitions of ``test/test_rules.jl:23-32``, the blinker and glider
patterns ``test/test_rules.jl:109-122``, ``Stochastic(1.0) == Synchronous``
``test/test_schemes.jl:8-9``, Moran's I of a checkerboard ``test/test_extras.jl:140-141``
and Lenia direct-vs-FFT ``test/test_extras.jl:121-123``; see ``tests/test_oracle.py``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

RULE_LIFE, RULE_GENERATIONS, RULE_FOREST_FIRE, RULE_SI_FIELD = 1, 2, 3, 5
# dispersal kernel kinds of or_kernel_weights
K_GAUSSIAN, K_EXPONENTIAL, K_POWERLAW, K_UNIFORM, K_LENIA, K_ANISOTROPIC, K_EMPIRICAL = 1, 2, 3, 4, 5, 6, 7
MOORE, VON_NEUMANN = 1, 2
PERIODIC, REFLECTING, CONSTANT = 0, 1, 2
SYNCHRONOUS, STOCHASTIC, CHECKERBOARD = 0, 1, 2


class OrProblem(ctypes.Structure):
    _fields_ = [
        ("rule", ctypes.c_int32), ("nbhd", ctypes.c_int32), ("radius", ctypes.c_int32),
        ("states", ctypes.c_int32), ("birth", ctypes.c_uint64), ("survive", ctypes.c_uint64),
        ("n1", ctypes.c_int64), ("n2", ctypes.c_int64), ("boundary", ctypes.c_int32 * 2),
        ("constant", ctypes.c_int32 * 2), ("seed", ctypes.c_uint64), ("scheme", ctypes.c_int32),
        ("scheme_p_f32", ctypes.c_int32), ("scheme_p", ctypes.c_double),
        ("params_f32", ctypes.c_int32), ("_pad", ctypes.c_int32),
    ]


class OrEnv(ctypes.Structure):
    _fields_ = [
        ("mask", ctypes.c_void_p), ("ntaps", ctypes.c_int32), ("field_f32", ctypes.c_int32),
        ("taps", ctypes.c_void_p), ("weights", ctypes.c_void_p), ("cov", ctypes.c_void_p),
        ("cov_nt", ctypes.c_int64), ("cov_f32", ctypes.c_int32), ("source", ctypes.c_int32),
    ]


def build() -> str:
    """Compile the oracle with its Makefile (gcc); returns the library path."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        L.or_philox4x32.argtypes = [P(ctypes.c_uint32), P(ctypes.c_uint32), P(ctypes.c_uint32)]
        L.or_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int64, ctypes.c_uint32]
        L.or_uniform.restype = ctypes.c_double
        L.or_uniform32.argtypes = L.or_uniform.argtypes
        L.or_uniform32.restype = ctypes.c_float
        L.or_offsets.argtypes = [ctypes.c_int32, ctypes.c_int32, P(ctypes.c_int32)]
        L.or_step_reference.argtypes = [P(OrProblem), ctypes.c_void_p, ctypes.c_int64, P(ctypes.c_double)]
        L.or_run_array.argtypes = [P(OrProblem), ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                   P(ctypes.c_double), ctypes.c_int32]
        L.or_state_counts.argtypes = [ctypes.c_void_p, ctypes.c_int64, P(ctypes.c_int64), ctypes.c_int32,
                                      P(ctypes.c_int64)]
        L.or_morans_i.argtypes = [P(OrProblem), ctypes.c_void_p]
        L.or_morans_i.restype = ctypes.c_double
        L.or_soup.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p]
        L.or_step_reference_env.argtypes = [P(OrProblem), P(OrEnv), ctypes.c_void_p, ctypes.c_int64,
                                            P(ctypes.c_double)]
        L.or_run_array_env.argtypes = [P(OrProblem), P(OrEnv), ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                       P(ctypes.c_double), ctypes.c_int32]
        L.or_kernel_field.argtypes = [P(OrProblem), P(OrEnv), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.or_kernel_weights.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int32, P(ctypes.c_double), ctypes.c_int32,
                                        P(ctypes.c_double), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                        P(ctypes.c_int32), P(ctypes.c_double)]
        L.or_lenia_weights.argtypes = [ctypes.c_int32, P(ctypes.c_double), ctypes.c_int32,
                                       P(ctypes.c_int32), P(ctypes.c_double)]
        for name in ("or_lenia_step_f64", "or_lenia_step_f32"):
            getattr(L, name).argtypes = [ctypes.c_int64, ctypes.c_int64, P(ctypes.c_int32), ctypes.c_void_p,
                                         ctypes.c_int32, P(ctypes.c_double), ctypes.c_int32, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_int32]
        _lib = L
    return _lib


# ----------------------------------------------------------------- problems


@dataclass
class Problem:
    """Everything the oracle needs about an Int8 problem (rule, lattice, seed, scheme)."""
    rule: int
    n1: int
    n2: int
    nbhd: int = MOORE
    radius: int = 1
    birth: int = 0
    survive: int = 0
    states: int = 2
    boundary: tuple = (PERIODIC, PERIODIC)
    constant: tuple = (0, 0)
    seed: int = 0
    scheme: int = SYNCHRONOUS
    scheme_p: float = 1.0
    scheme_p_f32: bool = False
    params_f32: bool = False

    def c(self) -> OrProblem:
        p = OrProblem()
        p.rule, p.nbhd, p.radius, p.states = self.rule, self.nbhd, self.radius, self.states
        p.birth, p.survive = self.birth, self.survive
        p.n1, p.n2 = self.n1, self.n2
        p.boundary[0], p.boundary[1] = self.boundary
        p.constant[0], p.constant[1] = self.constant
        p.seed = self.seed % (1 << 64)
        p.scheme, p.scheme_p, p.scheme_p_f32 = self.scheme, self.scheme_p, int(self.scheme_p_f32)
        p.params_f32 = int(self.params_f32)
        return p


def mask(counts) -> int:
    """rules.jl:267-275: bit c set for every count c (0..63)."""
    m = 0
    for c in counts:
        if not 0 <= c <= 63:
            raise ValueError(f"neighbour counts must be in 0:63, got {c}")
        m |= 1 << c
    return m


def _params(params) -> ctypes.Array:
    vals = list(params) if params is not None else []
    vals += [0.0] * (4 - len(vals))
    return (ctypes.c_double * len(vals))(*vals)


def _u8(u: np.ndarray) -> np.ndarray:
    """A Fortran-ordered (column-major, axis 1 contiguous) Int8 copy."""
    return np.asfortranarray(np.array(u, dtype=np.int8, copy=True))


@dataclass
class Env:
    """A sweep's environment: mask (True = the cell updates), one kernel field (taps to
    read and FP64 weights, Float32 when field_f32) and one covariate (n1 x n2 or
    n1 x n2 x nt, Float64 or Float32)."""
    mask: np.ndarray | None = None
    taps: np.ndarray | None = None
    weights: np.ndarray | None = None
    field_f32: bool = False
    cov: np.ndarray | None = None
    identity: bool = False       # field source x itself instead of x == 1

    def c(self):
        e = OrEnv()
        e.source = int(self.identity)
        keep = []
        if self.mask is not None:
            m = np.asfortranarray(np.asarray(self.mask, dtype=np.uint8))
            keep.append(m)
            e.mask = m.ctypes.data
        if self.taps is not None:
            t = np.ascontiguousarray(np.asarray(self.taps, dtype=np.int32).reshape(-1, 2))
            w = np.ascontiguousarray(np.asarray(self.weights, dtype=np.float64))
            keep += [t, w]
            e.ntaps, e.taps, e.weights, e.field_f32 = len(w), t.ctypes.data, w.ctypes.data, int(self.field_f32)
        if self.cov is not None:
            c = np.asfortranarray(self.cov)
            keep.append(c)
            e.cov, e.cov_nt = c.ctypes.data, (c.shape[2] if c.ndim == 3 else 1)
            e.cov_f32 = int(c.dtype == np.float32)
        return e, keep


def kernel_weights(kind: int, radius: int, a: float = 0.0, *, base: int = 0, direction: float = 0.0,
                   strength: float = 0.0, peaks=(1.0,), empirical=None, include_centre: bool = True):
    """kernels.jl:174-203 then environment.jl:60-63: (taps to read as (di, dj) rows, weights)."""
    pk = (ctypes.c_double * max(1, len(peaks)))(*peaks)
    if empirical is not None:
        E = np.asfortranarray(np.asarray(empirical, dtype=np.float64))
        cap = E.size
        emp, e1, e2 = E.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), E.shape[0], E.shape[1]
    else:
        cap = (2 * radius + 1) ** 2
        emp, e1, e2 = None, 0, 0
    off = (ctypes.c_int32 * (2 * cap))()
    w = (ctypes.c_double * cap)()
    m = lib().or_kernel_weights(kind, base, a, direction, strength, radius, pk, len(peaks), emp, e1, e2,
                                int(include_centre), off, w)
    if m < 0:
        raise ValueError("the kernel has no positive weight")
    return np.array(off[:2 * m], dtype=np.int32).reshape(m, 2), np.array(w[:m])


def kernel_field(prob: Problem, env: Env, u: np.ndarray):
    """environment.jl:151-160: the field of every cell (Float64, or Float32 when env.field_f32)."""
    a = _u8(u)
    e, keep = env.c()
    f64 = np.zeros(a.shape, dtype=np.float64, order="F")
    f32 = np.zeros(a.shape, dtype=np.float32, order="F")
    rc = lib().or_kernel_field(ctypes.byref(prob.c()), ctypes.byref(e), a.ctypes.data, f64.ctypes.data,
                               f32.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"or_kernel_field failed: {rc}")
    return f32 if env.field_f32 else f64


def step_reference_env(prob: Problem, env: Env, u: np.ndarray, t: int, params=None) -> np.ndarray:
    """One step with an environment (ReferenceBackend semantics)."""
    a = _u8(u)
    e, keep = env.c()
    rc = lib().or_step_reference_env(ctypes.byref(prob.c()), ctypes.byref(e), a.ctypes.data, t, _params(params))
    if rc != 0:
        raise RuntimeError(f"or_step_reference_env failed: {rc}")
    return a


def run_array_env(prob: Problem, env: Env, u: np.ndarray, t0: int, nsteps: int, params=None,
                  nthreads: int = 1) -> np.ndarray:
    """nsteps steps with an environment (ArrayBackend semantics)."""
    a = _u8(u)
    e, keep = env.c()
    rc = lib().or_run_array_env(ctypes.byref(prob.c()), ctypes.byref(e), a.ctypes.data, t0, nsteps,
                                _params(params), nthreads)
    if rc != 0:
        raise RuntimeError(f"or_run_array_env failed: {rc}")
    return a


def step_reference(prob: Problem, u: np.ndarray, t: int, params=None) -> np.ndarray:
    """One step t -> t+1, ReferenceBackend semantics (backends.jl:264-278,314-322)."""
    a = _u8(u)
    rc = lib().or_step_reference(ctypes.byref(prob.c()), a.ctypes.data, t, _params(params))
    if rc != 0:
        raise RuntimeError(f"or_step_reference failed: {rc}")
    return a


def run_array(prob: Problem, u: np.ndarray, t0: int, nsteps: int, params=None, nthreads: int = 1) -> np.ndarray:
    """nsteps steps from t0, ArrayBackend semantics (backends.jl:408-506), threaded slabs."""
    a = _u8(u)
    rc = lib().or_run_array(ctypes.byref(prob.c()), a.ctypes.data, t0, nsteps, _params(params), nthreads)
    if rc != 0:
        raise RuntimeError(f"or_run_array failed: {rc}")
    return a


def solve(prob: Problem, u0: np.ndarray, tspan, saveat=None, params=None, nthreads: int = 1):
    """problem.jl:336-370,451-462: saved times and states of a Synchronous run (no callbacks)."""
    t0, t1 = (0, int(tspan)) if np.isscalar(tspan) else (int(tspan[0]), int(tspan[1]))
    ts, us = [t0], [_u8(u0)]
    u, t = _u8(u0), t0
    while t < t1:
        if saveat is None:
            nxt = t + 1
        else:
            nxt = min(t1, t0 + ((t - t0) // saveat + 1) * saveat)
        u = run_array(prob, u, t, nxt - t, params, nthreads)
        t = nxt
        ts.append(t)
        us.append(u.copy())
    return ts, us


def philox4x32(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().or_philox4x32(c, k, o)
    return tuple(int(x) for x in o)


def uniform(seed: int, cellid: int, t: int, k: int = 1) -> float:
    return lib().or_uniform(seed % (1 << 64), cellid, t, k)


def uniform32(seed: int, cellid: int, t: int, k: int = 1) -> float:
    return lib().or_uniform32(seed % (1 << 64), cellid, t, k)


def offsets(nbhd: int, radius: int):
    buf = (ctypes.c_int32 * (2 * (2 * radius + 1) ** 2))()
    m = lib().or_offsets(nbhd, radius, buf)
    return [(buf[2 * k], buf[2 * k + 1]) for k in range(m)]


def state_counts(u: np.ndarray, nvals: int = 3):
    a = _u8(u)
    c = (ctypes.c_int64 * nvals)()
    other = ctypes.c_int64()
    lib().or_state_counts(a.ctypes.data, a.size, c, nvals, ctypes.byref(other))
    return [int(x) for x in c], int(other.value)


def morans_i(prob: Problem, u: np.ndarray) -> float:
    a = _u8(u)
    return lib().or_morans_i(ctypes.byref(prob.c()), a.ctypes.data)


def soup(seed: int, n1: int, n2: int, density: float) -> np.ndarray:
    """The backend's device-generated Bernoulli(density) soup of 0/1 (an n1 x n2 Int8 state)."""
    a = np.zeros((n1, n2), dtype=np.int8, order="F")
    lib().or_soup(seed % (1 << 64), n1, n2, density, a.ctypes.data)
    return a


# ----------------------------------------------------------------- Lenia


def lenia_weights(R: int = 13, peaks=(1.0,)):
    """kernels.jl:174-189 + environment.jl:60-63: (offsets to read, FP64 weights)."""
    cap = (2 * R + 1) ** 2
    off = (ctypes.c_int32 * (2 * cap))()
    w = (ctypes.c_double * cap)()
    pk = (ctypes.c_double * len(peaks))(*peaks)
    m = lib().or_lenia_weights(R, pk, len(peaks), off, w)
    return np.array([(off[2 * k], off[2 * k + 1]) for k in range(m)], dtype=np.int64), np.array(w[:m])


def lenia_step_direct(u: np.ndarray, R=13, peaks=(1.0,), mu=0.15, sigma=0.015, dt=0.1,
                      boundary=(PERIODIC, PERIODIC), f32=False, nthreads: int = 1) -> np.ndarray:
    """One Lenia step with the direct field (environment.jl:151-160, lenia.jl:42-47)."""
    a = np.asfortranarray(np.array(u, dtype=np.float32 if f32 else np.float64, copy=True))
    bnd = (ctypes.c_int32 * 2)(*boundary)
    pk = (ctypes.c_double * len(peaks))(*peaks)
    fn = lib().or_lenia_step_f32 if f32 else lib().or_lenia_step_f64
    rc = fn(a.shape[0], a.shape[1], bnd, a.ctypes.data, R, pk, len(peaks), mu, sigma, dt, nthreads)
    if rc != 0:
        raise RuntimeError("lenia step failed")
    return a


class LeniaFFT:
    """ext/CellularAutomataCoreFFTWExt.jl:17-30 in numpy, FP64: the field is
    irfft(rfft(src) .* conj(rfft(kpad))) with the kernel wrapped by mod1(o + 1, dims)."""

    def __init__(self, n1: int, n2: int, R=13, peaks=(1.0,)):
        off, w = lenia_weights(R, peaks)
        kpad = np.zeros((n1, n2))
        for (o1, o2), wk in zip(off, w):
            kpad[o1 % n1, o2 % n2] += wk
        self.kf = np.conj(np.fft.rfft2(kpad))
        self.shape = (n1, n2)

    def field(self, u: np.ndarray) -> np.ndarray:
        return np.fft.irfft2(np.fft.rfft2(np.asarray(u, dtype=np.float64)) * self.kf, s=self.shape)

    def step(self, u: np.ndarray, mu=0.15, sigma=0.015, dt=0.1) -> np.ndarray:
        U = self.field(u)
        g = 2.0 * np.exp(-((U - mu) * (U - mu)) / (2.0 * (sigma * sigma))) - 1.0
        return np.clip(np.asarray(u, dtype=np.float64) + dt * g, 0.0, 1.0)
