"""Batched ensembles on the GPU: every trajectory of an EnsembleProblem in one persistent,
graph-captured launch (gbca_ensemble_* in include/gbca.h), and rejection ABC on top of it.

`solve_ensemble(eprob, alg, EnsembleGB300(), trajectories=n)` is the counterpart of
`solve(EnsembleProblem(prob), alg, EnsembleThreads(); trajectories=n, save_everystep=false)`
(src/problem.jl:557-589 with SciMLBase's ensemble driver): trajectory i is
`eprob.prob_func(prob, i)` (seed_trajectory by default: seed prob.seed + i), each keeps its
own size, rule and parameters, and the result of trajectory i is
`eprob.output_func(sol, i)` with `sol.u == [u0, u_end]`, `sol.t == [t0, t1]`. The device
also returns each trajectory's state_counts and Moran's I (src/measures.jl) without copying
states back (`states=False`)."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Any, Callable, Optional

import numpy as np

from . import capi
from .backend import _params_tuple, make_desc
from .errors import ArgumentError
from .model import ForestFire, Synchronous
from .problem import CAProblem, CASolution, EnsembleProblem, solve


class EnsembleGB300:
    """The batched ensemble algorithm (the GPU counterpart of EnsembleThreads)."""

    def __repr__(self):
        return "EnsembleGB300()"


class BatchedEnsemble:
    """A set of problems resident on the device, advanced together."""

    def __init__(self, probs, alg=None):
        alg = Synchronous() if alg is None else alg
        self.probs = list(probs)
        if not self.probs:
            raise ArgumentError("an ensemble needs at least one problem")
        descs = (capi.Desc * len(self.probs))()
        for i, p in enumerate(self.probs):
            descs[i] = make_desc(p, alg)
        self.handle = ctypes.c_void_p()
        capi.check(capi.lib().gbca_ensemble_create(descs, len(self.probs), ctypes.byref(self.handle)))
        self.n = len(self.probs)

    def set_initial_states(self):
        for i, p in enumerate(self.probs):
            a = np.asfortranarray(np.asarray(p.u0, dtype=np.int8))
            capi.check(capi.lib().gbca_ensemble_set_state(self.handle, i, a.ctypes.data, a.nbytes))

    def fill(self, value: int):
        capi.check(capi.lib().gbca_ensemble_fill(self.handle, int(value)))

    def run(self, t0=None, nsteps=None, params=None):
        """One launch: instance i from t0[i] for nsteps[i] steps (default: its tspan), with the
        parameters of its problem (or params[i])."""
        n = self.n
        t0 = [p.tspan[0] for p in self.probs] if t0 is None else list(t0)
        nsteps = [p.tspan[1] - p.tspan[0] for p in self.probs] if nsteps is None else list(nsteps)
        vals = []
        for i, p in enumerate(self.probs):
            pv = _params_tuple(p.rule, p.p if params is None else params[i]) if isinstance(p.rule, ForestFire) else ()
            vals.extend(list(pv) + [0.0] * (2 - len(pv)))
        T = (ctypes.c_int64 * n)(*t0)
        S = (ctypes.c_int64 * n)(*nsteps)
        P = (ctypes.c_double * (2 * n))(*vals)
        capi.check(capi.lib().gbca_ensemble_run(self.handle, T, S, P, 2))

    def sync(self):
        capi.check(capi.lib().gbca_ensemble_sync(self.handle))

    def set_geometry(self, tile: int = 128, depth: int = 0):
        """The batched kernel's tile side (64, 128, 192) and steps per pass (0: deepest)."""
        capi.check(capi.lib().gbca_ensemble_set_geometry(self.handle, int(tile), int(depth)))

    def set_large(self, min_cells: int = 1 << 18, steps_per_pass: int = 1):
        """Forest-fire instances of at least min_cells cells (0: none) run as batched multi-CTA
        passes of steps_per_pass steps instead of on one CTA of the persistent kernel."""
        capi.check(capi.lib().gbca_ensemble_set_large(self.handle, int(min_cells), int(steps_per_pass)))

    def geometry(self):
        """dict(tile, depth, large_cells, large_steps, n_large) of the next run."""
        v = [ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()]
        capi.check(capi.lib().gbca_ensemble_geometry(self.handle, *[ctypes.byref(x) for x in v]))
        return dict(zip(("tile", "depth", "large_cells", "large_steps", "n_large"), (int(x.value) for x in v)))

    def tune(self, probe_steps: int = 16, params=None):
        """Times every (tile, depth) on this ensemble's instances for probe_steps steps from
        their current states (restored afterwards), keeps the fastest; returns it."""
        n = self.n
        vals = []
        for i, p in enumerate(self.probs):
            pv = _params_tuple(p.rule, p.p if params is None else params[i]) if isinstance(p.rule, ForestFire) else ()
            vals.extend(list(pv) + [0.0] * (2 - len(pv)))
        P = (ctypes.c_double * (2 * n))(*vals)
        tile, depth = ctypes.c_int32(), ctypes.c_int32()
        capi.check(capi.lib().gbca_ensemble_tune(self.handle, int(probe_steps), P, 2, ctypes.byref(tile),
                                                 ctypes.byref(depth)))
        return int(tile.value), int(depth.value)

    def summaries(self, nvals: int = 3):
        """(counts[n][nvals], other[n], morans[n]) of every instance's state after the last run."""
        n = self.n
        C = (ctypes.c_int64 * (n * nvals))()
        O = (ctypes.c_int64 * n)()
        M = (ctypes.c_double * n)()
        capi.check(capi.lib().gbca_ensemble_summaries(self.handle, C, nvals, O, M))
        counts = np.frombuffer(C, dtype=np.int64).reshape(n, nvals).copy()
        return counts, np.frombuffer(O, dtype=np.int64).copy(), np.frombuffer(M, dtype=np.float64).copy()

    def state(self, i: int) -> np.ndarray:
        p = self.probs[i]
        out = np.empty(p.space.dims, dtype=np.int8, order="F")
        capi.check(capi.lib().gbca_ensemble_get_state(self.handle, int(i), out.ctypes.data, out.nbytes))
        return out

    def close(self):
        if self.handle:
            capi.lib().gbca_ensemble_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class EnsembleResult:
    """Outputs of every trajectory, plus their device summaries."""
    u: list
    counts: np.ndarray
    other: np.ndarray
    morans: np.ndarray


def solve_ensemble(eprob: EnsembleProblem, alg=None, ensemblealg=None, trajectories: int = 1, states: bool = True,
                   nvals: int = 3) -> EnsembleResult:
    """Solve every trajectory of `eprob`: batched on the device for EnsembleGB300() (the
    default), one solve per trajectory otherwise."""
    alg = Synchronous() if alg is None else alg
    probs = [eprob.prob_func(eprob.prob, i) for i in range(1, trajectories + 1)]
    if ensemblealg is not None and not isinstance(ensemblealg, EnsembleGB300):
        outs = []
        for i, p in enumerate(probs, start=1):
            outs.append(eprob.output_func(solve(p, alg, save_everystep=False), i))
        return EnsembleResult(outs, np.zeros((0, nvals), np.int64), np.zeros(0, np.int64), np.zeros(0))
    ens = BatchedEnsemble(probs, alg)
    try:
        ens.set_initial_states()
        ens.run()
        counts, other, morans = ens.summaries(nvals)
        outs = []
        for i, p in enumerate(probs, start=1):
            if states:
                sol = CASolution([np.asfortranarray(np.asarray(p.u0, dtype=np.int8)), ens.state(i - 1)],
                                 [p.tspan[0], p.tspan[1]], p, alg, ensemblealg, "Success")
                outs.append(eprob.output_func(sol, i))
            else:
                outs.append(None)
        return EnsembleResult(outs, counts, other, morans)
    finally:
        ens.close()


@dataclass
class ABCResult:
    """src/calibration.jl:21-27."""
    samples: list
    distances: list
    tolerance: float
    proposals: list
    proposal_distances: list


def abc_rejection(prob: CAProblem, proposals, distance: Callable, observed, keep: Optional[int] = None,
                  tolerance: float = float("inf"), alg=None, ensemblealg=None) -> ABCResult:
    """Rejection ABC (src/calibration.jl:66-91): proposal i runs as trajectory i with
    p = proposals[i] and seed prob.seed + i, scored by distance(sol, observed); the `keep`
    closest proposals within `tolerance` are accepted. Batched on the device by default."""
    ps = list(proposals)
    n = len(ps)
    if n < 1:
        raise ArgumentError("abc_rejection needs at least one proposal")
    keep = max(1, round(n / 20)) if keep is None else int(keep)
    if not 1 <= keep <= n:
        raise ArgumentError(f"keep must be between 1 and the number of proposals ({n}), got {keep}")
    from .problem import seed_trajectory
    eprob = EnsembleProblem(prob, prob_func=lambda pr, i: seed_trajectory(pr, i).remake(p=ps[i - 1]),
                            output_func=lambda sol, i: float(distance(sol, observed)))
    res = solve_ensemble(eprob, alg, EnsembleGB300() if ensemblealg is None else ensemblealg, trajectories=n)
    d = [float(x) for x in res.u]
    order = sorted(range(n), key=lambda i: (np.isnan(d[i]), d[i]))
    accepted = [i for i in order if d[i] <= tolerance][:keep]
    tol = float(tolerance) if not accepted else d[accepted[-1]]
    return ABCResult([ps[i] for i in accepted], [d[i] for i in accepted], tol, ps, d)
