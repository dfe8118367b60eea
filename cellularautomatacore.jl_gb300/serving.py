"""Serving: simulation requests of different rules, sizes and step counts, admitted by HBM
budget into a device-resident loop that batches them continuously (gbca_server_* in
include/gbca.h). A request is a CAProblem plus a step count; its result is the summary the
reference computes from a final state: state_counts and morans_i (src/measures.jl)."""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import capi
from .backend import _params_tuple, make_desc
from .model import ForestFire, Synchronous


class Server:
    """A running request loop on the current GPU."""

    def __init__(self, hbm_budget: int = 8 << 30, chunk_steps: int = 64, big_cells: int = 1 << 20, max_big: int = 8,
                 big_chunk_us: int = 0):
        cfg = capi.ServerConfig()
        cfg.hbm_budget, cfg.chunk_steps, cfg.big_cells, cfg.max_big = int(hbm_budget), int(chunk_steps), \
            int(big_cells), int(max_big)
        cfg.big_chunk_us = int(big_chunk_us)
        self.handle = ctypes.c_void_p()
        capi.check(capi.lib().gbca_server_start(ctypes.byref(cfg), ctypes.byref(self.handle)))

    def submit(self, prob, nsteps=None, t0=None, density=None, init_seed=0) -> int:
        """Queue `prob` for `nsteps` steps (default: its tspan) from t0. With `density`, the
        initial state is a Bernoulli(density) soup of 0/1 drawn on the device from
        `init_seed` instead of prob.u0."""
        d = make_desc(prob, Synchronous())
        t0 = prob.tspan[0] if t0 is None else int(t0)
        nsteps = prob.tspan[1] - prob.tspan[0] if nsteps is None else int(nsteps)
        pv = _params_tuple(prob.rule, prob.p) if isinstance(prob.rule, ForestFire) else ()
        P = (ctypes.c_double * 2)(*(list(pv) + [0.0] * (2 - len(pv))))
        rid = ctypes.c_uint64()
        if density is None:
            a = np.asfortranarray(np.asarray(prob.u0, dtype=np.int8))
            rc = capi.lib().gbca_server_submit(self.handle, ctypes.byref(d), a.ctypes.data, a.nbytes, 0.0, 0, t0,
                                               nsteps, P, 2 if pv else 0, ctypes.byref(rid))
        else:
            rc = capi.lib().gbca_server_submit(self.handle, ctypes.byref(d), None, 0, float(density), int(init_seed),
                                               t0, nsteps, P, 2 if pv else 0, ctypes.byref(rid))
        capi.check(rc)
        return int(rid.value)

    def poll(self, max_results: int = 4096):
        buf = (capi.Result * max_results)()
        n = ctypes.c_int32()
        capi.check(capi.lib().gbca_server_poll(self.handle, buf, max_results, ctypes.byref(n)))
        out = []
        for k in range(n.value):
            r = buf[k]
            out.append({"id": int(r.id), "status": int(r.status), "counts": [int(x) for x in r.counts],
                        "other": int(r.other), "morans": float(r.morans), "t_submit": r.t_submit,
                        "t_admit": r.t_admit, "t_done": r.t_done, "latency": r.t_done - r.t_submit})
        return out

    def status(self):
        q, a, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        capi.check(capi.lib().gbca_server_status(self.handle, ctypes.byref(q), ctypes.byref(a), ctypes.byref(c)))
        return int(q.value), int(a.value), float(c.value)

    def stats(self):
        """Occupancy so far: seconds each large-request lane and the small requests' stream had
        work in flight, the server's clock, and the number of large-request chunks run."""
        busy = (ctypes.c_double * 64)()
        n, small, wall, chunks = ctypes.c_int32(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        capi.check(capi.lib().gbca_server_stats(self.handle, busy, 64, ctypes.byref(n), ctypes.byref(small),
                                                ctypes.byref(wall), ctypes.byref(chunks)))
        return {"lane_busy_s": [float(busy[k]) for k in range(min(n.value, 64))], "small_busy_s": float(small.value),
                "wall_s": float(wall.value), "chunks": int(chunks.value)}

    def wait(self, ids, timeout: float = 600.0):
        """Poll until every id in `ids` has a result; returns {id: result}."""
        want, got = set(ids), {}
        t_end = time.monotonic() + timeout
        while want - set(got):
            for r in self.poll():
                got[r["id"]] = r
            if time.monotonic() > t_end:
                raise TimeoutError(f"{len(want - set(got))} requests unfinished after {timeout} s")
            time.sleep(0.0005)
        return got

    def stop(self):
        if self.handle:
            capi.lib().gbca_server_stop(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass
