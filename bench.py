"""Benchmark of the GB300 stencil-sweep backend (one JSON line on rank 0).

Workload (the single-instance sweeps at scale):
  (a) Larger than Life, Moore(5), birth 34..45 / survive 34..58, 8192 x 8192 Int8 torus,
      density 0.5 from seed 2, 1000 Synchronous steps;
  (b) forest fire, VonNeumann(1), Int8 codes {0 empty, 1 tree, 2 fire}, 16384 x 16384 Grid
      with Constant(0) edges, all empty at t = 0, p = 0.03, f = 1e-4, seed 3, 500 steps.
One bench step runs both from their initial states. Metric: Gcell-updates/s
(cells x steps / time) over the whole step.

  value : device-resident — initial states are copied device-to-device into the handles,
          then advanced; CUDA events on the stream the library launches on.
  e2e   : the same through the C ABI with host buffers — every step copies both initial
          states from pinned host memory (gbca_set_state_async), advances them, and copies both
          results back to pinned host memory (gbca_get_state_async); two handles per lattice
          and two sets of result buffers are used in turn, each handle on its own stream, so a
          step's copies overlap the neighbouring steps' sweeps; the clock stops when the last
          result is on the host, and the last results are checked against the device-resident
          run's.
  roofline: the dominant kernel (by device time), algorithmic bytes 2 B per cell-update
          (Int8 read + write) over its average launch duration, against the measured HBM copy
          bandwidth in MEASURED_PEAKS.json.
  cpu_baseline: the CPU oracle (C restatement of the reference's threaded ArrayBackend slab
          sweep) on a bounded sample of the same workload, on this host's cores.

--impl reference times that CPU implementation alone (the reference is Julia, which is not
installed; its C restatement runs in its place) on bounded samples of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LTL = dict(name="ltl", n1=8192, n2=8192, steps=1000, radius=5)
FIRE = dict(name="fire", n1=16384, n2=16384, steps=500, p=0.03, f=1e-4, seed=3)
BYTES_PER_CELL_UPDATE = 2  # one Int8 read + one Int8 write


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the served-stream measurement")
    ap.add_argument("--case", choices=["ltl", "fire", "lenia", "lenia-fft", "ensemble"], default=None,
                    help="time single passes of one kernel on an n x n lattice (for profiling)")
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--no-tune", action="store_true", help="keep the kernels' default sweep geometry")
    ap.add_argument("--spp", type=int, default=0, help="--case: pin this many steps per pass (no tuning)")
    ap.add_argument("--staging", type=int, default=0, help="--case with --spp: 1 stages fire tiles by TMA")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--no-saves", action="store_true", help="skip the save-path measurement")
    ap.add_argument("--no-sparse", action="store_true", help="skip the active-tile measurement")
    ap.add_argument("--no-lenia", action="store_true", help="skip the Lenia measurement")
    ap.add_argument("--sharded", action="store_true",
                    help="run each lattice as slabs over the ranks (halo exchange over NCCL; strong scaling) "
                         "instead of one replica of the workload per rank")
    ap.add_argument("--slabs", type=int, default=2, help="--sharded in one process: this many slabs on one GPU")
    ap.add_argument("--large", default=None, help="ensemble case: 'min_cells,steps_per_pass' of the batched "
                    "large-instance passes (0,1: none)")
    ap.add_argument("--side-range", default="", help="ensemble case: keep the instances with lo <= side < hi "
                    "('lo,hi')")
    ap.add_argument("--pin", default="", help="pin the sweeps' geometry instead of tuning, e.g. "
                    "'ltl=6,216,0;fire=1,0,1' (steps per pass, tile rows, staging), for profiling runs")
    return ap.parse_args()


def initial_states():
    rng = np.random.Generator(np.random.PCG64(2))
    ltl0 = np.asfortranarray((rng.random((LTL["n1"], LTL["n2"])) < 0.5).astype(np.int8))
    fire0 = np.zeros((FIRE["n1"], FIRE["n2"]), dtype=np.int8, order="F")
    return ltl0, fire0


def cell_updates():
    return LTL["n1"] * LTL["n2"] * LTL["steps"] + FIRE["n1"] * FIRE["n2"] * FIRE["steps"]


def descs(capi):
    from cellularautomatacore_jl_gb300.model import Life
    d1 = capi.Desc()
    life = Life(range(34, 46), range(34, 59))
    d1.rule, d1.nbhd, d1.radius, d1.states = capi.RULE_LIFE, capi.MOORE, 5, 2
    d1.birth, d1.survive = life.birth, life.survive
    d1.n1, d1.n2, d1.seed = LTL["n1"], LTL["n2"], 2
    d2 = capi.Desc()
    d2.rule, d2.nbhd, d2.radius = capi.RULE_FOREST_FIRE, capi.VON_NEUMANN, 1
    d2.n1, d2.n2, d2.seed = FIRE["n1"], FIRE["n2"], FIRE["seed"]
    d2.boundary[0] = d2.boundary[1] = capi.CONSTANT
    return d1, d2


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc = index, None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(summary: str):
    """Per-launch DRAM bytes from a committed ncu summary under profiles/, when it has them
    (a line 'traffic_bytes_per_launch: N')."""
    path = os.path.join(ROOT, "profiles", summary)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    return None


def cpu_sample(nthreads: int):
    """The oracle (C restatement of ArrayBackend's threaded slab sweep) on a bounded sample of
    the workload itself: the first 3 steps of the LtL run on the 8192^2 torus and the first 2 of
    the forest-fire run on the 16384^2 grid, from their own initial states, extrapolated to the
    full runs by their step counts (every step of either rule costs the CPU the same: each LtL
    cell counts 120 neighbours, each non-burning fire cell makes one draw)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as o
    o.build()
    ltl0, fire0 = initial_states()
    P1 = o.Problem(o.RULE_LIFE, LTL["n1"], LTL["n2"], radius=5, birth=o.mask(range(34, 46)),
                   survive=o.mask(range(34, 59)))
    P2 = o.Problem(o.RULE_FOREST_FIRE, FIRE["n1"], FIRE["n2"], nbhd=o.VON_NEUMANN, seed=FIRE["seed"],
                   boundary=(o.CONSTANT, o.CONSTANT))
    t0 = time.perf_counter()
    o.run_array(P1, ltl0, 0, 3, None, nthreads)
    t1 = time.perf_counter()
    o.run_array(P2, fire0, 0, 2, (FIRE["p"], FIRE["f"]), nthreads)
    t2 = time.perf_counter()
    cu = 3 * LTL["n1"] * LTL["n2"] + 2 * FIRE["n1"] * FIRE["n2"]
    # weight the two parts as the full workload does (1000:500 steps on 8192^2:16384^2)
    r1 = 3 * LTL["n1"] * LTL["n2"] / (t1 - t0)
    r2 = 2 * FIRE["n1"] * FIRE["n2"] / (t2 - t1)
    w1 = LTL["n1"] * LTL["n2"] * LTL["steps"]
    w2 = FIRE["n1"] * FIRE["n2"] * FIRE["steps"]
    rate = (w1 + w2) / (w1 / r1 + w2 / r2)
    return {"value": rate / 1e9, "unit": "Gcell-updates/s", "cores": nthreads, "kind": "port",
            "sample": "C restatement of ArrayBackend (threaded slabs): the first 3 steps of the 8192^2 LtL run and "
                      "the first 2 of the 16384^2 forest-fire run (all empty at t = 0), each from the workload's own "
                      "initial state, combined with the workload's 1000:500 step weights",
            "parts_gcells": {"ltl": r1 / 1e9, "fire": r2 / 1e9}, "seconds": t2 - t0, "cell_updates": cu}


WORKLOAD = ("single-instance sweeps: Larger-than-Life Moore(5) B34..45/S34..58 on an 8192^2 Int8 torus x 1000 "
            "steps + forest fire VonNeumann(1) on a 16384^2 Grid Constant(0) x 500 steps (p=0.03, f=1e-4)")


def run_reference(args, rank, world):
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(nthreads)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_sample(nthreads)["value"])
    wall = time.perf_counter() - t0
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": "Gcell-updates/s", "value": v, "unit": "Gcell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int8", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cell_updates_per_step": cell_updates(), "parallelism": "replicas x1",
                       "sample": "each step times the workload's first steps on the host cores (3 LtL steps on "
                                 "8192^2 and 2 forest-fire steps on 16384^2 from their initial states, weighted "
                                 "1000:500)"},
            "cpu_baseline": {"value": v, "unit": "Gcell-updates/s", "cores": nthreads, "kind": "port",
                             "sample": "per step: the first 3 LtL steps on 8192^2 + the first 2 forest-fire steps "
                                       "on 16384^2"},
            "e2e": {"value": v, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ensemble_case(capi, lib, args):
    """`steps` timed runs of a batched forest-fire ensemble of `n` instances (the batched
    workload's size distribution and parameters, 100 steps each), after `warmup` runs."""
    sides, ps, fs, seeds = ensemble_instances()
    if args.side_range:
        lo, hi = (int(x) for x in args.side_range.split(","))
        keep = (sides >= lo) & (sides < hi)
        sides, ps, fs, seeds = sides[keep], ps[keep], fs[keep], seeds[keep]
    n = min(args.n, len(sides))
    descs = (capi.Desc * n)()
    for i in range(n):
        descs[i] = fire_desc(capi, sides[i], seeds[i])
    e = ctypes.c_void_p()
    capi.check(lib.gbca_ensemble_create(descs, n, ctypes.byref(e)))
    if args.spp:
        capi.check(lib.gbca_ensemble_set_geometry(e, 128, args.spp))
    if args.large is not None:
        cells, k = (int(x) for x in args.large.split(","))
        capi.check(lib.gbca_ensemble_set_large(e, cells, k))
    T0 = (ctypes.c_int64 * n)()
    S = (ctypes.c_int64 * n)(*([100] * n))
    P = (ctypes.c_double * (2 * n))(*np.column_stack([ps[:n], fs[:n]]).ravel().tolist())

    def run():
        capi.check(lib.gbca_ensemble_fill(e, 0))
        capi.check(lib.gbca_ensemble_run(e, T0, S, P, 2))
        capi.check(lib.gbca_ensemble_sync(e))

    for _ in range(args.warmup):
        run()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run()
    dt = (time.perf_counter() - t0) / args.steps
    cu = float((sides[:n].astype(np.float64) ** 2).sum() * 100)
    geo = [ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()]
    capi.check(lib.gbca_ensemble_geometry(e, *[ctypes.byref(x) for x in geo]))
    print(json.dumps({"case": "ensemble", "instances": n, "s_per_run": dt, "sims_per_s": n / dt,
                      "gcell_updates_s": cu / dt / 1e9, "large_cells": geo[2].value, "large_steps": geo[3].value,
                      "large_instances": geo[4].value}))
    lib.gbca_ensemble_destroy(e)


def run_case(args):
    """`steps` timed passes (one kernel launch each for the sweeps, one step for Lenia) of
    one workload on an n x n lattice after `warmup` untimed ones."""
    import torch
    import __graft_entry__ as ge
    ge.build()
    ca = ge.load_package()
    capi, lib = ca.capi, ca.capi.lib()
    if args.case == "ensemble":
        return run_ensemble_case(capi, lib, args)
    n = args.n
    d1, d2 = descs(capi)
    rng = np.random.Generator(np.random.PCG64(2))
    if args.case == "ltl":
        d, per, params, dtype = d1, 4, None, np.int8
        u0 = (rng.random((n, n)) < 0.5).astype(np.int8)
    elif args.case == "fire":
        d, per, dtype = d2, 8, np.int8
        params = (ctypes.c_double * 2)(FIRE["p"], FIRE["f"])
        pct = rng.integers(0, 100, size=(n, n), dtype=np.int8)
        u0 = (pct >= 40).astype(np.int8) + (pct >= 99).astype(np.int8)
    else:
        d = capi.Desc()
        d.rule, d.lenia_R, d.lenia_npeaks, d.lenia_peaks[0] = capi.RULE_LENIA, 13, 1, 1.0
        d.lenia_mu, d.lenia_sigma, d.lenia_dt = 0.15, 0.015, 0.1
        d.lenia_method = capi.FFT if args.case == "lenia-fft" else capi.DIRECT
        per, params, dtype = 1, None, np.float32
        u0 = np.zeros((n, n), np.float32)
        c = n // 2
        u0[c - 128:c + 128, c - 128:c + 128] = rng.random((256, 256))
    d.n1 = d.n2 = n
    h = ctypes.c_void_p()
    capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(h)))
    a = np.asfortranarray(u0.astype(dtype))
    capi.check(lib.gbca_set_state(h, a.ctypes.data, a.nbytes))
    stream = torch.cuda.Stream()
    capi.check(lib.gbca_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
    nparams = 2 if params is not None else 0
    geometry = None
    if args.case in ("ltl", "fire") and args.spp > 0:
        capi.check(lib.gbca_set_geometry(h, args.spp, 0, args.staging))
        per = args.spp
    elif args.case in ("ltl", "fire") and not args.no_tune:
        geometry = tune(capi, lib, h, params, nparams)
        per = geometry[0] or per
    t = 0
    for _ in range(args.warmup):
        capi.check(lib.gbca_advance(h, t, per, params, nparams))
        t += per
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        capi.check(lib.gbca_advance(h, t, per, params, nparams))
        t += per
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    cu = n * n * per
    out = {"case": args.case, "n": n, "steps_per_pass": per, "geometry": geometry, "ms_per_pass": ms,
           "gcell_updates_s": cu / (ms * 1e-3) / 1e9}
    if args.case in ("ltl", "fire"):
        out["hbm_frac_per_effective_step"] = BYTES_PER_CELL_UPDATE * cu / (ms * 1e-3) / 1e9 / measured_peaks()[0]
    else:
        out["gflops_direct_equiv"] = n * n * 516 * 2 / (ms * 1e-3) / 1e9
    print(json.dumps(out))
    lib.gbca_destroy(h)


ENS = dict(n=4096, steps=500, plain_sample=256)


def tune(capi, lib, h, params, nparams):
    """The autotuner's (steps per pass, tile rows, staging) for the handle's shape, timed on its state."""
    k, rows, staging = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    capi.check(lib.gbca_tune(h, params, nparams, ctypes.byref(k), ctypes.byref(rows), ctypes.byref(staging)))
    return int(k.value), int(rows.value), int(staging.value)


SAVES = [dict(name="highlife-128", rule="highlife", n=128, steps=200, saveat=20),
         dict(name="conway-4096", rule="conway", n=4096, steps=200, saveat=20)]


def bench_saves(ca, reps: int = 5):
    """A solve with saveat through the public API (saves staged on the device and copied out
    on a second stream) against the same run saving as the reference's integrator does: the
    queued steps flushed and the state copied synchronously at every save."""
    capi, lib = ca.capi, ca.capi.lib()
    out = {}
    for cfg in SAVES:
        n, steps, every = cfg["n"], cfg["steps"], cfg["saveat"]
        u0 = (np.random.Generator(np.random.PCG64(1)).random((n, n)) < 0.5).astype(np.int8)
        prob = ca.CAProblem.new(ca.Life(":" + cfg["rule"]), u0, steps)
        B = ca.GB300Backend()

        def run_api():
            return ca.solve(prob, ca.Synchronous(), backend=B, saveat=every)

        def run_sync():
            st = ca.allocate_state(B, prob, ca.Synchronous())
            saves = [ca.current_state(B, st)]
            for t in range(0, steps, every):
                capi.check(lib.gbca_advance(st.handle, t, every, None, 0))
                saves.append(ca.current_state(B, st))
            st.close()
            return saves

        a, b = run_api(), run_sync()
        assert all(np.array_equal(x, y) for x, y in zip(a.u, b)) and len(a.u) == len(b)
        ta, tb = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            run_api()
            ta.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            run_sync()
            tb.append(time.perf_counter() - t0)
        out[cfg["name"]] = {"saves": len(b), "solve_ms": statistics.median(ta) * 1e3,
                            "sync_saves_ms": statistics.median(tb) * 1e3,
                            "speedup": statistics.median(tb) / statistics.median(ta)}
    return out


SPARSE = dict(n=16384, patch=1024, steps=500)


def bench_sparse(ca):
    """Active-tile sweeps against dense ones: Conway's Life on a 16384^2 torus, quiescent but
    for a 1024^2 Bernoulli(0.5) soup in the centre (PCG64(5)), 500 steps; device time of the
    advance, and the final states compared."""
    import torch
    capi, lib = ca.capi, ca.capi.lib()
    n, m, steps = SPARSE["n"], SPARSE["patch"], SPARSE["steps"]
    u0 = np.zeros((n, n), np.int8)
    c = (n - m) // 2
    u0[c:c + m, c:c + m] = (np.random.Generator(np.random.PCG64(5)).random((m, m)) < 0.5)
    prob = ca.CAProblem.new(ca.Life(":conway"), u0, steps)
    out, finals = {}, {}
    for name, backend in (("dense", ca.GB300Backend()), ("active_tiles", ca.GB300Backend(background=0))):
        st = ca.allocate_state(backend, prob, ca.Synchronous())
        stream = torch.cuda.Stream()
        capi.check(lib.gbca_set_stream(st.handle, ctypes.c_void_p(stream.cuda_stream)))
        capi.check(lib.gbca_advance(st.handle, 0, 2, None, 0))  # warm-up
        ca.set_state(backend, st, u0)  # timed from the initial state (tile flags rebuilt inside)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        capi.check(lib.gbca_advance(st.handle, 0, steps, None, 0))
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        finals[name] = ca.current_state(backend, st)
        out[name] = {"ms": ms, "gcell_updates_s": n * n * steps / (ms * 1e-3) / 1e9}
        st.close()
    out["equal"] = bool(np.array_equal(finals["dense"], finals["active_tiles"]))
    out["speedup"] = out["dense"]["ms"] / out["active_tiles"]["ms"]
    out["config"] = f"Life B3/S23 on a {n}^2 torus, {m}^2 soup in the centre, {steps} steps"
    return out


FIRE_FMAHEAVY_CYCLES_PER_WARP = 79.15  # k_fire: fmaheavy pipe cycles per 32 cell-updates (ncu)


def bench_lenia(capi, lib, reps: int = 3):
    """Lenia in Float32 on a 2048^2 torus (R = 13, one bump, mu = 0.15, sigma = 0.015, dt = 0.1,
    Uniform[0,1] in the central 256^2 patch from seed 4), 100 steps, by the direct field and by
    the FFT field: time per step with CUDA events on the handle's stream, the best of `reps`
    runs from the initial state."""
    import torch
    n, steps = 2048, 100
    rng = np.random.default_rng(4)
    u0 = np.zeros((n, n), np.float32)
    c = n // 2
    u0[c - 128:c + 128, c - 128:c + 128] = rng.random((256, 256)).astype(np.float32)
    a = np.asfortranarray(u0)
    stream = torch.cuda.Stream()
    out = {"workload": "Lenia Float32, 2048^2 torus, R = 13, 100 steps from a 256^2 soup", "paths": {}}
    for name, method in (("direct", capi.DIRECT), ("fft", capi.FFT)):
        d = capi.Desc()
        d.rule, d.lenia_R, d.lenia_npeaks, d.lenia_peaks[0] = capi.RULE_LENIA, 13, 1, 1.0
        d.lenia_mu, d.lenia_sigma, d.lenia_dt, d.lenia_method = 0.15, 0.015, 0.1, method
        d.n1 = d.n2 = n
        h = ctypes.c_void_p()
        capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(h)))
        capi.check(lib.gbca_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
        best = None
        for r in range(reps + 1):  # the first run warms up
            capi.check(lib.gbca_set_state(h, a.ctypes.data, a.nbytes))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            capi.check(lib.gbca_advance(h, 0, steps, None, 0))
            e1.record(stream)
            torch.cuda.synchronize()
            if r > 0:
                ms = e0.elapsed_time(e1) / steps
                best = ms if best is None else min(best, ms)
        lib.gbca_destroy(h)
        tflops = n * n * 516 * 2 / (best * 1e-3) / 1e12
        out["paths"][name] = {"ms_per_step": best, "gcell_updates_s": n * n / (best * 1e-3) / 1e9,
                              "direct_equivalent_tflops": tflops}
    out["fp32_fma_peak_tflops"] = 152 * 128 * 2 * 2.07e9 / 1e12
    out["paths"]["direct"]["frac_of_fp32_fma_peak"] = out["paths"]["direct"]["direct_equivalent_tflops"] / \
        out["fp32_fma_peak_tflops"]
    return out


def ensemble_instances():
    """4096 forest-fire instances: square sides log-uniform in 64..1024, p ~ U(0.01, 0.1),
    f ~ LogU(1e-5, 1e-3), seeds 1..4096 (numpy PCG64(4096))."""
    rng = np.random.Generator(np.random.PCG64(4096))
    n = ENS["n"]
    sides = np.round(np.exp(rng.uniform(np.log(64), np.log(1024), n))).astype(np.int64)
    ps = rng.uniform(0.01, 0.1, n)
    fs = np.exp(rng.uniform(np.log(1e-5), np.log(1e-3), n))
    return sides, ps, fs, np.arange(1, n + 1)


def fire_desc(capi, side, seed):
    d = capi.Desc()
    d.rule, d.nbhd, d.radius = capi.RULE_FOREST_FIRE, capi.VON_NEUMANN, 1
    d.n1 = d.n2 = int(side)
    d.boundary[0] = d.boundary[1] = capi.CONSTANT
    d.seed = int(seed)
    return d


def bench_batched(capi, lib, warmup: int, steps: int):
    """The batched ensemble (one persistent graph-captured launch per run) against one solve
    per instance through the same library, on a random sample; summaries compared exactly."""
    sides, ps, fs, seeds = ensemble_instances()
    n = len(sides)
    descs = (capi.Desc * n)()
    for i in range(n):
        descs[i] = fire_desc(capi, sides[i], seeds[i])
    e = ctypes.c_void_p()
    capi.check(lib.gbca_ensemble_create(descs, n, ctypes.byref(e)))
    T0 = (ctypes.c_int64 * n)()
    S = (ctypes.c_int64 * n)(*([ENS["steps"]] * n))
    P = (ctypes.c_double * (2 * n))(*np.column_stack([ps, fs]).ravel().tolist())

    def run():
        capi.check(lib.gbca_ensemble_fill(e, 0))
        capi.check(lib.gbca_ensemble_run(e, T0, S, P, 2))
        capi.check(lib.gbca_ensemble_sync(e))

    # the autotuner picks the batched kernel's tile side and pass depth (16-step probes)
    capi.check(lib.gbca_ensemble_fill(e, 0))
    tile, depth = ctypes.c_int32(), ctypes.c_int32()
    capi.check(lib.gbca_ensemble_tune(e, 16, P, 2, ctypes.byref(tile), ctypes.byref(depth)))
    for _ in range(warmup):
        run()
    geo = [ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()]
    capi.check(lib.gbca_ensemble_geometry(e, *[ctypes.byref(x) for x in geo]))
    l0 = lib.gbca_kernel_launches()
    t0 = time.perf_counter()
    for _ in range(steps):
        run()
    t_batched = (time.perf_counter() - t0) / steps
    launches = (lib.gbca_kernel_launches() - l0) / steps
    C = (ctypes.c_int64 * (3 * n))()
    O = (ctypes.c_int64 * n)()
    M = (ctypes.c_double * n)()
    capi.check(lib.gbca_ensemble_summaries(e, C, 3, O, M))
    lib.gbca_ensemble_destroy(e)

    # one solve per instance: create, upload, advance, summaries, destroy — a random sample
    rng = np.random.Generator(np.random.PCG64(1))
    sample = rng.choice(n, ENS["plain_sample"], replace=False)
    exact = 0
    t0 = time.perf_counter()
    for i in sample:
        h = ctypes.c_void_p()
        d = fire_desc(capi, sides[i], seeds[i])
        capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(h)))
        zeros = np.zeros(int(sides[i]) ** 2, np.int8)
        capi.check(lib.gbca_set_state(h, zeros.ctypes.data, zeros.nbytes))
        pr = (ctypes.c_double * 2)(ps[i], fs[i])
        capi.check(lib.gbca_advance(h, 0, ENS["steps"], pr, 2))
        c3 = (ctypes.c_int64 * 3)()
        o1 = ctypes.c_int64()
        m1 = ctypes.c_double()
        capi.check(lib.gbca_summaries(h, c3, 3, ctypes.byref(o1), ctypes.byref(m1)))
        lib.gbca_destroy(h)
        same = list(c3) == [C[3 * i + k] for k in range(3)] and (m1.value == M[i] or (np.isnan(m1.value) and
                                                                                          np.isnan(M[i])))
        exact += bool(same)
    t_plain = time.perf_counter() - t0
    cu = float((sides.astype(np.float64) ** 2).sum()) * ENS["steps"]
    sample_cu = float((sides[sample].astype(np.float64) ** 2).sum()) * ENS["steps"]
    plain_sims = len(sample) / t_plain
    return {"workload": "4096 forest-fire instances, square Grid sides log-uniform 64..1024, p ~ U(0.01, 0.1), "
                        "f ~ LogU(1e-5, 1e-3), seeds 1..4096, all empty at t = 0, 500 steps each",
            "sims_per_s": n / t_batched, "s_per_run": t_batched, "gcell_updates_s": cu / t_batched / 1e9,
            "plain_sims_per_s": plain_sims, "plain_sample": len(sample),
            "plain_gcell_updates_s": sample_cu / t_plain / 1e9,
            "speedup_vs_plain": (n / t_batched) / plain_sims,
            "exact_matches_in_sample": exact, "graph_launches_per_run": 1, "kernels_per_run": launches,
            "geometry": {"tile": tile.value, "depth": depth.value, "large_cells": geo[2].value,
                         "large_steps_per_pass": geo[3].value, "large_instances": geo[4].value,
                         "picked_by": "gbca_ensemble_tune"}}


SERVE = dict(rate=2000.0, seconds=2.0, plain_sample=48, hbm_budget=8 << 30, chunk_steps=100,
             big_cells=1 << 14, max_big=16)


def serve_requests(n: int, seed: int = 2000):
    """n requests of the served stream: Poisson arrivals at SERVE['rate'] per second; rule
    uniform over {Life B3/S23, Generations B2/S/C3, forest fire with p ~ U(0.01, 0.1),
    f ~ LogU(1e-5, 1e-3)}; square side log-uniform in 64..4096; steps uniform in 50..1000;
    independent seeds. Life and Generations start from a density-0.5 soup, the fire empty."""
    rng = np.random.Generator(np.random.PCG64(seed))
    arrivals = np.cumsum(rng.exponential(1.0 / SERVE["rate"], n))
    kinds = rng.integers(0, 3, n)
    sides = np.round(np.exp(rng.uniform(np.log(64), np.log(4096), n))).astype(np.int64)
    steps = rng.integers(50, 1001, n)
    ps = rng.uniform(0.01, 0.1, n)
    fs = np.exp(rng.uniform(np.log(1e-5), np.log(1e-3), n))
    seeds = rng.integers(1, 2 ** 62, n)
    return arrivals, kinds, sides, steps, ps, fs, seeds


def serve_desc(capi, kind, side, seed):
    from cellularautomatacore_jl_gb300.model import Generations, Life
    if kind == 2:
        return fire_desc(capi, side, seed)
    d = capi.Desc()
    r = Life("B3/S23") if kind == 0 else Generations("B2/S/C3")
    d.rule = capi.RULE_LIFE if kind == 0 else capi.RULE_GENERATIONS
    d.nbhd, d.radius, d.states = capi.MOORE, 1, 2 if kind == 0 else 3
    d.birth, d.survive = r.birth, r.survive
    d.n1 = d.n2 = int(side)
    d.seed = int(seed)
    return d


def run_stream(capi, lib, n, rate, seed):
    """Submit n requests of the served stream at Poisson rate `rate` into a fresh server and
    collect every result; returns (results {id: (status, t_submit, t_done, counts, other, morans)},
    requests, wall)."""
    arrivals, kinds, sides, steps, ps, fs, seeds = serve_requests(n, seed)
    arrivals = arrivals * (SERVE["rate"] / rate)
    cfg = capi.ServerConfig()
    cfg.hbm_budget, cfg.chunk_steps = SERVE["hbm_budget"], SERVE["chunk_steps"]
    cfg.big_cells, cfg.max_big = SERVE["big_cells"], SERVE["max_big"]
    srv = ctypes.c_void_p()
    capi.check(lib.gbca_server_start(ctypes.byref(cfg), ctypes.byref(srv)))
    descs = [serve_desc(capi, kinds[i], sides[i], seeds[i]) for i in range(n)]
    res_buf = (capi.Result * 4096)()
    got = {}
    rid = ctypes.c_uint64()
    nres = ctypes.c_int32()

    def drain():
        capi.check(lib.gbca_server_poll(srv, res_buf, 4096, ctypes.byref(nres)))
        for k in range(nres.value):
            r = res_buf[k]
            got[int(r.id)] = (r.status, r.t_submit, r.t_done, tuple(r.counts[k] for k in range(8)), r.other,
                              r.morans)

    t0 = time.perf_counter()
    for i in range(n):
        while time.perf_counter() - t0 < arrivals[i]:
            drain()
        P = (ctypes.c_double * 2)(ps[i], fs[i])
        dens = 0.0 if kinds[i] == 2 else 0.5
        capi.check(lib.gbca_server_submit(srv, ctypes.byref(descs[i]), None, 0, dens, int(seeds[i]), 0, int(steps[i]),
                                          P, 2 if kinds[i] == 2 else 0, ctypes.byref(rid)))
    while len(got) < n:
        drain()
        time.sleep(0.001)
    wall = time.perf_counter() - t0
    busy = (ctypes.c_double * 64)()
    nl, small, clock, chunks = ctypes.c_int32(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
    capi.check(lib.gbca_server_stats(srv, busy, 64, ctypes.byref(nl), ctypes.byref(small), ctypes.byref(clock),
                                     ctypes.byref(chunks)))
    lib.gbca_server_stop(srv)
    lanes = [busy[k] / clock.value for k in range(min(nl.value, 64))]
    occupancy = {"lanes": nl.value, "lane_busy_frac": [round(x, 3) for x in lanes],
                 "mean_lanes_busy": sum(lanes), "small_stream_busy_frac": small.value / clock.value,
                 "large_chunks": chunks.value}
    return got, (arrivals, kinds, sides, steps, ps, fs, seeds, descs), wall, occupancy


def bench_served(capi, lib):
    """Poisson arrivals at 2000 requests/s for SERVE['seconds'] s into the continuous-batching
    server (far above what one GPU completes, so latency is mostly queueing), then a stream at
    half the measured capacity (latency of the loop itself); latency = result time - submit
    time. Then the plain path: the same kind of requests one at a time through a handle each
    (create, the same device soup, advance, summaries, destroy), on a sample, whose summaries
    must equal the served ones exactly."""
    n = int(SERVE["rate"] * SERVE["seconds"])
    got, reqs, wall, occ = run_stream(capi, lib, n, SERVE["rate"], 2000)
    ids = sorted(got)  # ids are given in submission order
    arrivals, kinds, sides, steps, ps, fs, seeds, descs = reqs
    lat = np.array([v[2] - v[1] for v in got.values()])
    t_first = min(v[1] for v in got.values())
    t_last = max(v[2] for v in got.values())
    cu = float((sides.astype(np.float64) ** 2 * steps).sum())
    served = {"workload": f"{n} requests, Poisson arrivals at {SERVE['rate']:.0f}/s for {SERVE['seconds']} s; rule "
                          "uniform over Life B3/S23, Generations B2/S/C3, forest fire; side log-uniform 64..4096; steps "
                          "50..1000", "requests": n, "ok": int(sum(1 for v in got.values() if v[0] == 0)),
              "sims_per_s": n / (t_last - t_first), "gcell_updates_s": cu / (t_last - t_first) / 1e9,
              "offered_gcell_updates_s": cu / arrivals[-1] / 1e9,
              "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
              "wall_s": wall, "config": {k: SERVE[k] for k in ("hbm_budget", "chunk_steps", "big_cells", "max_big")},
              "occupancy": occ}

    # the plain per-request path on a random sample, one request at a time
    rng = np.random.Generator(np.random.PCG64(5))
    sample = rng.choice(n, SERVE["plain_sample"], replace=False)
    lat_plain, t_sum, exact = [], 0.0, 0
    for i in sample:
        d = descs[i]
        P = (ctypes.c_double * 2)(ps[i], fs[i])
        ts = time.perf_counter()
        h = ctypes.c_void_p()
        capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(h)))
        if kinds[i] != 2:  # the server's initial state: the same device soup from the same seed
            capi.check(lib.gbca_set_state_soup(h, 0.5, int(seeds[i])))
        capi.check(lib.gbca_advance(h, 0, int(steps[i]), P, 2 if kinds[i] == 2 else 0))
        c8 = (ctypes.c_int64 * 8)()
        o1 = ctypes.c_int64()
        m1 = ctypes.c_double()
        capi.check(lib.gbca_summaries(h, c8, 8, ctypes.byref(o1), ctypes.byref(m1)))
        lib.gbca_destroy(h)
        dt = time.perf_counter() - ts
        t_sum += dt
        lat_plain.append(dt)
        srv = got[ids[i]]
        same_m = srv[5] == m1.value or (np.isnan(srv[5]) and np.isnan(m1.value))
        exact += int(srv[0] == 0 and tuple(c8) == srv[3] and srv[4] == o1.value and same_m)
    # a stream at half the measured capacity, for the loop's latency when it keeps up
    rate2 = 0.5 * served["sims_per_s"]
    n2 = max(50, int(rate2 * 3.0))
    got2, reqs2, _, occ2 = run_stream(capi, lib, n2, rate2, 2001)
    lat2 = np.array([v[2] - v[1] for v in got2.values()])
    t2a, t2b = min(v[1] for v in got2.values()), max(v[2] for v in got2.values())
    served["at_half_capacity"] = {"rate_per_s": rate2, "requests": n2,
                                  "ok": int(sum(1 for v in got2.values() if v[0] == 0)),
                                  "sims_per_s": n2 / (t2b - t2a), "latency_p50_s": float(np.percentile(lat2, 50)),
                                  "latency_p99_s": float(np.percentile(lat2, 99)), "occupancy": occ2}
    served["plain_sims_per_s"] = len(sample) / t_sum
    served["plain_sample"] = len(sample)
    served["plain_service_p50_s"] = float(np.percentile(lat_plain, 50))
    served["exact_matches_in_sample"] = exact
    served["speedup_vs_plain"] = served["sims_per_s"] / served["plain_sims_per_s"]
    return served


def max_over_ranks(x: float, dist, device: str) -> float:
    """The largest of every rank's x (a time): the whole job is as slow as its slowest replica."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world: int, cell_updates_per_rank: float, ms_per_step: float) -> float:
    """Whole-job Gcell-updates/s of `world` replicas that each run the workload per step."""
    return world * cell_updates_per_rank / (ms_per_step * 1e-3) / 1e9


SHARD_STEPS = {"ltl": 6, "fire": 1}  # steps between halo exchanges


def run_sharded(args, rank, world, local):
    """The workload with each lattice split into column slabs: one per rank over NCCL, or
    --slabs of them on one GPU in one process. Every step restores each slab's initial columns
    from a device copy, then runs the lattice's steps with a halo exchange every
    SHARD_STEPS[lattice] steps. Total work is fixed (strong scaling)."""
    import torch
    import __graft_entry__ as ge
    ge.build()
    ca = ge.load_package()
    sl = ca.slabs
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ltl0, fire0 = initial_states()
    probs = [("ltl", ca.CAProblem.new(ca.Life(range(34, 46), range(34, 59), neighbourhood=ca.Moore(5)), ltl0,
                                      LTL["steps"], space=ca.Torus(LTL["n1"], LTL["n2"]), seed=2), None),
             ("fire", ca.CAProblem.new(ca.ForestFire(), fire0, FIRE["steps"], {"p": FIRE["p"], "f": FIRE["f"]},
                                       space=ca.Grid(FIRE["n1"], FIRE["n2"]), seed=FIRE["seed"]),
              (FIRE["p"], FIRE["f"]))]
    stream = torch.cuda.Stream()
    sch = ca.Synchronous()
    nslabs = world if world > 1 else max(1, args.slabs)
    runs, halos = [], {}
    for name, prob, params in probs:
        K = SHARD_STEPS[name]
        halos[name] = sl.halo_columns(prob.neighbours.radius, K)
        if world > 1:
            periodic = isinstance(prob.space.boundaries[1], ca.Periodic)
            slab = sl.plan(prob.space.dims[1], world, halos[name], periodic)[rank]
            shard = sl.DeviceSlab(prob, sch, slab, stream=stream)
            runner, shards = sl.SlabSweep(prob, sch, slab, shard, sl.ProcessGroupTransport(), K), [shard]
        else:
            runner = sl.LocalGroup(prob, sch, nslabs, K,
                                   make_shard=lambda s, prob=prob: sl.DeviceSlab(prob, sch, s, stream=stream))
            shards = runner.shards
        pristine = [torch.as_tensor(np.ascontiguousarray(np.asarray(prob.u0)[:, sh.cols].T), device="cuda")
                    for sh in shards]
        runs.append((prob, params, runner, shards, pristine))
    torch.cuda.synchronize()

    def step():
        with torch.cuda.stream(stream):
            for prob, params, runner, shards, pristine in runs:
                for sh, cols in zip(shards, pristine):
                    sh.set_state_device(cols)
                runner.run(0, prob.tspan[1], params)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), dist, "cuda") / args.steps
    if rank == 0:
        print(json.dumps({
            "metric": "Gcell-updates/s", "value": cell_updates() / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "int8", "data": "synthetic", "mode": "sharded",
            "config": {"workload": WORKLOAD, "parallelism": f"slabs x{nslabs}" + ("" if world > 1 else " on one GPU"),
                       "steps_per_exchange": SHARD_STEPS, "halo_columns": halos},
            "clocks": clocks.summary()}))
    for prob, params, runner, shards, pristine in runs:
        for sh in shards:
            sh.close()
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.case:
        return run_case(args)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.sharded:
        return run_sharded(args, rank, world, local)

    import torch
    import __graft_entry__ as ge
    ge.build()
    ca = ge.load_package()
    capi = ca.capi
    lib = capi.lib()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    ltl0, fire0 = initial_states()
    d1, d2 = descs(capi)
    handles = []
    for d in (d1, d2):
        h = ctypes.c_void_p()
        capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(h)))
        handles.append(h)
    stream = torch.cuda.Stream()
    for h in handles:
        capi.check(lib.gbca_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
    # pristine device copies of the initial states (column-major bytes)
    dev0 = [torch.from_numpy(np.ascontiguousarray(a.T)).cuda() for a in (ltl0, fire0)]
    params_fire = (ctypes.c_double * 2)(FIRE["p"], FIRE["f"])
    sizes = [(LTL["n1"], LTL["n2"]), (FIRE["n1"], FIRE["n2"])]

    def step_resident(events=None):
        for k, (h, d0, (n1, n2)) in enumerate(zip(handles, dev0, sizes)):
            capi.check(lib.gbca_set_state_device(h, ctypes.c_void_p(d0.data_ptr()), n1))
            if events is not None:
                events[2 * k].record(stream)
            if k == 0:
                capi.check(lib.gbca_advance(h, 0, LTL["steps"], None, 0))
            else:
                capi.check(lib.gbca_advance(h, 0, FIRE["steps"], params_fire, 2))
            if events is not None:
                events[2 * k + 1].record(stream)

    # the autotuner picks each sweep's geometry on the initial states (untimed, like warm-up)
    geometry = {}
    pins = dict(kv.split("=") for kv in args.pin.split(";") if kv) if args.pin else {}
    for name, h, d0, (n1, n2) in zip(("ltl", "fire"), handles, dev0, sizes):
        capi.check(lib.gbca_set_state_device(h, ctypes.c_void_p(d0.data_ptr()), n1))
        if name in pins:
            k, rows, staging = (int(x) for x in pins[name].split(","))
            capi.check(lib.gbca_set_geometry(h, k, rows, staging))
            geometry[name] = (k, rows, staging)
        elif not args.no_tune:
            geometry[name] = tune(capi, lib, h, params_fire if name == "fire" else None, 2 if name == "fire" else 0)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step_resident()
    torch.cuda.synchronize()

    # ---- device-resident timed region
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = lib.gbca_kernel_launches()
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        start.record(stream)
        for k in range(args.steps):
            step_resident(ev[k])
        stop.record(stream)
        torch.cuda.synchronize()
    barrier()
    launches = lib.gbca_kernel_launches() - launches0
    # the device-resident run's results, for the end-to-end run to match
    resident_out = [np.empty((n2, n1), np.int8) for n1, n2 in sizes]
    for h, r in zip(handles, resident_out):
        capi.check(lib.gbca_get_state(h, r.ctypes.data, r.nbytes))
    ms_total = start.elapsed_time(stop)
    part_ms = [sum(e[0].elapsed_time(e[1]) for e in ev), sum(e[2].elapsed_time(e[3]) for e in ev)]
    ms_total = max_over_ranks(ms_total, dist, "cuda")
    ms_per_step = ms_total / args.steps
    value = replica_value(world, cell_updates(), ms_per_step)

    # ---- roofline of the dominant kernel
    per_pass = {}
    for name, h in zip(("ltl", "fire"), handles):  # the geometry the sweeps ran with
        k, rows, staging = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        capi.check(lib.gbca_geometry(h, params_fire if name == "fire" else None, ctypes.byref(k), ctypes.byref(rows),
                                     ctypes.byref(staging)))
        per_pass[name] = max(1, k.value)
        geometry.setdefault(name, (k.value, rows.value, staging.value))
    parts = {}
    for name, cfg, ms in (("ltl", LTL, part_ms[0]), ("fire", FIRE, part_ms[1])):
        launches_part = -(-cfg["steps"] // per_pass[name])
        cu = cfg["n1"] * cfg["n2"] * cfg["steps"]
        avg_launch_s = ms / args.steps / launches_part * 1e-3
        alg_bytes_launch = BYTES_PER_CELL_UPDATE * cfg["n1"] * cfg["n2"] * (cfg["steps"] / launches_part)
        parts[name] = {"ms": ms / args.steps, "gcell_updates_s": cu / (ms / args.steps * 1e-3) / 1e9,
                       "launches": launches_part, "avg_launch_us": avg_launch_s * 1e6,
                       "alg_bytes_per_launch": alg_bytes_launch, "achieved_gbs": alg_bytes_launch / avg_launch_s / 1e9}
    dom = max(parts, key=lambda k: parts[k]["ms"])
    kernel = {"ltl": "k_life", "fire": "k_fire"}[dom]
    peak, peak_src = measured_peaks()
    achieved = parts[dom]["achieved_gbs"]
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_src, "kernel": kernel,
                "traffic": profiled_traffic({"k_life": "k_life_ltl_moore5_8192.md",
                                             "k_fire": "k_fire_forest_fire_16384.md"}[kernel])}
    for name in parts:
        parts[name]["hbm_frac_per_effective_step"] = parts[name]["achieved_gbs"] / peak
    # the forest fire's compute roof: one Philox4x32-10 draw per cell-update, measured alone
    rate = ctypes.c_double()
    capi.check(lib.gbca_philox_rate(20_000_000_000, ctypes.byref(rate)))
    fire_draws = parts["fire"]["gcell_updates_s"] * 1e9
    philox_roof = {"kernel": "k_fire", "achieved": fire_draws / 1e9, "peak": rate.value / 1e9, "unit": "Gdraws/s",
                   "frac": fire_draws / rate.value, "peak_source": "measured in this run (draw-only kernel)"}
    # the kernel's own pipe roof: its fmaheavy cycles per 32 cell-updates (from the ncu pipe
    # counters of a capture of this kernel) on every SM sub-partition at the SM clock seen in the
    # timed region
    sm_mhz = clocks.summary().get("sm_mhz") or 2070.0
    pipe_roof = 32 * 4 * 152 * sm_mhz * 1e6 / FIRE_FMAHEAVY_CYCLES_PER_WARP / 1e9
    philox_roof["pipe_roof"] = {"pipe": "fmaheavy (integer multiplies)", "cycles_per_32_cells": FIRE_FMAHEAVY_CYCLES_PER_WARP,
                                "gcell_updates_s": pipe_roof, "frac": fire_draws / 1e9 / pipe_roof,
                                "source": "instruction mix from ncu pipe counters x SM clock"}

    # ---- end to end through the C ABI with host buffers
    host_in = [torch.from_numpy(np.ascontiguousarray(a.T)).pin_memory() for a in (ltl0, fire0)]
    host_out = [[torch.empty_like(x).pin_memory() for x in host_in] for _ in range(2)]
    # two handles per lattice used in turn (the second takes the tuned geometry from the cache),
    # each on its own stream: a step's input copy runs on one handle's stream while the previous
    # step sweeps on the other's
    pairs = []
    for d, h in zip((d1, d2), handles):
        h2 = ctypes.c_void_p()
        capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(h2)))
        pairs.append((h, h2))
    for h in handles:
        capi.check(lib.gbca_set_stream(h, None))

    def step_e2e(k):
        # every copy queued: the inputs in, the sweeps, the results out into the step's result
        # buffers (two sets used in turn)
        hs = [pr[k % 2] for pr in pairs]
        for i, (h, hi) in enumerate(zip(hs, host_in)):
            capi.check(lib.gbca_set_state_async(h, ctypes.c_void_p(hi.data_ptr()), hi.numel()))
            if i == 0:
                capi.check(lib.gbca_advance(h, 0, LTL["steps"], None, 0))
            else:
                capi.check(lib.gbca_advance(h, 0, FIRE["steps"], params_fire, 2))
        for h, ho in zip(hs, host_out[k % 2]):
            capi.check(lib.gbca_get_state_async(h, ctypes.c_void_p(ho.data_ptr()), ho.numel()))

    def sync_all():
        for pr in pairs:
            for h in pr:
                capi.check(lib.gbca_sync(h))

    step_e2e(0)
    step_e2e(1)
    sync_all()
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as e2e_clocks:
        t0 = time.perf_counter()
        for k in range(args.steps):
            step_e2e(k)
        sync_all()
        e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    nbytes = sum(x.numel() for x in host_in)
    last = host_out[(args.steps - 1) % 2]
    e2e_equal = all(np.array_equal(o.numpy(), r) for o, r in zip(last, resident_out))
    e2e = {"value": replica_value(world, cell_updates(), e2e_s / args.steps * 1e3), "unit": "Gcell-updates/s",
           "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_s / args.steps * 1e3,
           "results_equal_resident": e2e_equal, "clocks": e2e_clocks.summary()}
    for pr in pairs:
        lib.gbca_destroy(pr[1])
    if not e2e_equal:
        raise SystemExit("end-to-end results differ from the device-resident run's")

    batched = None
    if rank == 0 and not args.no_batched:
        batched = bench_batched(capi, lib, max(1, args.warmup // 2), max(1, args.steps // 2))
    saves = bench_saves(ca) if rank == 0 and not args.no_saves else None
    sparse = bench_sparse(ca) if rank == 0 and not args.no_sparse else None
    lenia = bench_lenia(capi, lib) if rank == 0 and not args.no_lenia else None
    served = bench_served(capi, lib) if rank == 0 and not args.no_serve else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_sample(os.cpu_count() or 1)
    for h in handles:
        lib.gbca_destroy(h)
    if rank == 0:
        line = {"metric": "Gcell-updates/s", "value": value, "unit": "Gcell-updates/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "int8", "data": "synthetic",
                "config": {"workload": WORKLOAD,
                           "cell_updates_per_step": cell_updates(), "parallelism": f"replicas x{world}",
                           "geometry": {k: {"steps_per_pass": v[0], "tile_rows": v[1], "tma_staging": v[2]}
                                        for k, v in geometry.items()},
                           "l2": "inputs larger than L2: the 16384^2 state is 268 MB, and each step re-copies "
                                 "335 MB of initial states"},
                "roofline": roofline, "philox_roof": philox_roof, "parts": parts, "e2e": e2e, "gpu_launches": launches,
                "clocks": clocks.summary(), "cpu_baseline": cpu, "batched": batched, "served": served,
                "saves": saves, "sparse": sparse, "lenia": lenia}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
