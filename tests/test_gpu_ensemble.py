"""Batched ensembles on the GPU: one persistent launch over instances of different sizes,
rules, boundaries, seeds, parameters and step counts must give, instance by instance, the
final states of one solve per instance and of the oracle, and state counts / Moran's I
identical (==) to the single-handle device summaries (src/problem.jl:571-589,
src/measures.jl:14-20,91-107). ABC on the batched ensemble equals the serial ensemble
(test/test_calibration.jl:21-33)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ca():
    import __graft_entry__ as ge
    ge.build()
    m = ge.load_package()
    if m.capi.lib().gbca_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return m


def mixed_problems(ca, n=36, seed=7):
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(n):
        side1 = int(rng.integers(10, 320))
        side2 = int(rng.integers(10, 320))
        steps = int(rng.integers(5, 40))
        kind = i % 4
        if kind == 0:
            rule, space, p, C = ca.ForestFire(), ca.Grid(side1, side2), {"p": float(rng.uniform(0.01, 0.3)),
                                                                        "f": float(rng.uniform(1e-4, 1e-2))}, 3
        elif kind == 1:
            rule, space, p, C = ca.Life("B3/S23"), ca.Torus(side1, side2), None, 2
        elif kind == 2:
            rule, space, p, C = ca.Generations(":brians_brain"), ca.Torus(side1, side2), None, 3
        else:
            rule = ca.Life(range(3, 9), range(2, 10), neighbourhood=ca.Moore(2))
            space, p, C = ca.Lattice((side1, side2), (ca.Reflecting(), ca.Constant(0))), None, 2
        u0 = rng.integers(0, C, (side1, side2)).astype(np.int8)
        probs.append(ca.CAProblem.new(rule, u0, steps, p, space=space, seed=100 + i))
    return probs


def single(ca, prob, t0, nsteps, u):
    """One problem alone through a GB300 handle: final state and device summaries."""
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    ca.set_state(B, st, u)
    for t in range(t0, t0 + nsteps):
        ca.advance(B, st, prob, ca.Synchronous(), prob.p, t)
    out = ca.current_state(B, st)
    counts, other, mi = ca.device_summaries(st, 3)
    st.close()
    return out, counts, other, mi


def test_batched_equals_one_solve_per_instance(ca, oracle):
    probs = mixed_problems(ca)
    ens = ca.BatchedEnsemble(probs)
    ens.set_initial_states()
    states = [np.asarray(p.u0) for p in probs]
    t0 = [0] * len(probs)
    for rnd in range(2):  # the second run continues the first
        steps = [p.tspan[1] for p in probs] if rnd == 0 else [7 + (i % 5) for i in range(len(probs))]
        ens.run(t0=t0, nsteps=steps)
        counts, other, morans = ens.summaries(3)
        for i, p in enumerate(probs):
            got = ens.state(i)
            want, c1, o1, m1 = single(ca, p, t0[i], steps[i], states[i])
            assert np.array_equal(got, want), f"instance {i} ({p.rule}, {p.space.dims}) run {rnd}"
            assert list(counts[i]) == c1 and other[i] == o1
            assert (morans[i] == m1) or (np.isnan(morans[i]) and np.isnan(m1)), (i, morans[i], m1)
            states[i] = got
            t0[i] += steps[i]
    # and against the oracle for a few instances
    for i in (0, 1, 2, 3):
        p = probs[i]
        o = oracle
        if isinstance(p.rule, ca.ForestFire):
            P = o.Problem(o.RULE_FOREST_FIRE, *p.space.dims, nbhd=o.VON_NEUMANN, seed=p.seed,
                          boundary=(o.CONSTANT, o.CONSTANT))
            par = (p.p["p"], p.p["f"])
        elif isinstance(p.rule, ca.Generations):
            P = o.Problem(o.RULE_GENERATIONS, *p.space.dims, birth=p.rule.birth, survive=p.rule.survive, states=3,
                          seed=p.seed)
            par = None
        elif p.neighbours.radius == 1:
            P = o.Problem(o.RULE_LIFE, *p.space.dims, birth=p.rule.birth, survive=p.rule.survive, seed=p.seed)
            par = None
        else:
            P = o.Problem(o.RULE_LIFE, *p.space.dims, radius=2, birth=p.rule.birth, survive=p.rule.survive,
                          boundary=(o.REFLECTING, o.CONSTANT), seed=p.seed)
            par = None
        want = o.run_array(P, p.u0, 0, t0[i], par, nthreads=8)
        assert np.array_equal(states[i], want), i
    ens.close()


def test_forest_fire_ensemble_from_empty(ca):
    """The batched forest-fire ensemble shape (square sides log-uniform, p ~ U(0.01, 0.1),
    f ~ LogU(1e-5, 1e-3), seeds 1..n, all empty at t = 0), at 48 instances and 120 steps."""
    rng = np.random.Generator(np.random.PCG64(4096))
    n = 48
    sides = np.round(np.exp(rng.uniform(np.log(64), np.log(1024), n))).astype(int)
    ps = rng.uniform(0.01, 0.1, n)
    fs = np.exp(rng.uniform(np.log(1e-5), np.log(1e-3), n))
    probs = [ca.CAProblem.new(ca.ForestFire(), np.zeros((s, s), np.int8), 120, {"p": ps[i], "f": fs[i]},
                              space=ca.Grid(int(s), int(s)), seed=i + 1) for i, s in enumerate(sides)]
    res = ca.solve_ensemble(ca.EnsembleProblem(probs[0]), trajectories=1)  # the API path works
    assert len(res.u) == 1
    ens = ca.BatchedEnsemble(probs)
    ens.fill(0)
    ens.run()
    counts, other, morans = ens.summaries(3)
    for i in (0, 5, int(np.argmax(sides)), int(np.argmin(sides))):
        _, c1, o1, m1 = single(ca, probs[i], 0, 120, np.zeros((sides[i], sides[i]), np.int8))
        assert list(counts[i]) == c1 and other[i] == o1 and morans[i] == m1
    assert counts.sum() == int((sides.astype(np.int64) ** 2).sum())
    ens.close()


def test_abc_batched_equals_serial(ca):
    """Proposal i runs with seed prob.seed + i and p = proposals[i]; distances and acceptance
    do not depend on the ensemble algorithm (test/test_calibration.jl:21-33)."""
    u0 = np.zeros((40, 30), np.int8)
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 25, {"p": 0.1, "f": 0.001}, space=ca.Grid(40, 30), seed=3)
    observed = ca.final_state(ca.solve(prob.remake(seed=100), save_everystep=False))
    trees = lambda u: int((np.asarray(u) == 1).sum())
    dist = lambda sol, obs: abs(trees(ca.final_state(sol)) - trees(obs))
    proposals = [{"p": float(b), "f": 0.001} for b in np.arange(0.02, 0.4, 0.02)]
    res = ca.abc_rejection(prob, proposals, dist, observed, keep=4)
    ser = ca.abc_rejection(prob, proposals, dist, observed, keep=4, ensemblealg=object())
    assert res.proposal_distances == ser.proposal_distances
    assert res.samples == ser.samples and len(res.samples) == 4
    for i in (1, 6, 12):
        s = ca.solve(prob.remake(p=proposals[i - 1], seed=prob.seed + i), save_everystep=False)
        assert res.proposal_distances[i - 1] == dist(s, observed)
    assert res.distances == sorted(res.proposal_distances)[:4]


def test_batched_geometries_and_tuner(ca):
    """Every tile side and pass depth of the batched kernel gives the same states and
    summaries; the tuner restores the states it probes and picks one of the candidates."""
    probs = mixed_problems(ca, n=20, seed=11)
    steps = [p.tspan[1] for p in probs]
    ref = None
    for tile in (64, 128, 192):
        for depth in (1, 3, 0):
            ens = ca.BatchedEnsemble(probs)
            ens.set_initial_states()
            ens.set_geometry(tile, depth)
            ens.run(nsteps=steps)
            out = [ens.state(i) for i in range(len(probs))], ens.summaries(3)
            ens.close()
            if ref is None:
                ref = out
                continue
            assert all(np.array_equal(a, b) for a, b in zip(out[0], ref[0])), (tile, depth)
            assert np.array_equal(out[1][0], ref[1][0]) and np.array_equal(out[1][1], ref[1][1])
    ens = ca.BatchedEnsemble(probs)
    ens.set_initial_states()
    tile, depth = ens.tune(probe_steps=6)
    assert tile in (64, 128, 192) and depth in (2, 4, 0)
    assert all(np.array_equal(ens.state(i), np.asarray(p.u0)) for i, p in enumerate(probs))
    ens.run(nsteps=steps)
    assert all(np.array_equal(ens.state(i), ref[0][i]) for i in range(len(probs)))
    ens.close()
    with pytest.raises(ca.ArgumentError):
        ca.BatchedEnsemble(probs).set_geometry(100, 0)


def large_split_problems(ca):
    """Forest fires on both sides of the 2^14-cell floor, ragged sides (not multiples of the
    256 x 128 output tile), every boundary kind the fire kernel maps, and a Life instance that
    always stays on the persistent kernel."""
    rng = np.random.default_rng(2024)
    shapes = [(130, 140), (300, 257), (1000, 20), (513, 129), (64, 300), (40, 50), (260, 600), (129, 127)]
    spaces = [lambda a, b: ca.Grid(a, b), lambda a, b: ca.Torus(a, b),
              lambda a, b: ca.Lattice((a, b), (ca.Reflecting(), ca.Constant(1))),
              lambda a, b: ca.Lattice((a, b), (ca.Constant(2), ca.Periodic()))]
    probs = []
    for i, (a, b) in enumerate(shapes):
        u0 = rng.integers(0, 3, (a, b)).astype(np.int8)
        p = {"p": float(rng.uniform(0.02, 0.2)), "f": float(rng.uniform(1e-4, 1e-2))}
        probs.append(ca.CAProblem.new(ca.ForestFire(), u0, 20, p, space=spaces[i % 4](a, b), seed=300 + i))
    probs.append(ca.CAProblem.new(ca.Life("B3/S23"), rng.integers(0, 2, (200, 180)).astype(np.int8), 20,
                                  space=ca.Torus(200, 180), seed=9))
    return probs


@pytest.mark.parametrize("k", [1, 3, 16])
def test_large_instances_as_batched_passes(ca, k):
    """Instances of at least 2^14 cells run as batched multi-CTA passes of k steps: states and
    summaries equal one solve per instance, over two runs with step counts that are not
    multiples of k (0 included), from t0 != 0."""
    probs = large_split_problems(ca)
    ens = ca.BatchedEnsemble(probs)
    ens.set_initial_states()
    ens.set_large(1 << 14, k)
    g = ens.geometry()
    assert g["large_cells"] == 1 << 14 and g["large_steps"] == k
    assert g["n_large"] == sum(isinstance(p.rule, ca.ForestFire) and np.prod(p.space.dims) >= 1 << 14 for p in probs)
    states = [np.asarray(p.u0) for p in probs]
    t0 = [3 + i for i in range(len(probs))]
    for rnd in range(2):
        steps = [(0, 1, 5, 13, 29, 2, 17, 8, 11)[(i + rnd) % 9] for i in range(len(probs))]
        ens.run(t0=t0, nsteps=steps)
        counts, other, morans = ens.summaries(3)
        for i, p in enumerate(probs):
            got = ens.state(i)
            want, c1, o1, m1 = single(ca, p, t0[i], steps[i], states[i])
            assert np.array_equal(got, want), f"instance {i} ({p.space.dims}) run {rnd} k {k}"
            assert list(counts[i]) == c1 and other[i] == o1, (i, rnd)
            assert (morans[i] == m1) or (np.isnan(morans[i]) and np.isnan(m1)), (i, morans[i], m1)
            states[i] = got
            t0[i] += steps[i]
    ens.close()


def test_large_split_tuner_and_refusals(ca):
    probs = large_split_problems(ca)
    ens = ca.BatchedEnsemble(probs)
    ens.set_initial_states()
    tile, depth = ens.tune(probe_steps=4)
    g = ens.geometry()
    assert (tile, depth) == (g["tile"], g["depth"])
    assert g["large_cells"] in (0, 1 << 14, 1 << 15, 1 << 16, 1 << 17, 1 << 18, 1 << 20)
    assert g["large_steps"] in (1, 2, 4)
    assert all(np.array_equal(ens.state(i), np.asarray(p.u0)) for i, p in enumerate(probs))
    with pytest.raises(ca.ArgumentError):
        ens.set_large(1000, 1)  # below the floor
    with pytest.raises(ca.ArgumentError):
        ens.set_large(1 << 18, 17)
    ens.set_large(0, 1)
    assert ens.geometry()["n_large"] == 0
    ens.close()


def test_config_sample_of_the_bench_ensemble_against_the_oracle(ca, oracle):
    """The bench's batched workload (4096 forest-fire instances from its own generator, all empty
    at t = 0, 500 steps, seeds 1..4096) run whole, under the bench's tuned geometry (64-cell
    tiles, 4 steps per pass, instances of 2^14 cells and more as batched one-step passes) and
    under the default one; 16 instances checked against the oracle: the smallest, the largest,
    the instances just below and at the large-instance split, and 12 at random. Final states are
    equal, state counts equal and Moran's I equal to 1e-12 (src/measures.jl:14-20,91-107)."""
    import ctypes
    import os

    import bench

    o = oracle
    capi, lib = ca.capi, ca.capi.lib()
    sides, ps, fs, seeds = bench.ensemble_instances()
    n, steps = len(sides), bench.ENS["steps"]
    order = np.argsort(sides, kind="stable")
    below = int(order[np.searchsorted(sides[order], 128) - 1])  # largest side under 128 (< 2^14 cells)
    at = int(order[np.searchsorted(sides[order], 128)])          # first side of 128 or more
    rng = np.random.default_rng(12)
    pick = [int(order[0]), int(order[-1]), below, at] + [int(x) for x in rng.choice(n, 12, replace=False)]
    want = {}
    for i in pick:
        P = o.Problem(o.RULE_FOREST_FIRE, int(sides[i]), int(sides[i]), nbhd=o.VON_NEUMANN, seed=int(seeds[i]),
                      boundary=(o.CONSTANT, o.CONSTANT))
        u = o.run_array(P, np.zeros((sides[i], sides[i]), np.int8), 0, steps, (ps[i], fs[i]), os.cpu_count() or 1)
        want[i] = (u, o.state_counts(u, 3), o.morans_i(P, u))
    descs = (capi.Desc * n)()
    for i in range(n):
        descs[i] = bench.fire_desc(capi, sides[i], seeds[i])
    T0 = (ctypes.c_int64 * n)()
    S = (ctypes.c_int64 * n)(*([steps] * n))
    Par = (ctypes.c_double * (2 * n))(*np.column_stack([ps, fs]).ravel().tolist())
    for geometry in ("bench", "default"):
        e = ctypes.c_void_p()
        capi.check(lib.gbca_ensemble_create(descs, n, ctypes.byref(e)))
        try:
            if geometry == "bench":
                capi.check(lib.gbca_ensemble_set_geometry(e, 64, 4))
                capi.check(lib.gbca_ensemble_set_large(e, 1 << 14, 1))
            capi.check(lib.gbca_ensemble_fill(e, 0))
            capi.check(lib.gbca_ensemble_run(e, T0, S, Par, 2))
            capi.check(lib.gbca_ensemble_sync(e))
            C = (ctypes.c_int64 * (3 * n))()
            O = (ctypes.c_int64 * n)()
            M = (ctypes.c_double * n)()
            capi.check(lib.gbca_ensemble_summaries(e, C, 3, O, M))
            for i in pick:
                u, (c3, other), mi = want[i]
                got = np.empty((sides[i], sides[i]), np.int8, order="F")
                capi.check(lib.gbca_ensemble_get_state(e, i, got.ctypes.data, got.nbytes))
                assert np.array_equal(got, u), f"{geometry}: instance {i} (side {sides[i]}) differs from the oracle"
                assert [C[3 * i + k] for k in range(3)] == c3 and O[i] == other == 0, (geometry, i)
                assert M[i] == pytest.approx(mi, rel=1e-12, abs=1e-15), (geometry, i, M[i], mi)
        finally:
            lib.gbca_ensemble_destroy(e)
    assert sum(want[i][1][0][1] for i in pick) > 0  # trees grew: the comparison means something
