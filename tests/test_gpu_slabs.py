"""The sharded single sweep on the GPU: every slab a libgbca handle placed with gbca_set_slab
(global cell ids and Checkerboard parities), two to four slabs run in one process on one GPU
with the halo exchanged by device copies between passes (LocalGroup). The whole lattice from
the slabs' owned columns must equal the oracle's run (src/backends.jl:457-479 splits the same
sweep among threads), on every kernel the slabs reach: the bit-sliced kernel (Larger than Life,
gated Life and Generations), the forest-fire kernel (synchronous, gated, masked) and the
general kernel; counts and Moran's I added across slabs equal one handle's."""
import zlib

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


def _problem(ca, o, name):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    if name == "LtL Moore(5) torus":
        n1, n2 = 1000, 600
        u0 = (rng.random((n1, n2)) < 0.5).astype(np.int8)
        rule = ca.Life(range(34, 46), range(34, 59), neighbourhood=ca.Moore(5))
        prob = ca.CAProblem.new(rule, u0, 12, space=ca.Torus(n1, n2))
        P = o.Problem(o.RULE_LIFE, n1, n2, radius=5, birth=o.mask(range(34, 46)), survive=o.mask(range(34, 59)))
        return prob, ca.Synchronous(), P, None, 12, 6
    if name == "forest fire grid":
        n1, n2 = 1000, 700
        u0 = rng.integers(0, 3, (n1, n2)).astype(np.int8)
        prob = ca.CAProblem.new(ca.ForestFire(), u0, 10, {"p": 0.05, "f": 0.002}, space=ca.Grid(n1, n2), seed=3)
        P = o.Problem(o.RULE_FOREST_FIRE, n1, n2, nbhd=o.VON_NEUMANN, seed=3, boundary=(o.CONSTANT, o.CONSTANT))
        return prob, ca.Synchronous(), P, (0.05, 0.002), 10, 4
    if name == "forest fire Stochastic(0.7), torus":
        n1, n2 = 512, 301
        u0 = rng.integers(0, 3, (n1, n2)).astype(np.int8)
        prob = ca.CAProblem.new(ca.ForestFire(), u0, 9, {"p": 0.05, "f": 0.01}, space=ca.Torus(n1, n2), seed=8)
        P = o.Problem(o.RULE_FOREST_FIRE, n1, n2, nbhd=o.VON_NEUMANN, seed=8, scheme=o.STOCHASTIC, scheme_p=0.7)
        return prob, ca.Stochastic(0.7), P, (0.05, 0.01), 9, 3
    if name == "Life Checkerboard, odd torus":
        n1, n2 = 300, 251
        u0 = (rng.random((n1, n2)) < 0.4).astype(np.int8)
        prob = ca.CAProblem.new(ca.Life(), u0, 9, space=ca.Torus(n1, n2))
        P = o.Problem(o.RULE_LIFE, n1, n2, birth=o.mask([3]), survive=o.mask([2, 3]), scheme=o.CHECKERBOARD)
        return prob, ca.Checkerboard(), P, None, 9, 4
    if name == "Brian's Brain Stochastic(0.6), reflecting":
        n1, n2 = 257, 190
        u0 = rng.integers(0, 3, (n1, n2)).astype(np.int8)
        space = ca.Lattice((n1, n2), (ca.Periodic(), ca.Reflecting()))
        prob = ca.CAProblem.new(ca.Generations(":brians_brain"), u0, 10, space=space, seed=6)
        P = o.Problem(o.RULE_GENERATIONS, n1, n2, birth=o.mask([2]), survive=o.mask([]), states=3, seed=6,
                      boundary=(o.PERIODIC, o.REFLECTING), scheme=o.STOCHASTIC, scheme_p=0.6)
        return prob, ca.Stochastic(0.6), P, None, 10, 5
    if name == "Generations C=10 Checkerboard, odd torus (general kernel)":
        n1, n2 = 120, 97
        u0 = rng.integers(0, 10, (n1, n2)).astype(np.int8)
        prob = ca.CAProblem.new(ca.Generations("B23/S345/C10"), u0, 8, space=ca.Torus(n1, n2))
        P = o.Problem(o.RULE_GENERATIONS, n1, n2, birth=o.mask([2, 3]), survive=o.mask([3, 4, 5]), states=10,
                      scheme=o.CHECKERBOARD)
        return prob, ca.Checkerboard(), P, None, 8, 2
    if name == "masked forest fire, Constant(1) x reflecting":
        n1, n2 = 400, 330
        u0 = rng.integers(0, 3, (n1, n2)).astype(np.int8)
        mask = rng.random((n1, n2)) < 0.8
        space = ca.Lattice((n1, n2), (ca.Constant(1), ca.Reflecting()))
        prob = ca.CAProblem.new(ca.ForestFire(), u0, 8, {"p": 0.1, "f": 0.01}, space=space, seed=12, mask=mask)
        P = o.Problem(o.RULE_FOREST_FIRE, n1, n2, nbhd=o.VON_NEUMANN, seed=12, boundary=(o.CONSTANT, o.REFLECTING),
                      constant=(1, 0))
        return prob, ca.Synchronous(), P, (0.1, 0.01), 8, 3
    raise KeyError(name)


NAMES = ["LtL Moore(5) torus", "forest fire grid", "forest fire Stochastic(0.7), torus",
         "Life Checkerboard, odd torus", "Brian's Brain Stochastic(0.6), reflecting",
         "Generations C=10 Checkerboard, odd torus (general kernel)", "masked forest fire, Constant(1) x reflecting"]


def _oracle_run(o, P, prob, params, steps):
    u0 = np.asarray(prob.u0)
    if prob.mask is not None:
        env = o.Env(mask=np.asarray(prob.mask))
        return o.run_array_env(P, env, u0, 0, steps, params, nthreads=16)
    return o.run_array(P, u0, 0, steps, params, nthreads=16)


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("name", NAMES)
def test_slabs_equal_the_oracle(ca, oracle, name, world):
    prob, scheme, P, params, steps, K = _problem(ca, oracle, name)
    grp = ca.slabs.LocalGroup(prob, scheme, world, K)
    try:
        grp.run(0, steps, params)
        got = grp.state()
        want = _oracle_run(oracle, P, prob, params, steps)
        assert np.array_equal(got, want), f"{name}, {world} slabs: {(got != want).sum()} cells differ"
        assert not np.array_equal(want, np.asarray(prob.u0))
        counts, other, mi = grp.summaries(3)
    finally:
        grp.close()
    # one handle's device summaries of the same state
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, scheme)
    ca.set_state(B, st, want)
    c1, o1, m1 = ca.device_summaries(st, 3)
    st.close()
    assert list(counts) == list(c1) and other == o1
    assert mi == pytest.approx(m1, rel=1e-12, nan_ok=True)


def test_four_slabs_of_a_larger_fire_equal_one_handle(ca):
    """A 4096 x 2048 forest-fire Grid in four slabs (TMA-staged one-step tiles), 6 steps with an
    exchange after every 2, against one handle of the whole lattice."""
    n1, n2 = 4096, 2048
    rng = np.random.default_rng(31)
    pct = rng.integers(0, 100, size=(n1, n2))
    u0 = ((pct >= 40).astype(np.int8) + (pct >= 99).astype(np.int8))
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 6, {"p": 0.03, "f": 1e-4}, space=ca.Grid(n1, n2), seed=3)
    grp = ca.slabs.LocalGroup(prob, ca.Synchronous(), 4, 2)
    try:
        grp.run(0, 6, (0.03, 1e-4))
        got = grp.state()
    finally:
        grp.close()
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    for t in range(6):
        ca.advance(B, st, prob, ca.Synchronous(), prob.p, t)
    want = ca.current_state(B, st)
    st.close()
    assert np.array_equal(got, want), f"{(got != want).sum()} cells differ"


def test_set_slab_refusals(ca):
    import ctypes
    lib = ca.capi.lib()
    life = ca.CAProblem.new(ca.Life(), np.zeros((64, 40), np.int8), 3)
    st = ca.allocate_state(ca.GB300Backend(), life, ca.Synchronous())
    with pytest.raises(ca.ArgumentError):
        ca.capi.check(lib.gbca_set_slab(st.handle, 0, 39))  # larger lattice narrower than the slab
    with pytest.raises(ca.ArgumentError):
        ca.capi.check(lib.gbca_set_slab(st.handle, 100, 100))  # first column out of range
    ca.capi.check(lib.gbca_set_slab(st.handle, -5, 100))
    with pytest.raises(ca.UnsupportedCombinationError):
        ca.capi.check(lib.gbca_set_sparse(st.handle, 1, 0, 64))
    ca.capi.check(lib.gbca_set_slab(st.handle, 0, 40))  # a lattice of its own again
    ca.capi.check(lib.gbca_set_sparse(st.handle, 1, 0, 64))
    with pytest.raises(ca.UnsupportedCombinationError):
        ca.capi.check(lib.gbca_set_slab(st.handle, 3, 100))
    sums = (ctypes.c_int64 * 261)()
    with pytest.raises(ca.ArgumentError):
        ca.capi.check(lib.gbca_slab_sums(st.handle, 5, 41, sums))
    st.close()
    lenia = ca.CAProblem.new(ca.Lenia(precision="Float32"), np.zeros((32, 32), np.float32), 1)
    st = ca.allocate_state(ca.GB300Backend(), lenia, ca.Synchronous())
    with pytest.raises(ca.UnsupportedCombinationError):
        ca.capi.check(lib.gbca_set_slab(st.handle, 0, 64))
    st.close()


def _gloo_device_rank(rank, world, port, name, out):
    import os

    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle as o
        import __graft_entry__ as ge
        ca = ge.load_package()
        prob, scheme, P, params, steps, K = _problem(ca, o, name)
        sl = ca.slabs
        h = sl.halo_columns(prob.neighbours.radius, K, sl.gates_of(scheme))
        periodic = isinstance(prob.space.boundaries[1], ca.Periodic)
        slab = sl.plan(prob.space.dims[1], world, h, periodic)[rank]
        tr = sl.ProcessGroupTransport()
        shard = sl.DeviceSlab(prob, scheme, slab)
        sw = sl.SlabSweep(prob, scheme, slab, shard, tr, K)
        sw.run(0, steps, params)
        full = tr.gather_owned(sw.owned(), slab, prob.space.dims[1])
        summ = sw.summaries(3)
        if rank == 0:
            want = _oracle_run(o, P, prob, params, steps)
            out[rank] = (bool(np.array_equal(full, want)), int((full != want).sum()), summ,
                         [int((want == v).sum()) for v in range(3)])
        else:
            out[rank] = (full is None, 0, summ, None)
        shard.close()
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name", ["forest fire grid", "Life Checkerboard, odd torus"])
def test_two_processes_over_gloo_equal_the_oracle(ca, oracle, name):
    """The distributed form end to end on one GPU: two processes, each holding its slab in a
    libgbca handle, the halo exchanged by ProcessGroupTransport over gloo (device columns staged
    through host memory; no kernel waits on another process), the lattice gathered on rank 0
    and compared with the oracle, counts added by an all-reduce."""
    import os

    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = 29100 + (os.getpid() + len(name)) % 700
        procs = [ctx.Process(target=_gloo_device_rank, args=(r, 2, port, name, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
        assert all(p.exitcode == 0 for p in procs)
        ok0, bad, summ0, counts = out[0]
        ok1, _, summ1, _ = out[1]
        assert ok0 and ok1, f"{name}: {bad} cells differ from the oracle"
        assert summ0[0] == counts and summ1[0] == counts
