"""The sharded single sweep's host side: slabs along the last axis (src/backends.jl:457-479), halo
exchange, and summaries added across ranks. Host shards stand in for the GPUs: each holds its
padded slab as a NumPy array and steps it with the oracle, on a copy of the lattice in which
every column outside the slab is zero (so a slab's outer columns read wrong neighbours, as a
GPU slab's do). The whole lattice, gathered from the ranks' owned columns after several
exchanges, must equal the oracle's single run; counts and Moran's I, added across ranks, the
oracle's state_counts and morans_i (src/measures.jl:14-20,91-107). Ranks run in one process
(LocalGroup) and as two gloo processes (ProcessGroupTransport)."""
import os
import zlib

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _ca():
    import __graft_entry__ as ge
    return ge.load_package()


def _map(b, g, n, o):
    g = np.asarray(g)
    if b == o.PERIODIC:
        return g % n
    if b == o.REFLECTING:
        m = g % (2 * n)
        return np.where(m < n, m, 2 * n - 1 - m)
    return np.where((g >= 0) & (g < n), g, -1)


class OracleSlab:
    """A padded slab on the host, stepped by the oracle on a zero-filled copy of the lattice."""

    def __init__(self, o, P, slab, u):
        self.o, self.P, self.slab = o, P, slab
        self.n1, self.n2 = P.n1, P.n2
        self.cols = (slab.col0 + np.arange(slab.width)) % self.n2
        self.u = np.asfortranarray(np.asarray(u, np.int8)[:, self.cols])

    def _view(self):
        g = np.zeros((self.n1, self.n2), np.int8, order="F")
        g[:, self.cols] = self.u
        return g

    def step(self, t, k, params):
        out = self.o.run_array(self.P, self._view(), t, k, params)
        self.u = np.asfortranarray(out[:, self.cols])

    def columns(self, a, k):
        return torch.from_numpy(self.u.T[a:a + k])  # a view: receives land in the slab

    def read(self):
        return self.u

    def sums(self, j_lo, j_hi):
        o, g = self.o, self._view().astype(np.int64)
        b1, b2 = self.P.boundary
        own = self.cols[j_lo:j_hi]
        x = g[:, own]
        out = np.zeros(261, np.int64)
        out[:256] = np.bincount((x + 128).ravel(), minlength=256)
        out[256], out[257] = x.sum(), (x * x).sum()
        ii = np.arange(self.n1)[:, None]
        jj = own[None, :]
        for di, dj in ((0, -1), (-1, 0), (1, 0), (0, 1)):
            a = _map(b1, ii + di, self.n1, o) + 0 * jj
            b = _map(b2, jj + dj, self.n2, o) + 0 * ii
            ok = (a >= 0) & (b >= 0)
            y = g[np.where(ok, a, 0), np.where(ok, b, 0)]
            out[258] += (x * y)[ok].sum()
            out[259] += (x + y)[ok].sum()
            out[260] += ok.sum()
        return out


def _case(name, o, ca):
    """(product problem, scheme, oracle problem, params, steps) of a named case."""
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    if name == "fire grid":
        n1, n2 = 40, 61
        u0 = rng.integers(0, 3, (n1, n2)).astype(np.int8)
        prob = ca.CAProblem.new(ca.ForestFire(), u0, 12, {"p": 0.2, "f": 0.02}, space=ca.Grid(n1, n2), seed=9)
        P = o.Problem(o.RULE_FOREST_FIRE, n1, n2, nbhd=o.VON_NEUMANN, seed=9, boundary=(o.CONSTANT, o.CONSTANT))
        return prob, ca.Synchronous(), P, (0.2, 0.02), 12
    if name == "ltl torus":
        n1, n2 = 33, 70
        u0 = (rng.random((n1, n2)) < 0.45).astype(np.int8)
        rule = ca.Life(range(5, 12), range(4, 14), neighbourhood=ca.Moore(2))
        prob = ca.CAProblem.new(rule, u0, 10, space=ca.Torus(n1, n2))
        P = o.Problem(o.RULE_LIFE, n1, n2, radius=2, birth=o.mask(range(5, 12)), survive=o.mask(range(4, 14)))
        return prob, ca.Synchronous(), P, None, 10
    if name == "generations checkerboard, odd torus":
        n1, n2 = 21, 45
        u0 = rng.integers(0, 4, (n1, n2)).astype(np.int8)
        prob = ca.CAProblem.new(ca.Generations("B2/S345/C4"), u0, 9, space=ca.Torus(n1, n2))
        P = o.Problem(o.RULE_GENERATIONS, n1, n2, birth=o.mask([2]), survive=o.mask([3, 4, 5]), states=4,
                      scheme=o.CHECKERBOARD)
        return prob, ca.Checkerboard(), P, None, 9
    if name == "stochastic life, reflecting":
        n1, n2 = 30, 52
        u0 = (rng.random((n1, n2)) < 0.4).astype(np.int8)
        space = ca.Lattice((n1, n2), (ca.Periodic(), ca.Reflecting()))
        prob = ca.CAProblem.new(ca.Life(), u0, 11, space=space, seed=4)
        P = o.Problem(o.RULE_LIFE, n1, n2, birth=o.mask([3]), survive=o.mask([2, 3]), seed=4,
                      boundary=(o.PERIODIC, o.REFLECTING), scheme=o.STOCHASTIC, scheme_p=0.6)
        return prob, ca.Stochastic(0.6), P, None, 11
    raise KeyError(name)


NAMES = ["fire grid", "ltl torus", "generations checkerboard, odd torus", "stochastic life, reflecting"]


def test_slab_bounds_and_plan(gbca):
    sl = gbca.slabs
    assert sl.slab_bounds(10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert sl.halo_columns(5, 6) == 30 and sl.halo_columns(1, 3, 2) == 6
    torus = sl.plan(100, 4, 6, True)
    assert [(s.j0, s.j1, s.lpad, s.rpad, s.left, s.right) for s in torus] == [
        (0, 25, 6, 6, 3, 1), (25, 50, 6, 6, 0, 2), (50, 75, 6, 6, 1, 3), (75, 100, 6, 6, 2, 0)]
    assert torus[0].col0 == -6 and torus[0].width == 37
    grid = sl.plan(100, 4, 6, False)
    assert [(s.lpad, s.rpad, s.left, s.right) for s in grid] == [(0, 6, None, 1), (6, 6, 0, 2), (6, 6, 1, 3),
                                                                 (6, 0, 2, None)]
    assert sl.plan(50, 1, 9, True)[0].width == 50
    with pytest.raises(gbca.ArgumentError):
        sl.plan(20, 4, 6, True)  # slabs of 5 columns, halo 6
    with pytest.raises(gbca.ArgumentError):
        sl.plan(30, 2, 10, True)  # padded slab 35 > 30
    with pytest.raises(gbca.ArgumentError):
        sl.slab_bounds(3, 4)
    # two ranks on a torus: the sends of one pair with the receives of the other in posting order
    a, b = sl.plan(40, 2, 3, True)
    sa = [op for op in sl.exchange_ops(a) if op[0] == "send"]
    rb = [op for op in sl.exchange_ops(b) if op[0] == "recv"]
    assert [(op[3], op[4]) for op in sa] == [(20, 3), (3, 3)]
    assert [(op[3], op[4]) for op in rb] == [(0, 3), (23, 3)]


def test_slabs_refuse_kernel_fields(gbca):
    ca = gbca
    u0 = np.zeros((12, 10), np.float32)
    lenia = ca.CAProblem.new(ca.Lenia(precision="Float32"), u0, 1)
    with pytest.raises(ca.UnsupportedCombinationError):
        ca.slabs.LocalGroup(lenia, ca.Synchronous(), 2, 1, make_shard=lambda s: None)


def test_morans_from_sums_is_exact(gbca, oracle):
    rng = np.random.default_rng(3)
    u = rng.integers(0, 3, (17, 23)).astype(np.int8)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, 17, 23, nbhd=oracle.VON_NEUMANN,
                       boundary=(oracle.CONSTANT, oracle.PERIODIC))
    sl = gbca.slabs
    sh = OracleSlab(oracle, P, sl.plan(23, 1, 0, True)[0], u)
    counts, other, mi = sl.summaries_from_sums(sh.sums(0, 23), 17 * 23)
    assert counts == [int((u == v).sum()) for v in range(3)] and other == 0
    assert mi == pytest.approx(oracle.morans_i(P, u), rel=1e-12)


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("name", NAMES)
def test_local_group_equals_one_run(gbca, oracle, name, world):
    ca = gbca
    prob, scheme, P, params, steps = _case(name, oracle, ca)
    K = 3
    grp = ca.slabs.LocalGroup(prob, scheme, world, K,
                              make_shard=lambda s: OracleSlab(oracle, P, s, np.asarray(prob.u0)))
    grp.run(0, steps, params)
    want = oracle.run_array(P, np.asarray(prob.u0), 0, steps, params)
    got = grp.state()
    assert np.array_equal(got, want), f"{(got != want).sum()} cells differ"
    counts, other, mi = grp.summaries(4)
    assert counts == [int((want == v).sum()) for v in range(4)] and other == int((want >= 4).sum())
    assert mi == pytest.approx(oracle.morans_i(P, want), rel=1e-12, nan_ok=True)


def _gloo_rank(rank, world, port, name, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle as o
        o.build()
        ca = _ca()
        prob, scheme, P, params, steps = _case(name, o, ca)
        K = 4
        h = ca.slabs.halo_columns(prob.neighbours.radius, K, ca.slabs.gates_of(scheme))
        periodic = isinstance(prob.space.boundaries[1], ca.Periodic)
        slab = ca.slabs.plan(P.n2, world, h, periodic)[rank]
        tr = ca.slabs.ProcessGroupTransport()
        sw = ca.slabs.SlabSweep(prob, scheme, slab, OracleSlab(o, P, slab, np.asarray(prob.u0)), tr, K)
        sw.run(0, steps, params)
        full = tr.gather_owned(sw.owned(), slab, P.n2)
        summ = sw.summaries(3)
        if rank == 0:
            want = o.run_array(P, np.asarray(prob.u0), 0, steps, params)
            out[rank] = (bool(np.array_equal(full, want)), summ,
                         ([int((want == v).sum()) for v in range(3)], float(o.morans_i(P, want))))
        else:
            out[rank] = (full is None, summ, None)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name", ["fire grid", "generations checkerboard, odd torus"])
def test_two_gloo_ranks_equal_one_run(name):
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = 29500 + (os.getpid() + len(name)) % 400
        procs = [ctx.Process(target=_gloo_rank, args=(r, 2, port, name, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(180)
        assert all(p.exitcode == 0 for p in procs)
        ok0, summ0, (counts, mi) = out[0]
        ok1, summ1, _ = out[1]
        assert ok0 and ok1, "the gathered lattice differs from the oracle's run"
        assert summ0 == summ1 or (summ0[0] == summ1[0] and np.isnan(summ0[2]) and np.isnan(summ1[2]))
        assert summ0[0] == counts
        assert summ0[2] == pytest.approx(mi, rel=1e-12)
