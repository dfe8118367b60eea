"""Active-tile sweeps (GB300Backend(background=...)), the GPU form of SparseBackend
(src/sparse.jl): only tiles holding a non-background cell, and tiles within reach of them,
are swept. Results must equal the oracle's dense sweep cell for cell, as
test/backend_conformance.jl:187-189 demands of SparseBackend on the quiescent cases."""
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


def _patch(name, n1, n2, C, size, bg=0):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    u = np.full((n1, n2), bg, np.int8)
    for _ in range(3):
        i, j = rng.integers(0, n1 - size), rng.integers(0, n2 - size)
        u[i:i + size, j:j + size] = rng.integers(0, C, (size, size))
    return u


CASES = [
    # name, rule, dims, space, scheme, tilesize, steps, saveat
    ("Life, 1000 x 700 torus (partial tiles wrap)", "life", (1000, 700), "torus", "sync", 64, 120, 20),
    ("HighLife, grid, 32-cell tiles", "highlife", (600, 520), "grid", "sync", 32, 80, 40),
    ("Life, Constant(1) edges", "life", (300, 260), "const1", "sync", 64, 40, 20),
    ("Brian's Brain, torus", "brain", (500, 500), "torus", "sync", 64, 60, 30),
    ("Stochastic(0.5) Life", "life", (400, 300), "torus", "stoch", 64, 50, 25),
    ("Larger than Life Moore(4)", "ltl4", (512, 512), "torus", "sync", 128, 30, 15),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_sparse_matches_oracle(ca, oracle, case):
    name, rule, (n1, n2), space, scheme, ts, steps, saveat = case
    o = oracle
    if rule == "life":
        R, P = ca.Life(":conway"), o.Problem(o.RULE_LIFE, n1, n2, birth=o.mask([3]), survive=o.mask([2, 3]))
        C = 2
    elif rule == "highlife":
        R, P = ca.Life(":highlife"), o.Problem(o.RULE_LIFE, n1, n2, birth=o.mask([3, 6]), survive=o.mask([2, 3]))
        C = 2
    elif rule == "ltl4":
        b, s = range(15, 25), range(14, 30)
        R = ca.Life(list(b), list(s), neighbourhood=ca.Moore(4))
        P = o.Problem(o.RULE_LIFE, n1, n2, radius=4, birth=o.mask(b), survive=o.mask(s))
        C = 2
    else:
        R, P = ca.Generations(":brians_brain"), o.Problem(o.RULE_GENERATIONS, n1, n2, birth=o.mask([2]), survive=0,
                                                         states=3)
        C = 3
    if space == "torus":
        sp = ca.Torus(n1, n2)
    elif space == "grid":
        sp = ca.Grid(n1, n2)
        P.boundary = (o.CONSTANT, o.CONSTANT)
    else:
        sp = ca.Grid(n1, n2, boundary=ca.Constant(1))
        P.boundary, P.constant = (o.CONSTANT, o.CONSTANT), (1, 1)
    sch = ca.Synchronous()
    if scheme == "stoch":
        sch = ca.Stochastic(0.5)
        P.scheme, P.scheme_p = o.STOCHASTIC, 0.5
    P.seed = 7
    u0 = _patch(name, n1, n2, C, 40)
    prob = ca.CAProblem.new(R, u0, steps, space=sp, seed=7)
    sol = ca.solve(prob, sch, backend=ca.GB300Backend(background=0, tilesize=ts), saveat=saveat)
    ts_, us = o.solve(P, u0, steps, saveat=saveat, nthreads=16)
    assert sol.t == ts_
    for k, (a, b) in enumerate(zip(sol.u, us)):
        assert np.array_equal(a, b), f"{name}: save {k} differs in {(a != b).sum()} cells"


def test_sparse_fire_through_a_forest(ca, oracle):
    """A forest fire on trees (background 1) with f = 0, p = 0.3: a tree without a burning
    neighbour stays a tree, so the all-tree tiles are quiescent while the front moves."""
    n1, n2 = 700, 500
    u0 = np.ones((n1, n2), np.int8)
    u0[350, 250] = 2
    u0[10:14, 480:484] = 2
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 150, {"p": 0.3, "f": 0.0}, space=ca.Grid(n1, n2), seed=3)
    got = ca.final_state(ca.solve(prob, ca.Synchronous(), backend=ca.GB300Backend(background=1),
                                  save_everystep=False))
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, n1, n2, nbhd=oracle.VON_NEUMANN, seed=3,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT))
    want = oracle.run_array(P, u0, 0, 150, (0.3, 0.0), nthreads=16)
    assert np.array_equal(got, want) and (want != 1).sum() > 1000


def test_sparse_with_mask_and_state_writes(ca, oracle):
    """A mask, and integ.u changed by a callback mid-run (the tile flags are rebuilt)."""
    n1, n2 = 320, 256
    u0 = _patch("mask", n1, n2, 2, 30)
    mask = np.ones((n1, n2), bool)
    mask[100:140, :] = False
    prob = ca.CAProblem.new(ca.Life(":conway"), u0, 60, mask=mask)

    def affect(integ):
        u = integ.u.copy()
        u[200:210, 20:30] = 1
        integ.u = u

    cb = ca.DiscreteCallback(lambda u, t, integ: t == 25, affect)
    got = ca.final_state(ca.solve(prob, ca.Synchronous(), backend=ca.GB300Backend(background=0), callback=cb,
                                  save_everystep=False))
    P = oracle.Problem(oracle.RULE_LIFE, n1, n2, birth=oracle.mask([3]), survive=oracle.mask([2, 3]))
    E = oracle.Env(mask=mask)
    u = oracle.run_array_env(P, E, u0, 0, 25)
    u[200:210, 20:30] = 1
    want = oracle.run_array_env(P, E, u, 25, 35)
    assert np.array_equal(got, want)


def test_sparse_refusals(ca):
    u = np.zeros((64, 64), np.int8)
    B = ca.GB300Backend(background=0)
    with pytest.raises(ca.ArgumentError):  # B0: an empty neighbourhood gives birth
        ca.solve(ca.CAProblem.new(ca.Life("B0123/S"), u, 3), ca.Synchronous(), backend=B)
    with pytest.raises(ca.ArgumentError):  # growth on empty cells (p > 0): not quiescent
        ca.solve(ca.CAProblem.new(ca.ForestFire(), u, 3, {"p": 0.1, "f": 0.0}), ca.Synchronous(), backend=B)
    with pytest.raises(ca.UnsupportedCombinationError):
        ca.solve(ca.CAProblem.new(ca.Life(":conway"), u, 3), ca.Checkerboard(), backend=B)
    with pytest.raises(ca.ArgumentError):  # Generations' dying states always move on
        ca.solve(ca.CAProblem.new(ca.Generations(":brians_brain"), u, 3), ca.Synchronous(),
                 backend=ca.GB300Backend(background=2))


def test_sparse_generations_on_live_background(ca, oracle):
    """Background 1 for a Generations rule that keeps a fully live neighbourhood alive
    (S8 on Moore(1)): the bit-sliced kernel's two state planes against that background."""
    n1, n2 = 480, 352
    u0 = _patch("gen-bg1", n1, n2, 4, 36, bg=1)
    prob = ca.CAProblem.new(ca.Generations("B2/S345678/C4"), u0, 40)
    sol = ca.solve(prob, ca.Synchronous(), backend=ca.GB300Backend(background=1, tilesize=32), saveat=10)
    P = oracle.Problem(oracle.RULE_GENERATIONS, n1, n2, birth=oracle.mask([2]), survive=oracle.mask(range(3, 9)),
                       states=4)
    ts, us = oracle.solve(P, u0, 40, saveat=10, nthreads=16)
    assert sol.t == ts and all(np.array_equal(a, b) for a, b in zip(sol.u, us))
    assert (us[-1] != 1).sum() > 0
