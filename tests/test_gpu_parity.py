"""GPU parity: the GB300 backend, driven through solve() and the C ABI, reproduces the
oracle (the reference's ReferenceBackend / ArrayBackend arithmetic) bit for bit on the
Int8 conformance cases, as test/backend_conformance.jl:264-287 demands of every backend
(`sol.t == ref.t && sol.u == ref.u`)."""
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


def spec_pair(ca, o, kind, n1, n2, *, nb="moore", r=1, birth=(), survive=(), states=2, bnd=("p", "p"),
              const=(0, 0), seed=0, scheme="sync", sp=1.0, sp32=False, f32=False):
    """The same problem for the product (rule, space, scheme) and for the oracle."""
    bk = {"p": (ca.Periodic(), o.PERIODIC), "r": (ca.Reflecting(), o.REFLECTING)}
    bounds, obounds = [], []
    for a, b in enumerate(bnd):
        if b == "c":
            bounds.append(ca.Constant(const[a]))
            obounds.append(o.CONSTANT)
        else:
            bounds.append(bk[b][0])
            obounds.append(bk[b][1])
    N = ca.Moore(r) if nb == "moore" else ca.VonNeumann(r)
    if kind == "life":
        rule = ca.Life(list(birth), list(survive), neighbourhood=N)
        orule = o.RULE_LIFE
    elif kind == "gen":
        rule = ca.Generations("B" + "".join(map(str, birth)) + "/S" + "".join(map(str, survive)) + f"/C{states}",
                              neighbourhood=N)
        orule = o.RULE_GENERATIONS
    else:
        rule = ca.ForestFire(neighbourhood=N, float32=f32)
        orule = o.RULE_FOREST_FIRE
    scheme = {"sync": ca.Synchronous(), "stoch": ca.Stochastic(sp, float32=sp32), "check": ca.Checkerboard()}[scheme]
    P = o.Problem(orule, n1, n2, nbhd=o.MOORE if nb == "moore" else o.VON_NEUMANN, radius=r,
                  birth=o.mask(birth), survive=o.mask(survive), states=states, boundary=tuple(obounds),
                  constant=tuple(int(c) for c in const), seed=seed,
                  scheme={ca.Synchronous: o.SYNCHRONOUS, ca.Stochastic: o.STOCHASTIC,
                          ca.Checkerboard: o.CHECKERBOARD}[type(scheme)],
                  scheme_p=scheme.p if isinstance(scheme, ca.Stochastic) else 1.0, scheme_p_f32=sp32, params_f32=f32)
    return rule, ca.Lattice((n1, n2), tuple(bounds)), scheme, P


CASES = [
    # name, kind, dims, kwargs, steps, saveat, params
    ("Life on a torus", "life", (20, 24), dict(birth=[3], survive=[2, 3]), 30, 1, None),
    ("Life on a cylinder", "life", (20, 24), dict(birth=[3], survive=[2, 3], bnd=("p", "c")), 30, 7, None),
    ("radius-2 von Neumann, mixed edges", "life", (15, 17),
     dict(nb="vn", r=2, birth=[3], survive=[2, 3, 4, 5], bnd=("r", "c"), const=(0, 1)), 20, 3, None),
    ("Brian's Brain", "gen", (18, 18), dict(birth=[2], survive=[], states=3), 25, 5, None),
    ("Star Wars, reflecting", "gen", (37, 29), dict(birth=[2], survive=[3, 4, 5], states=4, bnd=("r", "r")), 25, 25,
     None),
    ("Moore(4) wider than the torus", "life", (3, 7), dict(r=4, birth=[5, 6, 7], survive=[4, 5, 6, 7, 8]), 8, 1,
     None),
    ("Larger than Life Moore(5) torus", "life", (97, 83), dict(r=5, birth=range(34, 46), survive=range(34, 59)), 40,
     10, None),
    # rules of three and four count intervals: the eight-interval comparator form
    ("Replicator B1357/S1357, reflecting", "life", (150, 70), dict(birth=[1, 3, 5, 7], survive=[1, 3, 5, 7],
                                                                     bnd=("r", "r")), 20, 5, None),
    ("Morley B368/S245 torus", "life", (200, 96), dict(birth=[3, 6, 8], survive=[2, 4, 5]), 30, 10, None),
    ("Moore(2) three intervals, Constant(1) edges", "life", (130, 77),
     dict(r=2, birth=[4, 7, 8, 12], survive=[3, 5, 6, 10, 11], bnd=("c", "c"), const=(1, 1)), 20, 4, None),
    ("Larger than Life Moore(3) grid", "life", (70, 90),
     dict(r=3, birth=range(9, 15), survive=range(8, 20), bnd=("c", "c")), 30, 10, None),
    ("Stochastic(0.4) Life", "life", (20, 20), dict(birth=[3], survive=[2, 3], seed=2, scheme="stoch", sp=0.4), 15,
     1, None),
    ("Stochastic(0.5f0) Life", "life", (33, 20),
     dict(birth=[3], survive=[2, 3], seed=12, scheme="stoch", sp=0.5, sp32=True), 15, 5, None),
    ("Checkerboard majority", "life", (18, 18),
     dict(nb="vn", birth=[5, 6, 7, 8], survive=[4, 5, 6, 7, 8], scheme="check"), 10, 1, None),
    ("Checkerboard odd torus", "life", (19, 17), dict(nb="vn", birth=[2, 3], survive=[1, 2], scheme="check"), 12, 4,
     None),
    # gated schemes in the bit-sliced kernel: Checkerboard across Constant and even Periodic edges,
    # Stochastic on every boundary (gate draws keyed by the mapped cells' ids at the edges)
    ("Checkerboard Life, even torus, tiled", "life", (200, 150), dict(birth=[3], survive=[2, 3], scheme="check"), 40,
     8, None),
    ("Checkerboard Life, Constant grid, odd sides", "life", (75, 61),
     dict(birth=[3], survive=[2, 3], scheme="check", bnd=("c", "c")), 30, 10, None),
    ("Checkerboard Life, odd torus", "life", (51, 40), dict(birth=[3], survive=[2, 3], scheme="check"), 20, 5, None),
    ("Checkerboard Life, odd x reflecting, tiled", "life", (301, 133),
     dict(birth=[3], survive=[2, 3], scheme="check", bnd=("p", "r")), 30, 10, None),
    ("Checkerboard Generations Moore(2), reflecting x odd torus", "gen", (96, 75),
     dict(r=2, birth=[3, 4], survive=[2, 3, 4, 5], states=3, scheme="check", bnd=("r", "p")), 20, 5, None),
    ("Checkerboard Moore(2), even torus x Constant(1)", "life", (128, 90),
     dict(r=2, birth=[5, 6, 7], survive=[4, 5, 6, 7, 8], scheme="check", bnd=("p", "c"), const=(0, 1)), 25, 25, None),
    ("Stochastic(0.3) Moore(2) Life, reflecting", "life", (90, 70),
     dict(r=2, birth=[5, 6, 7], survive=[4, 5, 6, 7, 8], seed=21, scheme="stoch", sp=0.3, bnd=("r", "r")), 30, 6,
     None),
    ("Stochastic(0.6f0) Life, tiled torus", "life", (257, 129),
     dict(birth=[3], survive=[2, 3], seed=22, scheme="stoch", sp=0.6, sp32=True), 40, 40, None),
    ("Stochastic(0.6) Brian's Brain, tiled torus", "gen", (300, 200),
     dict(birth=[2], survive=[], states=3, seed=23, scheme="stoch", sp=0.6), 30, 10, None),
    ("Checkerboard Generations C=4, Constant edges", "gen", (130, 100),
     dict(birth=[2], survive=[3, 4, 5], states=4, scheme="check", bnd=("c", "c"), const=(1, 2)), 24, 6, None),
    ("Stochastic(0.5) Generations Moore(2), cylinder", "gen", (160, 96),
     dict(r=2, birth=[3, 4, 5], survive=[2, 3, 4, 5, 6], states=4, seed=24, scheme="stoch", sp=0.5,
          bnd=("p", "c"), const=(0, 3)), 20, 4, None),
    # von Neumann(1) in the bit-sliced kernel: the row's 3-cell count plus the cells above and below
    ("von Neumann(1) Life-like, tiled torus", "life", (300, 200), dict(nb="vn", birth=[2], survive=[1, 2]), 40, 8,
     None),
    ("von Neumann(1) majority, Checkerboard, Constant grid", "life", (129, 77),
     dict(nb="vn", birth=[3, 4], survive=[2, 3, 4], scheme="check", bnd=("c", "c"), const=(0, 1)), 30, 10, None),
    ("von Neumann(1) Generations C=3, reflecting", "gen", (150, 90),
     dict(nb="vn", birth=[2], survive=[1], states=3, bnd=("r", "r")), 30, 10, None),
    ("von Neumann(1) Stochastic(0.4), cylinder", "life", (200, 64),
     dict(nb="vn", birth=[1, 3], survive=[2, 3], seed=41, scheme="stoch", sp=0.4, bnd=("p", "c")), 25, 5, None),
    # gated forest fires in the fire kernel, one sub-step per launch
    ("forest fire, Checkerboard, Constant grid", "fire", (257, 190),
     dict(nb="vn", seed=51, bnd=("c", "c"), scheme="check"), 20, 5, (0.1, 0.01)),
    ("forest fire, Stochastic(0.3f0), tiled torus", "fire", (700, 300),
     dict(nb="vn", seed=52, scheme="stoch", sp=0.3, sp32=True), 20, 10, (0.05, 0.002)),
    ("forest fire, Checkerboard, reflecting x odd torus, tiled", "fire", (513, 301),
     dict(nb="vn", seed=53, bnd=("r", "p"), scheme="check"), 16, 4, (0.05, 0.002)),
    ("forest fire, Stochastic(1.0), TMA-staged grid", "fire", (1024, 300),
     dict(nb="vn", seed=54, bnd=("c", "c"), scheme="stoch", sp=1.0), 10, 10, (0.05, 0.002)),
    ("forest fire, small grid", "fire", (40, 30), dict(nb="vn", seed=3, bnd=("c", "c")), 30, 3, (0.3, 0.01)),
    ("forest fire, Float32 parameters, torus", "fire", (33, 21), dict(nb="vn", seed=5, f32=True), 30, 10,
     (0.3, 0.01)),
    ("forest fire, tiled grid", "fire", (1000, 700), dict(nb="vn", seed=3, bnd=("c", "c")), 37, 37, (0.05, 0.001)),
    ("forest fire, tiled torus", "fire", (800, 520), dict(nb="vn", seed=8), 21, 7, (0.05, 0.001)),
    ("forest fire, reflecting, Moore(1)", "fire", (130, 90), dict(nb="moore", seed=4, bnd=("r", "r")), 20, 10,
     (0.1, 0.002)),
    ("forest fire, Stochastic(0.7)", "fire", (64, 80), dict(nb="vn", seed=6, scheme="stoch", sp=0.7), 20, 5,
     (0.2, 0.01)),
    ("Brian's Brain, tiled torus", "gen", (300, 200), dict(birth=[2], survive=[], states=3), 30, 10, None),
    ("Generations Moore(2), Constant edges", "gen", (150, 170),
     dict(r=2, birth=[3, 4, 5], survive=[2, 3, 4, 5, 6], states=4, bnd=("c", "c"), const=(1, 2)), 20, 5, None),
    ("Generations C=4 reflecting, tiled", "gen", (400, 130),
     dict(birth=[2], survive=[3, 4, 5], states=4, bnd=("r", "p")), 25, 25, None),
    ("forest fire, Constant(6) and Constant(2) edges", "fire", (600, 290),
     dict(nb="vn", seed=4, bnd=("c", "c"), const=(6, 2)), 12, 4, (0.2, 0.01)),
    ("forest fire, Constant(3) edges", "fire", (280, 130), dict(nb="vn", seed=5, bnd=("c", "p"), const=(3, 0)), 12, 6,
     (0.2, 0.01)),
    ("forest fire, p = 1 and f = 1", "fire", (520, 300), dict(nb="vn", seed=2, bnd=("c", "c")), 10, 3, (1.0, 1.0)),
    ("forest fire, p = 0, f = 1, Float32", "fire", (300, 260), dict(nb="vn", seed=2, f32=True), 9, 9, (0.0, 1.0)),
    ("forest fire, reflecting edges, tiled", "fire", (700, 300), dict(nb="vn", seed=12, bnd=("r", "p")), 17, 17,
     (0.07, 0.003)),
    # n1 a multiple of 16 on a Constant(0) grid: every tile, edges included, staged by TMA
    ("forest fire, TMA-staged grid", "fire", (1024, 600), dict(nb="vn", seed=13, bnd=("c", "c")), 25, 25,
     (0.05, 0.001)),
    ("forest fire, TMA-staged interior, torus", "fire", (1536, 520), dict(nb="vn", seed=14), 19, 19, (0.05, 0.002)),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_conformance(ca, oracle, case):
    name, kind, (n1, n2), kw, steps, saveat, params = case
    rule, space, scheme, P = spec_pair(ca, oracle, kind, n1, n2, **kw)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    C = 3 if kind == "fire" else P.states
    u0 = rng.integers(0, C, (n1, n2)).astype(np.int8)
    pd = None if params is None else {"p": params[0], "f": params[1]}
    prob = ca.CAProblem.new(rule, u0, steps, pd, space=space, seed=kw.get("seed", 0))
    sol = ca.solve(prob, scheme, backend=ca.GB300Backend(), saveat=saveat)
    ts, us = oracle.solve(P, u0, steps, saveat=saveat, params=params, nthreads=8)
    assert sol.t == ts
    for k, (a, b) in enumerate(zip(sol.u, us)):
        assert np.array_equal(a, b), f"{name}: save {k} (t = {ts[k]}) differs in {(a != b).sum()} cells"
    assert not np.array_equal(us[-1], u0)


LTL_WIDE = [
    # name, r, dims, boundaries, density, birth, survive, steps
    ("Moore(6) torus, one interval each", 6, (230, 170), ("p", "p"), 0.25, range(38, 51), range(36, 56), 24),
    ("Moore(7) grid, Constant(1) edges", 7, (300, 200), ("c", "c"), 0.2, range(40, 53), range(38, 59), 16),
    ("Moore(7) reflecting x torus, several intervals", 7, (250, 180), ("r", "p"), 0.2,
     [40, 41, 42, 43, 47, 48, 49, 50], [38, 39, 40, 41, 44, 45, 46, 47, 48, 49, 50, 51, 52, 53, 54, 55, 60], 16),
    ("Moore(6) lattice narrower than a halo word", 6, (40, 33), ("p", "p"), 0.25, range(38, 51), range(36, 56), 12),
]


@pytest.mark.parametrize("case", LTL_WIDE, ids=[c[0] for c in LTL_WIDE])
def test_larger_than_life_radius_6_7(ca, oracle, case):
    """Larger than Life on Moore(6) and Moore(7) (169 and 225 cells: eight count planes) runs
    the bit-sliced kernel, its one- and eight-interval forms, on every boundary kind: the
    state equals the oracle's after the first, middle and last steps and after whole queued
    passes, and the geometry query names a bit-sliced geometry. Sparse soups keep the first
    steps' counts near the intervals (the reference's count masks stop at 63, so a denser
    lattice dies at once): step 1 births most cells and step 2 kills most of them, counts
    spanning every interval and the gaps between them."""
    import ctypes
    name, r, (n1, n2), bnd, dens, birth, survive, steps = case
    const = (1, 1) if "Constant(1)" in name else (0, 0)
    rule, space, scheme, P = spec_pair(ca, oracle, "life", n1, n2, r=r, birth=birth, survive=survive, bnd=bnd,
                                       const=const)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    u0 = (rng.random((n1, n2)) < dens).astype(np.int8)
    prob = ca.CAProblem.new(rule, u0, 2 * steps, space=space)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, scheme)
    want = u0
    for t in range(steps):
        ca.advance(B, st, prob, scheme, None, t)
        want = oracle.run_array(P, want, t, 1, nthreads=8)
        if t == 0:
            assert (want != u0).sum() > 0.05 * want.size
        if t in (0, 1, steps // 2, steps - 1):
            got = ca.current_state(B, st)
            assert np.array_equal(got, want), f"{name}, step {t + 1}: {(got != want).sum()} cells differ"
    k, rows, staging = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    ca.capi.check(ca.capi.lib().gbca_geometry(st.handle, None, ctypes.byref(k), ctypes.byref(rows),
                                              ctypes.byref(staging)))
    assert k.value > 0, "Moore(r <= 7) Life fell back to the general kernel"
    for t in range(steps, 2 * steps):
        ca.advance(B, st, prob, scheme, None, t)
    want = oracle.run_array(P, want, steps, steps, nthreads=8)
    assert np.array_equal(ca.current_state(B, st), want)
    st.close()


def test_fire_states_outside_range(ca, oracle):
    """A forest-fire state written with values other than 0, 1, 2 (trees in the rule) takes
    exact byte compares on the first step and bit tests after it."""
    rng = np.random.default_rng(9)
    prob = ca.CAProblem.new(ca.ForestFire(), np.zeros((600, 300), np.int8), 20, {"p": 0.1, "f": 0.01},
                            space=ca.Grid(600, 300), seed=4)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    odd = rng.integers(-4, 8, (600, 300)).astype(np.int8)
    ca.set_state(B, st, odd)
    for t in range(20):
        ca.advance(B, st, prob, ca.Synchronous(), prob.p, t)
    got = ca.current_state(B, st)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, 600, 300, nbhd=oracle.VON_NEUMANN, seed=4,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT))
    assert np.array_equal(got, oracle.run_array(P, odd, 0, 20, (0.1, 0.01)))
    st.close()


@pytest.mark.parametrize("scheme", ["stoch", "check"])
def test_gated_fire_states_outside_range(ca, oracle, scheme):
    """A gated forest fire keeps closed cells' values, so a state written with values other than
    0, 1, 2 stays exact (byte compares) for as long as such values remain."""
    rng = np.random.default_rng(19)
    prob = ca.CAProblem.new(ca.ForestFire(), np.zeros((300, 280), np.int8), 12, {"p": 0.1, "f": 0.01},
                            space=ca.Grid(300, 280), seed=6)
    sch = ca.Stochastic(0.4) if scheme == "stoch" else ca.Checkerboard()
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, sch)
    odd = rng.integers(-4, 8, (300, 280)).astype(np.int8)
    ca.set_state(B, st, odd)
    for t in range(12):
        ca.advance(B, st, prob, sch, prob.p, t)
    got = ca.current_state(B, st)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, 300, 280, nbhd=oracle.VON_NEUMANN, seed=6,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT),
                       scheme=oracle.STOCHASTIC if scheme == "stoch" else oracle.CHECKERBOARD, scheme_p=0.4)
    assert np.array_equal(got, oracle.run_array(P, odd, 0, 12, (0.1, 0.01)))
    st.close()


def test_generations_states_outside_range(ca, oracle):
    """A state written with values outside 0..C-1 (here -3..6 for C = 3) evolves as the
    reference's rule says (s + 1 < C ? s + 1 : 0 for s not 0 or 1), through the general
    kernel, and the bit-sliced kernel takes over once every state is valid again."""
    rng = np.random.default_rng(8)
    u0 = rng.integers(0, 3, (64, 96)).astype(np.int8)
    prob = ca.CAProblem.new(ca.Generations(":brians_brain"), u0, 10)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    odd = rng.integers(-3, 7, (64, 96)).astype(np.int8)
    ca.set_state(B, st, odd)
    for t in range(12):
        ca.advance(B, st, prob, ca.Synchronous(), None, t)
    got = ca.current_state(B, st)
    P = oracle.Problem(oracle.RULE_GENERATIONS, 64, 96, birth=oracle.mask([2]), survive=0, states=3)
    assert np.array_equal(got, oracle.run_array(P, odd, 0, 12))
    st.close()


@pytest.mark.parametrize("scheme", ["stoch", "check"])
def test_gated_life_states_outside_range(ca, oracle, scheme):
    """Gated Life on a state holding values other than 0 and 1: a closed cell keeps its value
    (which the bit-sliced kernel's indicator bits cannot hold), so the sweep runs the general
    kernel until every state is 0 or 1; the result equals the oracle's throughout."""
    rng = np.random.default_rng(10)
    odd = rng.integers(-2, 4, (96, 64)).astype(np.int8)
    prob = ca.CAProblem.new(ca.Life(":conway"), np.zeros((96, 64), np.int8), 12, seed=31)
    sch = ca.Stochastic(0.5) if scheme == "stoch" else ca.Checkerboard()
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, sch)
    ca.set_state(B, st, odd)
    for t in range(12):
        ca.advance(B, st, prob, sch, None, t)
    got = ca.current_state(B, st)
    P = oracle.Problem(oracle.RULE_LIFE, 96, 64, birth=oracle.mask([3]), survive=oracle.mask([2, 3]), seed=31,
                       scheme=oracle.STOCHASTIC if scheme == "stoch" else oracle.CHECKERBOARD, scheme_p=0.5)
    assert np.array_equal(got, oracle.run_array(P, odd, 0, 12))
    st.close()


def test_highlife_128_config(ca, oracle):
    """Life(:highlife) on a 128x128 torus, Bernoulli(0.5) Int8 soup from seed 1, 200 steps, saveat=20:
    all 11 saved states equal the oracle's."""
    u0 = np.random.default_rng(1).integers(0, 2, (128, 128)).astype(np.int8)
    prob = ca.CAProblem.new(ca.Life(":highlife"), u0, 200)
    sol = ca.solve(prob, ca.Synchronous(), backend=ca.GB300Backend(), saveat=20)
    P = oracle.Problem(oracle.RULE_LIFE, 128, 128, birth=oracle.mask([3, 6]), survive=oracle.mask([2, 3]))
    ts, us = oracle.solve(P, u0, 200, saveat=20, nthreads=8)
    assert sol.t == ts == list(range(0, 201, 20))
    assert all(np.array_equal(a, b) for a, b in zip(sol.u, us))


def test_state_round_trip_and_cells(ca):
    u = np.random.default_rng(3).integers(-128, 128, (37, 45)).astype(np.int8)
    prob = ca.CAProblem.new(ca.ForestFire(), np.zeros((37, 45), np.int8), 5, {"p": 0.1, "f": 0.0})
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    ca.set_state(B, st, u)
    assert np.array_equal(ca.current_state(B, st), u)
    assert ca.read_cell(B, st, (5, 7)) == u[4, 6]
    ca.write_cell(B, st, (37, 45), -7)
    assert ca.read_cell(B, st, (37, 45)) == -7
    with pytest.raises(ca.ArgumentError):
        ca.read_cell(B, st, (38, 1))
    with pytest.raises(ca.StateShapeError):
        ca.set_state(B, st, np.zeros((3, 3), np.int8))
    st.close()


def test_integrator_modification_and_reinit(ca, oracle):
    """test/test_backend_interface.jl:86-97: a changed integ.u is applied before the next
    step; reinit! replays the run (draws are a pure function of seed, cell and time)."""
    u0 = np.random.default_rng(4).integers(0, 3, (50, 40)).astype(np.int8)
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 20, {"p": 0.2, "f": 0.01}, space=ca.Grid(50, 40), seed=9)
    integ = ca.init(prob, backend=ca.GB300Backend())
    ca.step(integ, 4)
    u = integ.u.copy()
    u[0, 0] = 2
    integ.u = u
    ca.step(integ)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, 50, 40, nbhd=oracle.VON_NEUMANN, seed=9,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT))
    ref = oracle.run_array(P, u0, 0, 4, (0.2, 0.01))
    ref[0, 0] = 2
    ref = oracle.run_array(P, ref, 4, 1, (0.2, 0.01))
    assert np.array_equal(integ.u, ref) and integ.t == 5
    # parameters changed by a callback apply from the next step on
    integ.p = {"p": 0.0, "f": 0.0}
    ca.step(integ, 3)
    assert np.array_equal(integ.u, oracle.run_array(P, ref, 5, 3, (0.0, 0.0)))
    integ.p = prob.p  # reinit! keeps the integrator's p (src/problem.jl:508-531)
    ca.reinit(integ)
    ca.step(integ, 6)
    assert np.array_equal(integ.u, oracle.run_array(P, u0, 0, 6, (0.2, 0.01)))


def test_device_summaries(ca, oracle):
    rng = np.random.default_rng(5)
    for bnd, ob in (((ca.Periodic(), ca.Periodic()), (oracle.PERIODIC, oracle.PERIODIC)),
                    ((ca.Constant(0), ca.Constant(0)), (oracle.CONSTANT, oracle.CONSTANT)),
                    ((ca.Reflecting(), ca.Constant(0)), (oracle.REFLECTING, oracle.CONSTANT))):
        u = rng.integers(0, 3, (300, 170)).astype(np.int8)
        prob = ca.CAProblem.new(ca.ForestFire(), u, 1, {"p": 0.0, "f": 0.0}, space=ca.Lattice((300, 170), bnd))
        B = ca.GB300Backend()
        st = ca.allocate_state(B, prob, ca.Synchronous())
        counts, other, mi = ca.device_summaries(st, 3)
        want_counts, want_other = oracle.state_counts(u, 3)
        want_mi = oracle.morans_i(oracle.Problem(oracle.RULE_LIFE, 300, 170, boundary=ob), u)
        assert counts == want_counts and other == want_other
        assert abs(mi - want_mi) <= 1e-12 * max(1.0, abs(want_mi)), (mi, want_mi)
        st.close()
    checker = np.array([[(i + j) % 2 for j in range(6)] for i in range(6)], np.int8)
    st = ca.allocate_state(ca.GB300Backend(), ca.CAProblem.new(ca.Life(), checker, 1), ca.Synchronous())
    assert abs(ca.device_summaries(st, 2)[2] + 1.0) < 1e-15  # test/test_extras.jl:140-141


GEN_WIDE = [
    # name, dims, kwargs, steps, saveat
    ("C=5 Moore(1) torus", (300, 200), dict(birth=[2], survive=[3, 4], states=5), 30, 10),
    ("C=6 Moore(2), Constant(4) and Constant(1) edges", (150, 170),
     dict(r=2, birth=[3, 4, 5], survive=[2, 3, 4, 5, 6], states=6, bnd=("c", "c"), const=(4, 1)), 20, 5),
    ("C=7 reflecting x torus, tiled", (400, 130), dict(birth=[2, 3], survive=[3, 4, 5], states=7, bnd=("r", "p")),
     25, 25),
    ("C=8 Moore(1) torus (a dying 7 wraps to 0)", (200, 96), dict(birth=[2], survive=[2, 3], states=8), 30, 6),
    ("C=5 von Neumann(1), reflecting", (150, 90), dict(nb="vn", birth=[1], survive=[1, 2], states=5,
                                                       bnd=("r", "r")), 30, 10),
    ("C=8 von Neumann(1) Checkerboard, Constant grid", (129, 77),
     dict(nb="vn", birth=[2], survive=[1, 2], states=8, scheme="check", bnd=("c", "c"), const=(0, 5)), 24, 6),
    ("C=6 Stochastic(0.6) Moore(2), cylinder", (160, 96),
     dict(r=2, birth=[3, 4, 5], survive=[2, 3, 4, 5, 6], states=6, seed=24, scheme="stoch", sp=0.6,
          bnd=("p", "c"), const=(0, 3)), 20, 4),
    ("C=7 Checkerboard Moore(1), odd torus", (51, 40), dict(birth=[2, 3], survive=[3, 4, 5], states=7, scheme="check"),
     20, 5),
]


@pytest.mark.parametrize("case", GEN_WIDE, ids=[c[0] for c in GEN_WIDE])
def test_generations_three_planes(ca, oracle, case):
    """Generations with 5..8 states (src/rules.jl:424-456) in the bit-sliced kernel's three-plane
    form, on every boundary kind and scheme: every save equals the oracle's, and the geometry
    query names a bit-sliced geometry (not the general kernel)."""
    import ctypes
    name, (n1, n2), kw, steps, saveat = case
    rule, space, scheme, P = spec_pair(ca, oracle, "gen", n1, n2, **kw)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    u0 = rng.integers(0, P.states, (n1, n2)).astype(np.int8)
    prob = ca.CAProblem.new(rule, u0, steps, space=space, seed=kw.get("seed", 0))
    sol = ca.solve(prob, scheme, backend=ca.GB300Backend(), saveat=saveat)
    ts, us = oracle.solve(P, u0, steps, saveat=saveat, nthreads=8)
    assert sol.t == ts
    for k, (a, b) in enumerate(zip(sol.u, us)):
        assert np.array_equal(a, b), f"{name}: save {k} (t = {ts[k]}) differs in {(a != b).sum()} cells"
    assert not np.array_equal(us[-1], u0) and (us[-1] >= 3).any()
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, scheme)
    ca.advance(B, st, prob, scheme, None, 0)
    ca.current_state(B, st)  # the state scan has run
    k, rows, staging = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    ca.capi.check(ca.capi.lib().gbca_geometry(st.handle, None, ctypes.byref(k), ctypes.byref(rows),
                                              ctypes.byref(staging)))
    assert k.value > 0, f"{name} fell back to the general kernel"
    st.close()


WIDENED = [
    # name, kind, dims, kwargs, steps, saveat — von Neumann(2..7) and gated / masked Moore(3..5), which
    # the bit-sliced kernel runs
    ("von Neumann(2) Life-like torus", "life", (300, 200), dict(nb="vn", r=2, birth=[3, 4], survive=[2, 3, 4]), 30,
     10),
    ("von Neumann(3) Life-like, Constant(1) grid", "life", (257, 190),
     dict(nb="vn", r=3, birth=[5, 6, 7, 8], survive=[4, 5, 6, 7, 8, 9], bnd=("c", "c"), const=(1, 1)), 24, 8),
    ("von Neumann(3), reflecting x odd torus", "life", (129, 77),
     dict(nb="vn", r=3, birth=[6, 7, 8, 12], survive=[5, 6, 7, 8, 9, 10], bnd=("r", "p")), 20, 5),
    ("von Neumann(2) Generations C=4, reflecting", "gen", (150, 90),
     dict(nb="vn", r=2, birth=[3, 4], survive=[2, 3, 4, 5], states=4, bnd=("r", "r")), 30, 10),
    ("von Neumann(3) Generations C=6, torus", "gen", (200, 96),
     dict(nb="vn", r=3, birth=[4, 5, 6], survive=[3, 4, 5, 6, 7], states=6), 30, 6),
    ("von Neumann(2) Stochastic(0.5), cylinder", "life", (200, 64),
     dict(nb="vn", r=2, birth=[3, 4], survive=[2, 3, 4], seed=41, scheme="stoch", sp=0.5, bnd=("p", "c")), 25, 5),
    ("von Neumann(3) Checkerboard, Constant grid", "life", (131, 97),
     dict(nb="vn", r=3, birth=[5, 6, 7, 8], survive=[4, 5, 6, 7, 8, 9], scheme="check", bnd=("c", "c")), 20, 5),
    ("von Neumann(4) Life-like, reflecting x periodic", "life", (260, 190),
     dict(nb="vn", r=4, birth=range(10, 14), survive=range(8, 22), bnd=("r", "p")), 20, 5),
    ("von Neumann(5) Life-like, Constant(1) grid", "life", (231, 170),
     dict(nb="vn", r=5, birth=range(20, 24), survive=range(18, 32), bnd=("c", "c"), const=(1, 1)), 16, 4),
    ("von Neumann(6) Life-like torus", "life", (300, 140),
     dict(nb="vn", r=6, birth=range(32, 38), survive=range(36, 50)), 16, 4),
    ("von Neumann(7) Life-like, periodic x Constant(0)", "life", (257, 200),
     dict(nb="vn", r=7, birth=range(20, 32), survive=range(40, 54), bnd=("p", "c")), 12, 4),
    ("von Neumann(4) Stochastic(0.6), torus", "life", (200, 130),
     dict(nb="vn", r=4, birth=range(10, 14), survive=range(8, 22), seed=46, scheme="stoch", sp=0.6), 16, 4),
    ("von Neumann(5) Checkerboard, reflecting", "life", (151, 121),
     dict(nb="vn", r=5, birth=range(20, 24), survive=range(18, 32), scheme="check", bnd=("r", "r")), 12, 4),
    ("Checkerboard Moore(3), odd torus", "life", (151, 103),
     dict(r=3, birth=range(9, 15), survive=range(8, 20), scheme="check"), 20, 5),
    ("Stochastic(0.4) Moore(4), reflecting", "life", (180, 150),
     dict(r=4, birth=range(14, 25), survive=range(12, 30), seed=44, scheme="stoch", sp=0.4, bnd=("r", "r")), 20, 4),
    ("Checkerboard Larger than Life Moore(5), Constant grid", "life", (230, 170),
     dict(r=5, birth=range(34, 46), survive=range(34, 59), scheme="check", bnd=("c", "c")), 16, 4),
    ("Stochastic(0.7f0) Moore(5), torus, several intervals", "life", (200, 180),
     dict(r=5, birth=[34, 35, 36, 40, 41, 42], survive=range(34, 59), seed=45, scheme="stoch", sp=0.7, sp32=True),
     16, 8),
]


@pytest.mark.parametrize("case", WIDENED, ids=[c[0] for c in WIDENED])
def test_widened_bit_sliced(ca, oracle, case):
    """von Neumann(2) .. (7) (13 .. 113 cells, src/neighbourhoods.jl:33-42,148-153; radii 4..7 by
    the running count) and the gated schemes on Moore(3..5) run the bit-sliced kernel: every
    save equals the oracle's, and the geometry query names a bit-sliced geometry."""
    import ctypes
    name, kind, (n1, n2), kw, steps, saveat = case
    rule, space, scheme, P = spec_pair(ca, oracle, kind, n1, n2, **kw)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    u0 = rng.integers(0, P.states, (n1, n2)).astype(np.int8)
    prob = ca.CAProblem.new(rule, u0, steps, space=space, seed=kw.get("seed", 0))
    sol = ca.solve(prob, scheme, backend=ca.GB300Backend(), saveat=saveat)
    ts, us = oracle.solve(P, u0, steps, saveat=saveat, nthreads=8)
    assert sol.t == ts
    for k, (a, b) in enumerate(zip(sol.u, us)):
        assert np.array_equal(a, b), f"{name}: save {k} (t = {ts[k]}) differs in {(a != b).sum()} cells"
    assert not np.array_equal(us[-1], u0) and 0 < (us[-1] == 1).sum() < us[-1].size
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, scheme)
    ca.advance(B, st, prob, scheme, None, 0)
    ca.current_state(B, st)
    k, rows, staging = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    ca.capi.check(ca.capi.lib().gbca_geometry(st.handle, None, ctypes.byref(k), ctypes.byref(rows),
                                              ctypes.byref(staging)))
    assert k.value > 0, f"{name} fell back to the general kernel"
    st.close()


@pytest.mark.parametrize("r,nb", [(3, "moore"), (5, "moore"), (5, "vn")])
def test_masked_moore_bit_sliced(ca, oracle, r, nb):
    """A masked Larger-than-Life sweep on Moore(3), Moore(5) and von Neumann(5) (the running
    count; src/environment.jl:123-130): masked cells keep their state though their neighbours read
    them; equal to the oracle step by step."""
    n1, n2 = 170, 130
    if nb == "vn":
        birth, survive = range(20, 24), range(18, 32)
    else:
        birth, survive = (range(9, 15), range(8, 20)) if r == 3 else (range(34, 46), range(34, 59))
    rule, space, scheme, P = spec_pair(ca, oracle, "life", n1, n2, nb=nb, r=r, birth=birth, survive=survive,
                                       bnd=("p", "r"))
    rng = np.random.default_rng(70 + r)
    u0 = rng.integers(0, 2, (n1, n2)).astype(np.int8)
    mask = np.ones((n1, n2), bool)
    mask[40:90, 20:70] = False
    mask[::7, :] = False
    prob = ca.CAProblem.new(rule, u0, 12, space=space, mask=mask)
    sol = ca.solve(prob, scheme, backend=ca.GB300Backend(), saveat=4)
    env = oracle.Env(mask=mask)
    want = u0
    for k, t in enumerate(range(0, 12, 4)):
        want = oracle.run_array_env(P, env, want, t, 4, nthreads=8)
        assert np.array_equal(sol.u[k + 1], want), f"{nb}({r}) masked, t = {t + 4}"
    assert np.array_equal(sol.u[-1][~mask], u0[~mask]) and not np.array_equal(sol.u[-1], u0)


def _tie_cells(oracle, seed, n1, n2, u0, t):
    """Forest-fire parameters on the edge of chosen cells' draws (random.jl:116-120,129): p one
    unit (2^-53) above an empty cell's 53-bit draw (a hit), f equal to a tree's (no hit), so each
    draw agrees with its threshold in the first 32 bits and differs only in the last 21."""
    def x53(i, j, k):
        r = oracle.philox4x32(((i + j * n1 + 1) & 0xFFFFFFFF, 0, t, k), (seed & 0xFFFFFFFF, seed >> 32))
        return ((r[0] << 32) | r[1]) >> 11

    empties = [(i, j) for i, j in zip(*np.nonzero(u0 == 0))]
    trees = [(i, j) for i, j in zip(*np.nonzero(u0 == 1))]
    xe = next(x for x in (x53(i, j, 1) for i, j in empties[len(empties) // 3:]) if (x + 1) >> 21 == x >> 21)
    xt = x53(*trees[len(trees) // 2], 2)
    return (xe + 1) / 2.0**53, xt / 2.0**53


def test_fire_threshold_ties(ca, oracle):
    """Draws on the edge of their thresholds (see _tie_cells): every cell of the single-lattice
    sweep (one and several tiles) and of the batched engine (persistent and multi-lattice passes)
    equals the oracle, step by step."""
    n1, n2, seed = 600, 300, 11
    rng = np.random.default_rng(5)
    u0 = (rng.random((n1, n2)) < 0.5).astype(np.int8)  # empty and trees, no fire: every cell draws
    p, f = _tie_cells(oracle, seed, n1, n2, u0, 0)
    assert 0 < p < 1 and 0 < f < 1
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, n1, n2, nbhd=oracle.VON_NEUMANN, seed=seed,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT))
    want = oracle.run_array(P, u0, 0, 1, (p, f))
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 4, {"p": p, "f": f}, space=ca.Grid(n1, n2), seed=seed)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    ca.advance(B, st, prob, ca.Synchronous(), prob.p, 0)
    assert np.array_equal(ca.current_state(B, st), want)
    for t in range(1, 4):
        ca.advance(B, st, prob, ca.Synchronous(), prob.p, t)
    assert np.array_equal(ca.current_state(B, st), oracle.run_array(P, want, 1, 3, (p, f)))
    st.close()
    # the batched engine: the same lattice as a large instance (multi-lattice passes) and as a
    # small one (the persistent kernel), beside a second instance
    small = u0[:90, :70].copy()
    ps, fs = _tie_cells(oracle, seed + 1, 90, 70, small, 0)
    Ps = oracle.Problem(oracle.RULE_FOREST_FIRE, 90, 70, nbhd=oracle.VON_NEUMANN, seed=seed + 1,
                        boundary=(oracle.CONSTANT, oracle.CONSTANT))
    probs = [prob, ca.CAProblem.new(ca.ForestFire(), small, 4, {"p": ps, "f": fs}, space=ca.Grid(90, 70),
                                    seed=seed + 1)]
    for min_cells in (1 << 14, 1 << 30):
        ens = ca.BatchedEnsemble(probs)
        ens.set_large(min_cells, 1)
        ens.set_initial_states()
        ens.run(t0=[0, 0], nsteps=[1, 1])
        assert np.array_equal(ens.state(0), want)
        assert np.array_equal(ens.state(1), oracle.run_array(Ps, small, 0, 1, (ps, fs)))
        ens.close()


def test_fire_threshold_ties_float32(ca, oracle):
    """Float32 parameters: p equal to a draw's 24-bit value (r1 >> 8) * 2^-24 (random.jl:109-114,
    130), for a draw whose word 1 has a zero low byte: no hit, as the reference's compare gives."""
    n1, n2, seed = 300, 200, 21
    u0 = np.zeros((n1, n2), np.int8)
    cand = [q for q in range(n1 * n2) if oracle.philox4x32((q + 1, 0, 0, 1), (seed, 0))[0] & 0xFF == 0]
    assert cand
    r1 = oracle.philox4x32((cand[0] + 1, 0, 0, 1), (seed, 0))[0]
    p = np.float32((r1 >> 8) / 2.0**24)
    assert float(p) * 2**24 == r1 >> 8
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, n1, n2, nbhd=oracle.VON_NEUMANN, seed=seed,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT), params_f32=True)
    want = oracle.run_array(P, u0, 0, 2, (float(p), 1e-3))
    prob = ca.CAProblem.new(ca.ForestFire(float32=True), u0, 2, {"p": float(p), "f": 1e-3}, space=ca.Grid(n1, n2),
                            seed=seed)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    for t in range(2):
        ca.advance(B, st, prob, ca.Synchronous(), prob.p, t)
    assert np.array_equal(ca.current_state(B, st), want)
    st.close()
