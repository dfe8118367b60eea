"""The sweep autotuner and pinned geometries: every geometry a fast kernel accepts (steps per
temporally blocked pass x tile height) gives the oracle's states bit for bit, tuning leaves
the state as it found it, and a tuned shape keeps its results."""
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


def _run(ca, prob, st, t0, n, p=None):
    B = ca.GB300Backend()
    for t in range(t0, t0 + n):
        ca.advance(B, st, prob, ca.Synchronous(), p, t)
    return ca.current_state(B, st)


LTL = dict(birth=list(range(34, 46)), survive=list(range(34, 59)))


@pytest.mark.parametrize("steps,rows", [(1, 64), (2, 96), (3, 144), (5, 256), (6, 176), (4, 0)])
def test_ltl_geometries(ca, oracle, steps, rows):
    """Larger than Life Moore(5) on a 333 x 301 torus, 23 steps (no geometry divides it)."""
    u0 = np.random.default_rng(steps * 100 + rows).integers(0, 2, (333, 301)).astype(np.int8)
    prob = ca.CAProblem.new(ca.Life(LTL["birth"], LTL["survive"], neighbourhood=ca.Moore(5)), u0, 23)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ca.set_geometry(st, steps, rows)
    got = _run(ca, prob, st, 0, 23)
    P = oracle.Problem(oracle.RULE_LIFE, 333, 301, radius=5, birth=oracle.mask(LTL["birth"]),
                       survive=oracle.mask(LTL["survive"]))
    assert np.array_equal(got, oracle.run_array(P, u0, 0, 23, nthreads=8))
    st.close()


@pytest.mark.parametrize("steps,rows", [(32, 64), (24, 216), (8, 128), (12, 96)])
def test_life_constant_edges_geometries(ca, oracle, steps, rows):
    """HighLife on a 250 x 520 grid with Constant(1) on one axis, 50 steps."""
    u0 = np.random.default_rng(steps + rows).integers(0, 2, (250, 520)).astype(np.int8)
    space = ca.Lattice((250, 520), (ca.Periodic(), ca.Constant(1)))
    prob = ca.CAProblem.new(ca.Life(":highlife"), u0, 50, space=space)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ca.set_geometry(st, steps, rows)
    got = _run(ca, prob, st, 0, 50)
    P = oracle.Problem(oracle.RULE_LIFE, 250, 520, birth=oracle.mask([3, 6]), survive=oracle.mask([2, 3]),
                       boundary=(oracle.PERIODIC, oracle.CONSTANT), constant=(0, 1))
    assert np.array_equal(got, oracle.run_array(P, u0, 0, 50, nthreads=8))
    st.close()


@pytest.mark.parametrize("steps,rows", [(4, 64), (16, 128), (6, 256)])
def test_generations_geometries(ca, oracle, steps, rows):
    """Star Wars (C = 4) on a 200 x 330 reflecting lattice, 30 steps."""
    u0 = np.random.default_rng(rows).integers(0, 4, (200, 330)).astype(np.int8)
    space = ca.Lattice((200, 330), (ca.Reflecting(), ca.Reflecting()))
    prob = ca.CAProblem.new(ca.Generations("B2/S345/C4"), u0, 30, space=space)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ca.set_geometry(st, steps, rows)
    got = _run(ca, prob, st, 0, 30)
    P = oracle.Problem(oracle.RULE_GENERATIONS, 200, 330, birth=oracle.mask([2]), survive=oracle.mask([3, 4, 5]),
                       states=4, boundary=(oracle.REFLECTING, oracle.REFLECTING))
    assert np.array_equal(got, oracle.run_array(P, u0, 0, 30, nthreads=8))
    st.close()


@pytest.mark.parametrize("steps,staging,n1", [(1, 0, 900), (2, 1, 900), (5, 0, 1024), (12, 1, 1024), (16, 1, 912),
                                               (1, 2, 900), (1, 2, 1024), (1, 1, 912)])
def test_fire_geometries(ca, oracle, steps, staging, n1):
    """Forest fire on an n1 x 410 grid from t = 3, 29 steps; staging 1 stages tiles by TMA
    (interior tiles for n1 = 900, every tile for the multiples of 16)."""
    u0 = np.random.default_rng(steps).integers(0, 3, (n1, 410)).astype(np.int8)
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 40, {"p": 0.05, "f": 0.002}, space=ca.Grid(n1, 410), seed=7)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ca.set_geometry(st, steps, 0, staging)
    got = _run(ca, prob, st, 3, 29, prob.p)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, n1, 410, nbhd=oracle.VON_NEUMANN, seed=7,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT))
    assert np.array_equal(got, oracle.run_array(P, u0, 3, 29, (0.05, 0.002), nthreads=8))
    st.close()


def test_tune_keeps_state_and_results(ca, oracle):
    """gbca_tune on a 1536 x 1280 Life torus: the state is unchanged, the choice is a
    candidate, and the tuned sweep still matches the oracle."""
    u0 = np.random.default_rng(11).integers(0, 2, (1536, 1280)).astype(np.int8)
    prob = ca.CAProblem.new(ca.Life(":conway"), u0, 40)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    k, rows, staging = ca.tune(st, prob)
    assert k in (8, 12, 16, 24, 32) and rows in (64, 96, 128, 144, 176, 216, 256) and staging == 0
    assert np.array_equal(ca.current_state(B, st), u0)
    got = _run(ca, prob, st, 0, 40)
    P = oracle.Problem(oracle.RULE_LIFE, 1536, 1280, birth=oracle.mask([3]), survive=oracle.mask([2, 3]))
    assert np.array_equal(got, oracle.run_array(P, u0, 0, 40, nthreads=16))
    st.close()
    # a second handle of the same shape uses the cached choice
    st2 = ca.allocate_state(B, prob, ca.Synchronous())
    assert np.array_equal(_run(ca, prob, st2, 0, 40), got)
    st2.close()
    ca.capi.check(ca.capi.lib().gbca_forget_tuning())


def test_tune_fire_and_general(ca, oracle):
    u0 = np.random.default_rng(12).integers(0, 3, (1000, 600)).astype(np.int8)
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 20, {"p": 0.05, "f": 0.002}, space=ca.Grid(1000, 600), seed=3)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    k, rows, staging = ca.tune(st, prob)
    assert k in (1, 2, 3, 4, 6, 8) and rows == 0 and staging in (0, 1, 2)
    assert np.array_equal(ca.current_state(B, st), u0)
    got = _run(ca, prob, st, 0, 20, prob.p)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, 1000, 600, nbhd=oracle.VON_NEUMANN, seed=3,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT))
    assert np.array_equal(got, oracle.run_array(P, u0, 0, 20, (0.05, 0.002), nthreads=16))
    st.close()
    # Generations with 10 states runs on the general kernel: nothing to tune, no geometry to pin
    prob2 = ca.CAProblem.new(ca.Generations("B2/S/C10"), np.zeros((64, 64), np.int8), 5)
    st2 = ca.allocate_state(B, prob2, ca.Synchronous())
    assert ca.tune(st2, prob2) == (0, 0, 0)
    with pytest.raises(ca.UnsupportedCombinationError):
        ca.set_geometry(st2, 4, 0)
    st2.close()
    ca.capi.check(ca.capi.lib().gbca_forget_tuning())


def test_geometry_refusals(ca):
    B = ca.GB300Backend()
    fire = ca.CAProblem.new(ca.ForestFire(), np.zeros((64, 64), np.int8), 5, {"p": 0.1, "f": 0.0})
    st = ca.allocate_state(B, fire, ca.Synchronous())
    with pytest.raises(ca.ArgumentError):
        ca.set_geometry(st, 4, 300)  # fire tiles take 8..240 rows
    with pytest.raises(ca.ArgumentError):
        ca.set_geometry(st, 64, 240)  # beyond shared memory at 64 steps per pass
    with pytest.raises(ca.ArgumentError):
        ca.set_geometry(st, 0, 16)
    with pytest.raises(ca.ArgumentError):
        ca.set_geometry(st, 65, 0)
    with pytest.raises(ca.ArgumentError):
        ca.set_geometry(st, 4, 0, 3)  # staging is 0, 1 or 2
    st.close()
    ltl = ca.CAProblem.new(ca.Life(LTL["birth"], LTL["survive"], neighbourhood=ca.Moore(5)),
                           np.zeros((4096, 4096), np.int8), 5)
    st = ca.allocate_state(B, ltl, ca.Synchronous())
    with pytest.raises(ca.ArgumentError):
        ca.set_geometry(st, 6, 4000)  # far beyond shared memory
    ca.set_geometry(st, 0, 0)
    st.close()


@pytest.mark.parametrize("space", ["grid", "torus"])
def test_fire_persistent_multi_tile(ca, oracle, space):
    """The persistent prefetching kernel (staging 2) with more tiles than CTAs, so each CTA
    runs several tiles through both of its shared buffers: a 4096 x 4096 lattice (512 tiles),
    on a Constant(0) grid (every tile a TMA copy) and on a torus (edge tiles through the
    boundary map), 6 steps."""
    n = 4096
    u0 = np.random.default_rng(99).integers(0, 3, (n, n)).astype(np.int8)
    sp = ca.Grid(n, n) if space == "grid" else ca.Torus(n, n)
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 6, {"p": 0.05, "f": 0.002}, space=sp, seed=21)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ca.set_geometry(st, 1, 0, 2)
    got = _run(ca, prob, st, 0, 6, prob.p)
    bnd = (oracle.CONSTANT, oracle.CONSTANT) if space == "grid" else (oracle.PERIODIC, oracle.PERIODIC)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, n, n, nbhd=oracle.VON_NEUMANN, seed=21, boundary=bnd)
    assert np.array_equal(got, oracle.run_array(P, u0, 0, 6, (0.05, 0.002), nthreads=16))
    st.close()


@pytest.mark.parametrize("steps,rows,staging", [(1, 108, 1), (1, 72, 2), (1, 37, 0), (3, 200, 1), (8, 8, 0)])
def test_fire_pinned_tile_rows(ca, oracle, steps, rows, staging):
    """Pinned forest-fire tile heights that divide nothing (a 1000 x 770 grid: ragged tiles on
    both axes), each staging method, one and several steps per pass, from t = 2, 11 steps."""
    n1, n2 = 1000, 770
    u0 = np.random.default_rng(rows).integers(0, 3, (n1, n2)).astype(np.int8)
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 20, {"p": 0.05, "f": 0.002}, space=ca.Grid(n1, n2), seed=19)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ca.set_geometry(st, steps, rows, staging)
    got = _run(ca, prob, st, 2, 11, prob.p)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, n1, n2, nbhd=oracle.VON_NEUMANN, seed=19,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT))
    assert np.array_equal(got, oracle.run_array(P, u0, 2, 11, (0.05, 0.002), nthreads=16))
    st.close()


@pytest.mark.parametrize("side", [2048, 4096])
def test_fire_one_step_model_heights(ca, oracle, side):
    """The one-step model's tile heights (108 rows on 2048^2 and 4096^2 grids, whose tiles
    then spread evenly over the SMs), 3 steps from an oracle-checked state."""
    u0 = np.random.default_rng(side).integers(0, 3, (side, side)).astype(np.int8)
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 3, {"p": 0.05, "f": 0.002}, space=ca.Grid(side, side), seed=23)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ca.set_geometry(st, 1, 0, 1)
    got = _run(ca, prob, st, 0, 3, prob.p)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, side, side, nbhd=oracle.VON_NEUMANN, seed=23,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT))
    assert np.array_equal(got, oracle.run_array(P, u0, 0, 3, (0.05, 0.002), nthreads=16))
    st.close()


@pytest.mark.parametrize("n1,n2,space,staging", [(4000, 2999, "grid", 1), (4000, 2999, "grid", 2),
                                                 (2050, 2100, "torus", 1), (2050, 2100, "grid", 0)])
def test_fire_one_step_model_ragged(ca, oracle, n1, n2, space, staging):
    """The one-step model's heights on ragged lattices (158 rows on 4000 x 2999, a last tile
    of 155 rows and a last tile column of 160 cells; 132 rows on 2050 x 2100, two cells in the
    last tile column), TMA, persistent and vector-load staging, on a grid and a torus (edge
    tiles through the boundary map): 3 steps from t = 5 against the oracle."""
    u0 = np.random.default_rng(n1 + staging).integers(0, 3, (n1, n2)).astype(np.int8)
    sp = ca.Grid(n1, n2) if space == "grid" else ca.Torus(n1, n2)
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 8, {"p": 0.05, "f": 0.002}, space=sp, seed=29)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ca.set_geometry(st, 1, 0, staging)
    got = _run(ca, prob, st, 5, 3, prob.p)
    bnd = (oracle.CONSTANT, oracle.CONSTANT) if space == "grid" else (oracle.PERIODIC, oracle.PERIODIC)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, n1, n2, nbhd=oracle.VON_NEUMANN, seed=29, boundary=bnd)
    assert np.array_equal(got, oracle.run_array(P, u0, 5, 3, (0.05, 0.002), nthreads=16))
    st.close()


@pytest.mark.parametrize("staging", [0, 1, 2])
def test_fire_full_height_tiles(ca, oracle, staging):
    """A lattice with enough 256 x 128 tiles to fill every CTA slot twice keeps full-height
    tiles (smaller lattices take 64- or 32-row tiles): 4096 x 5120 (640 tiles), 3 steps of
    each staging method, against the oracle."""
    n1, n2 = 4096, 5120
    u0 = np.random.default_rng(31 + staging).integers(0, 3, (n1, n2)).astype(np.int8)
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 3, {"p": 0.05, "f": 0.002}, space=ca.Grid(n1, n2), seed=17)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ca.set_geometry(st, 1, 0, staging)
    got = _run(ca, prob, st, 0, 3, prob.p)
    P = oracle.Problem(oracle.RULE_FOREST_FIRE, n1, n2, nbhd=oracle.VON_NEUMANN, seed=17,
                       boundary=(oracle.CONSTANT, oracle.CONSTANT))
    assert np.array_equal(got, oracle.run_array(P, u0, 0, 3, (0.05, 0.002), nthreads=16))
    st.close()
