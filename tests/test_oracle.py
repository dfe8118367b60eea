"""Pins the CPU oracle to the reference's own known answers before anything is checked
against it: Philox vectors, rule definitions, classic patterns, scheme properties,
Moran's I and Lenia direct-vs-FFT. ReferenceBackend-style and ArrayBackend-style
(threaded, halo-padded) oracle runs must agree exactly, as the reference's conformance
battery demands of every backend (test/backend_conformance.jl:264-287)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_philox_known_answers(oracle):
    """test/test_random.jl:4-14 (vectors extracted into tests/golden/philox_kat.json)."""
    with open(os.path.join(GOLDEN, "philox_kat.json")) as f:
        kats = json.load(f)["vectors"]
    assert len(kats) == 3
    for v in kats:
        assert oracle.philox4x32(v["ctr"], v["key"]) == tuple(v["out"])


def test_uniform_pure_and_in_range(oracle):
    """test/test_random.jl:18-56."""
    u = oracle.uniform
    assert u(1, 7, 3, 1) == u(1, 7, 3, 1)
    assert u(1, 7, 3, 1) != u(1, 8, 3, 1)
    assert u(1, 7, 3, 1) != u(1, 7, 4, 1)
    assert u(1, 7, 3, 1) != u(2, 7, 3, 1)
    assert u(1, 7, 3, 1) != u(1, 7, 3, 2)
    xs = np.array([u(2026, i, 0, k) for i in range(1, 2001) for k in range(1, 5)])
    assert np.all((xs >= 0) & (xs < 1))
    assert abs(xs.mean() - 0.5) < 0.01
    assert abs((xs < 0.25).mean() - 0.25) < 0.02
    ys = np.array([oracle.uniform32(2026, i, 0, 1) for i in range(1, 5001)])
    assert np.all((ys >= 0) & (ys < 1)) and abs(ys.mean() - 0.5) < 0.015
    # the FP64 draw is built from words 1 and 2 of the Philox output, the FP32 draw from word 1
    r = oracle.philox4x32((7, 0, 3, 2), (1, 0))
    assert u(1, 7, 3, 2) == (((r[0] << 32) | r[1]) >> 11) * 2.0 ** -53
    assert oracle.uniform32(1, 7, 3, 2) == np.float32(r[0] >> 8) * np.float32(2.0 ** -24)


def naive_generations(birth, survive, C, u):
    """test/test_rules.jl:23-32, restated: Moore(1) on a torus; C = 2 is Life."""
    m, n = u.shape
    out = np.zeros_like(u)
    for i in range(m):
        for j in range(n):
            live = sum(u[(i + a) % m, (j + b) % n] == 1
                       for a in (-1, 0, 1) for b in (-1, 0, 1) if (a, b) != (0, 0))
            s = u[i, j]
            if s == 0:
                out[i, j] = 1 if live in birth else 0
            elif s == 1:
                out[i, j] = 1 if live in survive else (2 if C > 2 else 0)
            else:
                out[i, j] = s + 1 if s + 1 < C else 0
    return out


@pytest.mark.parametrize("b,s,C", [([3], [2, 3], 2), ([3, 6], [2, 3], 2), ([2], [], 2),
                                   ([2], [], 3), ([2], [3, 4, 5], 4)])
def test_life_generations_against_definition(oracle, b, s, C):
    rng = np.random.default_rng(C * 10 + len(b))
    for _ in range(3):
        u = rng.integers(0, C, size=(12, 15)).astype(np.int8)
        rule = oracle.RULE_LIFE if C == 2 else oracle.RULE_GENERATIONS
        P = oracle.Problem(rule, 12, 15, birth=oracle.mask(b), survive=oracle.mask(s), states=C)
        assert np.array_equal(oracle.step_reference(P, u, 0), naive_generations(b, s, C, u))
        assert np.array_equal(oracle.run_array(P, u, 0, 1, nthreads=3), naive_generations(b, s, C, u))


def _axis_images(oracle, kind, n, r):
    """0-based images of cells -r .. n+r-1 along one axis (src/spaces.jl:46-51): Periodic
    wraps, Reflecting mirrors with the edge cell repeated (period 2n), -1 beyond Constant."""
    j = np.arange(-r, n + r)
    if kind == oracle.PERIODIC:
        return j % n
    if kind == oracle.REFLECTING:
        m = j % (2 * n)
        return np.where(m < n, m, 2 * n - 1 - m)
    return np.where((j >= 0) & (j < n), j, -1)


def naive_life(oracle, u, r, nbhd, birth, survive, bnd, const):
    """Life / Larger than Life by definition (src/rules.jl:377-389): n counts the neighbours
    equal to 1 over Moore(r) or von Neumann(r) (centre excluded), read through the boundary
    images (beyond two Constant edges the second axis's value wins, src/backends.jl:177-184);
    the next state is bit n of the survival mask for a cell equal to 1, of the birth mask
    otherwise, and 0 when n >= 64 (UInt64 masks)."""
    n1, n2 = u.shape
    ix, iy = _axis_images(oracle, bnd[0], n1, r), _axis_images(oracle, bnd[1], n2, r)
    pad = u[np.clip(ix, 0, None)][:, np.clip(iy, 0, None)].astype(np.int64)
    if bnd[0] == oracle.CONSTANT:
        pad[ix < 0, :] = const[0]
    if bnd[1] == oracle.CONSTANT:
        pad[:, iy < 0] = const[1]
    alive = (pad == 1).astype(np.int64)
    n = np.zeros((n1, n2), np.int64)
    for a in range(-r, r + 1):
        for b in range(-r, r + 1):
            if (a, b) == (0, 0) or (nbhd == oracle.VON_NEUMANN and abs(a) + abs(b) > r):
                continue
            n += alive[r + a:r + a + n1, r + b:r + b + n2]
    masks = np.where(u == 1, np.uint64(survive), np.uint64(birth)).astype(np.uint64)
    bit = (masks >> np.minimum(n, 63).astype(np.uint64)) & np.uint64(1)
    return np.where(n < 64, bit, 0).astype(np.int8)


@pytest.mark.parametrize("nb,r,dims,bnd,const", [
    ("moore", 2, (20, 17), "pp", (0, 0)), ("moore", 5, (30, 24), "cc", (1, 0)), ("moore", 6, (5, 9), "pr", (0, 0)),
    ("moore", 7, (33, 40), "rc", (0, 1)), ("moore", 7, (16, 16), "cp", (1, 0)), ("vn", 1, (11, 13), "rr", (0, 0)),
    ("vn", 3, (14, 9), "cp", (1, 0)), ("vn", 7, (6, 20), "pc", (0, 1))])
def test_larger_than_life_against_definition(oracle, nb, r, dims, bnd, const):
    """The oracle's Life on Moore(r) and von Neumann(r) up to r = 7 against a numpy
    restatement of the definition, on every boundary kind (lattices smaller than the radius
    included), random 64-bit count masks and states holding values other than 0 and 1."""
    kinds = {"p": oracle.PERIODIC, "r": oracle.REFLECTING, "c": oracle.CONSTANT}
    bounds = (kinds[bnd[0]], kinds[bnd[1]])
    nbhd = oracle.MOORE if nb == "moore" else oracle.VON_NEUMANN
    rng = np.random.default_rng(1000 * r + dims[0])
    n1, n2 = dims
    for trial in range(3):
        birth = int(rng.integers(0, 2 ** 63)) | (int(rng.integers(0, 2)) << 63)
        survive = int(rng.integers(0, 2 ** 63))
        u = (rng.random((n1, n2)) < (0.15, 0.35, 0.6)[trial]).astype(np.int8)
        u[rng.random((n1, n2)) < 0.05] = 2
        u[rng.random((n1, n2)) < 0.02] = -1
        P = oracle.Problem(oracle.RULE_LIFE, n1, n2, nbhd=nbhd, radius=r, birth=birth, survive=survive,
                           boundary=bounds, constant=const)
        want = naive_life(oracle, u, r, nbhd, birth, survive, bounds, const)
        assert np.array_equal(oracle.step_reference(P, u, 0), want)
        assert np.array_equal(oracle.run_array(P, u, 0, 1, nthreads=3), want)


@pytest.mark.parametrize("nb,r,C,bnd,const", [("moore", 2, 3, "rc", (0, 2)), ("moore", 2, 4, "cc", (1, 3)),
                                              ("vn", 1, 4, "pr", (0, 0)), ("moore", 1, 3, "cp", (2, 0))])
def test_generations_radius_and_edges_against_definition(oracle, nb, r, C, bnd, const):
    """Generations (src/rules.jl:446-456) on Moore(2) and von Neumann(1) with Reflecting and
    Constant edges, by definition: the count of neighbours equal to 1 (naive_life's count),
    0 -> 1 on a birth count, 1 -> 1 on a survival count else 2 (or 0 when C = 2), s >= 2 ->
    s + 1 below C, else 0."""
    kinds = {"p": oracle.PERIODIC, "r": oracle.REFLECTING, "c": oracle.CONSTANT}
    bounds = (kinds[bnd[0]], kinds[bnd[1]])
    nbhd = oracle.MOORE if nb == "moore" else oracle.VON_NEUMANN
    rng = np.random.default_rng(100 * r + C)
    n1, n2 = 17, 12
    birth, survive = oracle.mask([2, 3, 7]), oracle.mask([1, 3, 4, 5, 9])
    for _ in range(3):
        u = rng.integers(0, C, (n1, n2)).astype(np.int8)
        # n: the neighbours equal to 1, read through the boundary images
        ix, iy = _axis_images(oracle, bounds[0], n1, r), _axis_images(oracle, bounds[1], n2, r)
        pad = u[np.clip(ix, 0, None)][:, np.clip(iy, 0, None)].astype(np.int64)
        if bounds[0] == oracle.CONSTANT:
            pad[ix < 0, :] = const[0]
        if bounds[1] == oracle.CONSTANT:
            pad[:, iy < 0] = const[1]
        n = np.zeros((n1, n2), np.int64)
        for a in range(-r, r + 1):
            for b in range(-r, r + 1):
                if (a, b) != (0, 0) and (nbhd == oracle.MOORE or abs(a) + abs(b) <= r):
                    n += pad[r + a:r + a + n1, r + b:r + b + n2] == 1
        bit = lambda m: ((np.uint64(m) >> n.astype(np.uint64)) & np.uint64(1)).astype(bool)
        want = np.where(u == 0, bit(birth).astype(np.int8),
                        np.where(u == 1, np.where(bit(survive), 1, 2 if C > 2 else 0),
                                 np.where(u + 1 < C, u + 1, 0))).astype(np.int8)
        P = oracle.Problem(oracle.RULE_GENERATIONS, n1, n2, nbhd=nbhd, radius=r, birth=birth, survive=survive,
                           states=C, boundary=bounds, constant=const)
        assert np.array_equal(oracle.step_reference(P, u, 0), want)
        assert np.array_equal(oracle.run_array(P, u, 0, 1, nthreads=2), want)


def _neighbour_images(oracle, u, nbhd, bnd, const):
    """The radius-1 neighbour values of every cell, read through the boundary images (as
    naive_life does), as a list of arrays in the neighbourhood's offset order."""
    n1, n2 = u.shape
    ix, iy = _axis_images(oracle, bnd[0], n1, 1), _axis_images(oracle, bnd[1], n2, 1)
    pad = u[np.clip(ix, 0, None)][:, np.clip(iy, 0, None)].astype(np.int64)
    if bnd[0] == oracle.CONSTANT:
        pad[ix < 0, :] = const[0]
    if bnd[1] == oracle.CONSTANT:
        pad[:, iy < 0] = const[1]
    offs = [(a, b) for b in (-1, 0, 1) for a in (-1, 0, 1) if (a, b) != (0, 0)
            and (nbhd == oracle.MOORE or abs(a) + abs(b) == 1)]
    return [pad[1 + a:1 + a + n1, 1 + b:1 + b + n2] for a, b in offs]


@pytest.mark.parametrize("nb,bnd,const,dims", [("vn", "cc", (0, 0), (12, 9)), ("vn", "pp", (0, 0), (10, 11)),
                                               ("moore", "rc", (0, 2), (9, 13)), ("vn", "cp", (2, 0), (7, 8))])
def test_forest_fire_against_definition(oracle, nb, bnd, const, dims):
    """One forest-fire step by definition (the package README's rule on Int8 codes), with
    draws from the oracle's Philox uniform (pinned by the known answers above) keyed by the
    1-based column-major cell id (i - 1) + (j - 1) n1 + 1, the time of the state read, and
    draw index 1 (empty -> tree) or 2 (lightning): 2 -> 0; 0 -> 1 iff u < p; any other state
    -> 2 next to a fire, else 2 iff u < f, else 1."""
    kinds = {"p": oracle.PERIODIC, "r": oracle.REFLECTING, "c": oracle.CONSTANT}
    bounds = (kinds[bnd[0]], kinds[bnd[1]])
    nbhd = oracle.MOORE if nb == "moore" else oracle.VON_NEUMANN
    n1, n2 = dims
    rng = np.random.default_rng(n1 * n2)
    p, f, seed = 0.4, 0.2, 17
    for t in (0, 5):
        u = rng.integers(0, 3, (n1, n2)).astype(np.int8)
        u[rng.random((n1, n2)) < 0.05] = 4
        fire_near = np.zeros((n1, n2), bool)
        for v in _neighbour_images(oracle, u, nbhd, bounds, const):
            fire_near |= v == 2
        want = np.zeros((n1, n2), np.int8)
        for i in range(n1):
            for j in range(n2):
                cid = i + j * n1 + 1
                c = u[i, j]
                if c == 2:
                    want[i, j] = 0
                elif c == 0:
                    want[i, j] = 1 if oracle.uniform(seed, cid, t, 1) < p else 0
                elif fire_near[i, j]:
                    want[i, j] = 2
                else:
                    want[i, j] = 2 if oracle.uniform(seed, cid, t, 2) < f else 1
        P = oracle.Problem(oracle.RULE_FOREST_FIRE, n1, n2, nbhd=nbhd, seed=seed, boundary=bounds, constant=const)
        assert np.array_equal(oracle.step_reference(P, u, t, (p, f)), want)
        assert np.array_equal(oracle.run_array(P, u, t, 1, (p, f), nthreads=2), want)


def test_stochastic_gate_against_definition(oracle):
    """Stochastic(p) (src/schemes.jl:84-89): a cell updates iff draw 0 of its id at the step's
    time falls below p, else keeps its state; the update is the synchronous rule's."""
    n1, n2, seed, p = 14, 11, 23, 0.45
    rng = np.random.default_rng(5)
    B3S23 = dict(birth=oracle.mask([3]), survive=oracle.mask([2, 3]))
    for t in (0, 3):
        u = (rng.random((n1, n2)) < 0.4).astype(np.int8)
        sync = naive_life(oracle, u, 1, oracle.MOORE, B3S23["birth"], B3S23["survive"],
                          (oracle.PERIODIC, oracle.PERIODIC), (0, 0))
        open_ = np.array([[oracle.uniform(seed, i + j * n1 + 1, t, 0) < p for j in range(n2)] for i in range(n1)])
        want = np.where(open_, sync, u).astype(np.int8)
        P = oracle.Problem(oracle.RULE_LIFE, n1, n2, seed=seed, scheme=oracle.STOCHASTIC, scheme_p=p, **B3S23)
        assert np.array_equal(oracle.step_reference(P, u, t), want)
        assert np.array_equal(oracle.run_array(P, u, t, 1, nthreads=2), want)
        assert 0 < open_.sum() < open_.size


def test_classic_patterns(oracle):
    """Blinker, block and glider (test/test_rules.jl:109-122)."""
    life = oracle.Problem(oracle.RULE_LIFE, 5, 5, birth=oracle.mask([3]), survive=oracle.mask([2, 3]))
    blinker = np.zeros((5, 5), np.int8)
    blinker[2, 1:4] = 1
    assert np.array_equal(oracle.run_array(life, blinker, 0, 1), blinker.T)
    assert np.array_equal(oracle.run_array(life, blinker, 0, 2), blinker)
    g = np.zeros((10, 10), np.int8)
    g[1, 2] = g[2, 3] = 1
    g[3, 1:4] = 1
    life10 = oracle.Problem(oracle.RULE_LIFE, 10, 10, birth=oracle.mask([3]), survive=oracle.mask([2, 3]))
    assert np.array_equal(oracle.run_array(life10, g, 0, 4), np.roll(g, (1, 1), (0, 1)))
    assert np.array_equal(oracle.run_array(life10, g, 0, 40), np.roll(g, (10, 10), (0, 1)))


def conformance_problems(oracle):
    """Int8 cases of the reference's conformance battery that this path covers
    (test/backend_conformance.jl:171-211), plus Larger-than-Life and forest fire."""
    o = oracle
    B3S23 = dict(birth=o.mask([3]), survive=o.mask([2, 3]))
    return [
        ("Life on a torus", o.Problem(o.RULE_LIFE, 20, 24, **B3S23), 30, None),
        ("Life on a cylinder", o.Problem(o.RULE_LIFE, 20, 24, boundary=(o.PERIODIC, o.CONSTANT), **B3S23), 30, None),
        ("radius-2 von Neumann, mixed edges",
         o.Problem(o.RULE_LIFE, 15, 17, nbhd=o.VON_NEUMANN, radius=2, birth=o.mask([3]),
                   survive=o.mask([2, 3, 4, 5]), boundary=(o.REFLECTING, o.CONSTANT), constant=(0, 1)), 20, None),
        ("Brian's Brain", o.Problem(o.RULE_GENERATIONS, 18, 18, birth=o.mask([2]), survive=0, states=3), 25, None),
        ("Moore(4) wider than the torus", o.Problem(o.RULE_LIFE, 3, 7, radius=4, birth=o.mask([5, 6, 7]),
                                                     survive=o.mask([4, 5, 6, 7, 8])), 8, None),
        ("Larger than Life, Moore(5)", o.Problem(o.RULE_LIFE, 40, 37, radius=5, birth=o.mask(range(34, 46)),
                                                 survive=o.mask(range(34, 59))), 12, None),
        ("Stochastic(0.4) Life", o.Problem(o.RULE_LIFE, 20, 20, seed=2, scheme=o.STOCHASTIC, scheme_p=0.4,
                                           **B3S23), 15, None),
        ("Stochastic(0.5f0) Life", o.Problem(o.RULE_LIFE, 20, 20, seed=12, scheme=o.STOCHASTIC, scheme_p=0.5,
                                             scheme_p_f32=True, **B3S23), 15, None),
        ("Checkerboard majority", o.Problem(o.RULE_LIFE, 18, 18, nbhd=o.VON_NEUMANN, birth=o.mask([5, 6, 7, 8]),
                                            survive=o.mask([4, 5, 6, 7, 8]), scheme=o.CHECKERBOARD), 10, None),
        ("forest fire, Grid Constant(0)", o.Problem(o.RULE_FOREST_FIRE, 40, 30, nbhd=o.VON_NEUMANN, seed=3,
                                                    boundary=(o.CONSTANT, o.CONSTANT)), 30, (0.3, 0.01)),
        ("forest fire, Float32 parameters", o.Problem(o.RULE_FOREST_FIRE, 33, 21, nbhd=o.VON_NEUMANN, seed=5,
                                                      params_f32=True), 30, (0.3, 0.01)),
    ]


def test_array_equals_reference(oracle):
    rng = np.random.default_rng(2026)
    for name, P, steps, params in conformance_problems(oracle):
        C = P.states if P.rule == oracle.RULE_GENERATIONS else (3 if P.rule == oracle.RULE_FOREST_FIRE else 2)
        u = rng.integers(0, C, size=(P.n1, P.n2)).astype(np.int8)
        ref = u.copy()
        for t in range(steps):
            ref = oracle.step_reference(P, ref, t, params)
        for nt in (1, 4):
            got = oracle.run_array(P, u, 0, steps, params, nthreads=nt)
            assert np.array_equal(got, ref), (name, nt)
        assert not np.array_equal(ref, u), name  # the battery is not vacuous


def test_stochastic_one_is_synchronous(oracle):
    """test/test_schemes.jl:8-9."""
    o = oracle
    u = np.random.default_rng(11).integers(0, 2, (20, 20)).astype(np.int8)
    a = o.Problem(o.RULE_LIFE, 20, 20, birth=o.mask([3]), survive=o.mask([2, 3]), scheme=o.STOCHASTIC, scheme_p=1.0)
    b = o.Problem(o.RULE_LIFE, 20, 20, birth=o.mask([3]), survive=o.mask([2, 3]))
    assert np.array_equal(o.run_array(a, u, 0, 5), o.run_array(b, u, 0, 5))


def test_checkerboard_against_definition(oracle):
    """schemes.jl:42-51: even index sums first, then odd ones, each reading the
    state the first half left (1-based indices)."""
    o = oracle
    u = np.random.default_rng(5).integers(0, 2, (9, 8)).astype(np.int8)
    P = o.Problem(o.RULE_LIFE, 9, 8, nbhd=o.VON_NEUMANN, birth=o.mask([2, 3]), survive=o.mask([1, 2]),
                  scheme=o.CHECKERBOARD)
    v = u.copy()
    for odd in (0, 1):
        w = v.copy()
        for i in range(9):
            for j in range(8):
                if ((i + 1 + j + 1) % 2) != odd:
                    continue
                n = sum(v[(i + a) % 9, (j + b) % 8] == 1 for a, b in ((0, -1), (-1, 0), (1, 0), (0, 1)))
                w[i, j] = (n in (1, 2)) if v[i, j] == 1 else (n in (2, 3))
        v = w
    assert np.array_equal(o.step_reference(P, u, 0), v)


@pytest.mark.parametrize("nb,r,dims,bnd,const", [("moore", 1, (9, 11), "rr", (0, 0)), ("moore", 2, (13, 10), "cp", (1, 0)),
                                                ("vn", 1, (7, 7), "pc", (0, 1)), ("moore", 2, (11, 9), "pp", (0, 0))])
def test_checkerboard_edges_against_definition(oracle, nb, r, dims, bnd, const):
    """Checkerboard (src/schemes.jl:42-51) on Reflecting, Constant and odd Periodic edges: the
    cells of even 1-based index sum take the synchronous rule's value (naive_life) from the
    current state, then the odd cells from the state the first half left; halo cells read
    through the boundary images, so they carry their images' states."""
    kinds = {"p": oracle.PERIODIC, "r": oracle.REFLECTING, "c": oracle.CONSTANT}
    bounds = (kinds[bnd[0]], kinds[bnd[1]])
    nbhd = oracle.MOORE if nb == "moore" else oracle.VON_NEUMANN
    n1, n2 = dims
    birth, survive = oracle.mask([2, 3, 6]), oracle.mask([1, 2, 4, 5])
    rng = np.random.default_rng(n1 * 31 + n2)
    i, j = np.meshgrid(np.arange(1, n1 + 1), np.arange(1, n2 + 1), indexing="ij")
    for _ in range(2):
        u = (rng.random((n1, n2)) < 0.4).astype(np.int8)
        v = u
        for odd in (0, 1):
            v = np.where((i + j) % 2 == odd, naive_life(oracle, v, r, nbhd, birth, survive, bounds, const), v)
        P = oracle.Problem(oracle.RULE_LIFE, n1, n2, nbhd=nbhd, radius=r, birth=birth, survive=survive,
                           boundary=bounds, constant=const, scheme=oracle.CHECKERBOARD)
        assert np.array_equal(oracle.step_reference(P, u, 0), v)
        assert np.array_equal(oracle.run_array(P, u, 0, 1, nthreads=2), v)


@pytest.mark.parametrize("scheme,bnd,const", [("sync", "rr", (0, 0)), ("stoch", "cp", (1, 0))])
def test_mask_against_definition(oracle, scheme, bnd, const):
    """A mask (src/environment.jl:123-130, src/backends.jl:448-450): a cell whose mask is
    false keeps its state in every step, while its neighbours still read it; the others take
    the scheme's update (Moore(2) Life here, the Stochastic gate as draw 0 below p)."""
    kinds = {"p": oracle.PERIODIC, "r": oracle.REFLECTING, "c": oracle.CONSTANT}
    bounds = (kinds[bnd[0]], kinds[bnd[1]])
    n1, n2, seed, p = 15, 12, 8, 0.6
    birth, survive = oracle.mask([4, 5, 6, 7]), oracle.mask([3, 4, 5, 6, 8])
    rng = np.random.default_rng(len(scheme) + n1)
    for t in (0, 2):
        u = (rng.random((n1, n2)) < 0.35).astype(np.int8)
        mask = rng.random((n1, n2)) < 0.7
        upd = naive_life(oracle, u, 2, oracle.MOORE, birth, survive, bounds, const)
        if scheme == "stoch":
            gate = np.array([[oracle.uniform(seed, i + j * n1 + 1, t, 0) < p for j in range(n2)] for i in range(n1)])
            upd = np.where(gate, upd, u)
        want = np.where(mask, upd, u).astype(np.int8)
        P = oracle.Problem(oracle.RULE_LIFE, n1, n2, radius=2, birth=birth, survive=survive, boundary=bounds,
                           constant=const, seed=seed, scheme=oracle.STOCHASTIC if scheme == "stoch" else
                           oracle.SYNCHRONOUS, scheme_p=p if scheme == "stoch" else 1.0)
        E = oracle.Env(mask=mask)
        assert np.array_equal(oracle.step_reference_env(P, E, u, t), want)
        assert np.array_equal(oracle.run_array_env(P, E, u, t, 1, nthreads=2), want)
        assert np.array_equal(want[~mask], u[~mask]) and not np.array_equal(want, u)


def test_forest_fire_rates(oracle):
    """bernoulli(p) hits at rate p (test/test_random.jl:51-56) through the rule."""
    o = oracle
    P = o.Problem(o.RULE_FOREST_FIRE, 200, 100, nbhd=o.VON_NEUMANN, seed=9, boundary=(o.CONSTANT, o.CONSTANT))
    u = o.run_array(P, np.zeros((200, 100), np.int8), 0, 1, (0.3, 0.0))
    assert abs((u == 1).mean() - 0.3) < 0.015
    assert np.all(o.run_array(P, np.zeros((200, 100), np.int8), 0, 3, (0.0, 0.0)) == 0)
    full = o.run_array(P, np.ones((200, 100), np.int8), 0, 1, (0.0, 1.0))
    assert np.all(full == 2)


def test_morans_i(oracle):
    """test/test_extras.jl:140-144 (measures.jl:91-107)."""
    o = oracle
    checker = np.array([[(i + j) % 2 for j in range(1, 7)] for i in range(1, 7)], np.int8)
    assert abs(o.morans_i(o.Problem(o.RULE_LIFE, 6, 6), checker) + 1.0) < 1e-12
    stripes = np.array([[1 if j <= 3 else 0 for j in range(1, 7)] for i in range(1, 7)], np.int8)
    grid = o.Problem(o.RULE_LIFE, 6, 6, boundary=(o.CONSTANT, o.CONSTANT))
    assert o.morans_i(grid, stripes) > 0.5
    assert np.isnan(o.morans_i(o.Problem(o.RULE_LIFE, 3, 3), np.ones((3, 3), np.int8)))
    counts, other = o.state_counts(np.array([[0, 1], [0, 0]], np.int8), 3)
    assert counts == [3, 1, 0] and other == 0


def test_lenia_direct_vs_fft(oracle):
    """test/test_extras.jl:121-123: FP64 direct and FFT agree to 1e-10 after 10 steps."""
    rng = np.random.default_rng(4)
    u = np.zeros((64, 64))
    u[20:40, 20:40] = rng.random((20, 20))
    off, w = oracle.lenia_weights(13)
    assert len(w) == 516 and abs(w.sum() - 1) < 1e-14
    fft = oracle.LeniaFFT(64, 64)
    a = u.copy()
    b = u.copy()
    for _ in range(10):
        a = oracle.lenia_step_direct(a, nthreads=4)
        b = fft.step(b)
    assert np.max(np.abs(a - b)) < 1e-10
    assert np.max(np.abs(a - u)) > 1e-3  # it moved
