"""GPU parity of the sweep's environment: masks on every Int8 rule and scheme, and the
kernel-field SI rule (direct and FFT fields, covariates, Float32 and Float64) against the
oracle, as test/backend_conformance.jl:52-57,72-75,158-167 demands of every backend.

The SI rule's probability is 1 - exp(-lambda): the device's exp and the C library's may
differ in the last bit, which changes an outcome only when a draw lands on that bit (about
2^-53 per drawing cell in Float64, 2^-24 x 2^-3 in Float32), so the states are compared
exactly. Float32 FFT fields differ from direct sums by rounding (~1e-7 relative); that
comparison allows a bounded share of differing cells, stated in the test."""
import math
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


def _bnd(ca, o, kinds):
    m = {"p": (ca.Periodic(), o.PERIODIC), "r": (ca.Reflecting(), o.REFLECTING), "c": (ca.Constant(0), o.CONSTANT)}
    return tuple(m[k][0] for k in kinds), tuple(m[k][1] for k in kinds)


SI_CASES = [
    # name, dims, boundaries, kernel (product, oracle args), precision, covariate nt, mask, scheme, beta, seed, steps
    ("kernel field, cycling covariate and mask (battery case)", (30, 26), "rc",
     ("aniso-exp", 1.5, math.pi / 4, 1.0), "Float64", 3, True, "sync", 4.0, 9, 12),
    ("Float32 kernel field (battery case)", (30, 26), "pp", ("aniso-gauss", 1.5, 1.0, 1.0), "Float32", 0, False,
     "sync", 2.0, 13, 12),
    ("Float64 Gaussian field, 700 x 450 torus, fixed covariate", (700, 450), "pp", ("gauss", 2.0, 0, 0), "Float64", 1,
     False, "sync", 3.0, 21, 25),
    ("Float32 exponential field, Stochastic(0.6), mask", (300, 260), "rr", ("exp", 2.0, 0, 0), "Float32", 0, True,
     "stoch", 2.5, 5, 20),
    ("Checkerboard, uniform radius 3, Float32 covariate", (128, 96), "cp", ("uniform", 3, 0, 0), "Float64", 2, False,
     "check", 1.5, 6, 15),
]


def _kernels(ca, o, spec):
    kind = spec[0]
    if kind == "aniso-exp":
        return (ca.AnisotropicKernel(ca.ExponentialKernel(spec[1]), spec[2], spec[3]),
                (o.K_ANISOTROPIC, int(math.ceil(5 * spec[1])), spec[1],
                 dict(base=o.K_EXPONENTIAL, direction=spec[2], strength=spec[3])))
    if kind == "aniso-gauss":
        return (ca.AnisotropicKernel(ca.GaussianKernel(spec[1]), spec[2], spec[3]),
                (o.K_ANISOTROPIC, int(math.ceil(3 * spec[1])), spec[1],
                 dict(base=o.K_GAUSSIAN, direction=spec[2], strength=spec[3])))
    if kind == "gauss":
        return ca.GaussianKernel(spec[1]), (o.K_GAUSSIAN, int(math.ceil(3 * spec[1])), spec[1], {})
    if kind == "exp":
        return ca.ExponentialKernel(spec[1]), (o.K_EXPONENTIAL, int(math.ceil(5 * spec[1])), spec[1], {})
    return ca.UniformKernel(spec[1]), (o.K_UNIFORM, spec[1], 0.0, {})


def _si_pair(ca, o, case, method="direct"):
    name, (n1, n2), bk, kspec, prec, nt, use_mask, scheme, beta, seed, steps = case
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    u0 = np.zeros((n1, n2), np.int8)
    for _ in range(max(1, n1 * n2 // 20000)):
        u0[rng.integers(n1), rng.integers(n2)] = 1
    u0[n1 // 2, n2 // 2] = 1
    bounds, obounds = _bnd(ca, o, bk)
    space = ca.Lattice((n1, n2), bounds)
    kern, (okind, orad, oa, okw) = _kernels(ca, o, kspec)
    f32 = prec == "Float32"
    fields = {"P": ca.KernelField(kern, "x == 1", method=method, precision=prec)}
    covs, cov = {}, None
    if nt:
        cov = rng.random((n1, n2, nt)) if nt > 1 else rng.random((n1, n2))
        if "Float32 covariate" in name:
            cov = cov.astype(np.float32)
        covs = {"suitability": cov}
    mask = None
    if use_mask:
        mask = np.ones((n1, n2), bool)
        mask[n1 // 6: n1 // 3, n2 // 6: 3 * n2 // 4] = False
    rule = ca.KernelSI("P", covariate="suitability" if nt else None, float32=f32)
    sch = {"sync": ca.Synchronous(), "stoch": ca.Stochastic(0.6), "check": ca.Checkerboard()}[scheme]
    pb = np.float32(beta) if f32 else beta
    prob = ca.CAProblem.new(rule, u0, steps, {"β": pb}, space=space, seed=seed, covariates=covs, fields=fields,
                            mask=mask)
    taps, w = o.kernel_weights(okind, orad, oa, **okw)
    E = o.Env(mask=mask, taps=taps, weights=w, field_f32=f32,
              cov=(cov if cov is None or cov.ndim == 3 else cov[:, :, None]))
    P = o.Problem(o.RULE_SI_FIELD, n1, n2, boundary=obounds, seed=seed,
                  scheme={"sync": o.SYNCHRONOUS, "stoch": o.STOCHASTIC, "check": o.CHECKERBOARD}[scheme],
                  scheme_p=0.6 if scheme == "stoch" else 1.0, params_f32=f32)
    return prob, sch, P, E, u0, float(pb), steps


@pytest.mark.parametrize("case", SI_CASES, ids=[c[0] for c in SI_CASES])
def test_si_field_direct(ca, oracle, case):
    prob, sch, P, E, u0, beta, steps = _si_pair(ca, oracle, case)
    saveat = max(1, steps // 4)
    sol = ca.solve(prob, sch, backend=ca.GB300Backend(), saveat=saveat)
    u, t = u0, 0
    for k, ts in enumerate(sol.t):
        if ts > t:
            u = oracle.run_array_env(P, E, u, t, ts - t, (beta,), nthreads=16)
            t = ts
        assert np.array_equal(sol.u[k], u), f"{case[0]}: t = {ts} differs in {(sol.u[k] != u).sum()} cells"
    assert u.sum() > u0.sum()  # the epidemic spread
    if E.mask is not None:
        assert np.array_equal(u[~E.mask], u0[~E.mask])


def test_si_field_fft_float64(ca, oracle):
    """method=:fft on a torus (this library's transforms: 384 = 2^7 3, 256 = 2^8): the Float64
    field differs from the direct sum by rounding (~1e-16), which changes an outcome with
    probability ~1e-16 per draw."""
    case = ("FFT Float64, 384 x 256 torus", (384, 256), "pp", ("exp", 2.0, 0, 0), "Float64", 2, True, "sync", 2.0,
            31, 20)
    prob, sch, P, E, u0, beta, steps = _si_pair(ca, oracle, case, method="fft")
    got = ca.final_state(ca.solve(prob, sch, backend=ca.GB300Backend(), save_everystep=False))
    want = oracle.run_array_env(P, E, u0, 0, steps, (beta,), nthreads=16)
    assert np.array_equal(got, want), f"{(got != want).sum()} cells differ"
    assert want.sum() > 50


@pytest.mark.parametrize("dims", [(256, 256), (512, 1024), (1024, 75)])
def test_si_field_fft_float32(ca, oracle, dims):
    """Float32 FFT fields carry ~1e-7 relative rounding, so an outcome changes when a
    24-bit draw falls within it: at most 0.1% of the cells may differ after 10 steps (256^2:
    the mixed-radix transforms; 512 x 1024: the ones compiled for power-of-two lengths;
    1024 x 75: those on axis 1 with an odd number of lines, the mixed-radix ones on axis 2)."""
    case = (f"FFT Float32, {dims[0]} x {dims[1]} torus", dims, "pp", ("gauss", 2.0, 0, 0), "Float32", 0, False, "sync",
            2.0, 17, 10)
    prob, sch, P, E, u0, beta, steps = _si_pair(ca, oracle, case, method="fft")
    got = ca.final_state(ca.solve(prob, sch, backend=ca.GB300Backend(), save_everystep=False))
    want = oracle.run_array_env(P, E, u0, 0, steps, (beta,), nthreads=16)
    assert (got != want).sum() <= 0.001 * got.size
    assert want.sum() > 50


def test_si_identity_source(ca, oracle):
    """source = identity: states other than 0 and 1 weigh the field by their value."""
    rng = np.random.default_rng(4)
    u0 = (rng.random((90, 70)) < 0.02).astype(np.int8) * rng.integers(1, 4, (90, 70)).astype(np.int8)
    kern = ca.GaussianKernel(1.5)
    prob = ca.CAProblem.new(ca.KernelSI("f"), u0, 10, {"β": 0.7}, seed=3,
                            fields={"f": ca.KernelField(kern, "identity")})
    got = ca.final_state(ca.solve(prob, ca.Synchronous(), backend=ca.GB300Backend(), save_everystep=False))
    taps, w = oracle.kernel_weights(oracle.K_GAUSSIAN, 5, 1.5)
    P = oracle.Problem(oracle.RULE_SI_FIELD, 90, 70, seed=3)
    want = oracle.run_array_env(P, oracle.Env(taps=taps, weights=w, identity=True), u0, 0, 10, (0.7,), nthreads=8)
    assert np.array_equal(got, want) and not np.array_equal(want, u0)


MASK_CASES = [
    ("Life torus", "life", (200, 150), dict(birth=[3], survive=[2, 3]), "sync", (0, 0), 30),
    ("Larger than Life Moore(3) grid", "life", (130, 110), dict(r=3, birth=range(9, 15), survive=range(8, 20)),
     "sync", (0, 0), 20),
    ("Brian's Brain", "gen", (120, 90), dict(birth=[2], survive=[], states=3), "sync", (0, 0), 25),
    ("forest fire grid", "fire", (300, 200), dict(nb="vn"), "sync", (0.05, 0.001), 30),
    ("forest fire, Stochastic(0.5), tiled", "fire", (600, 300), dict(nb="vn"), "stoch", (0.05, 0.001), 20),
    ("forest fire, Checkerboard, TMA-staged", "fire", (256, 512), dict(nb="vn"), "check", (0.1, 0.01), 16),
    ("Stochastic(0.5) Life", "life", (64, 80), dict(birth=[3], survive=[2, 3]), "stoch", (0, 0), 15),
    ("Checkerboard majority", "life", (70, 50), dict(nb="vn", birth=[3, 4], survive=[2, 3, 4]), "check", (0, 0), 12),
]


@pytest.mark.parametrize("case", MASK_CASES, ids=[c[0] for c in MASK_CASES])
def test_masks(ca, oracle, case):
    name, kind, (n1, n2), kw, scheme, params, steps = case
    o = oracle
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    r = kw.get("r", 1)
    nb = ca.VonNeumann(r) if kw.get("nb") == "vn" else ca.Moore(r)
    if kind == "life":
        rule = ca.Life(list(kw["birth"]), list(kw["survive"]), neighbourhood=nb)
        P = o.Problem(o.RULE_LIFE, n1, n2, nbhd=o.VON_NEUMANN if kw.get("nb") == "vn" else o.MOORE, radius=r,
                      birth=o.mask(kw["birth"]), survive=o.mask(kw["survive"]))
        C = 2
    elif kind == "gen":
        rule = ca.Generations(":brians_brain")
        P = o.Problem(o.RULE_GENERATIONS, n1, n2, birth=o.mask([2]), survive=0, states=3)
        C = 3
    else:
        rule = ca.ForestFire()
        P = o.Problem(o.RULE_FOREST_FIRE, n1, n2, nbhd=o.VON_NEUMANN, seed=4,
                      boundary=(o.CONSTANT, o.CONSTANT))
        C = 3
    space = ca.Grid(n1, n2) if kind == "fire" else (ca.Grid(n1, n2) if "grid" in name else ca.Torus(n1, n2))
    if "grid" in name and kind == "life":
        P.boundary = (o.CONSTANT, o.CONSTANT)
    P.seed = 4
    if scheme == "stoch":
        P.scheme, P.scheme_p = o.STOCHASTIC, 0.5
    elif scheme == "check":
        P.scheme = o.CHECKERBOARD
    sch = {"sync": ca.Synchronous(), "stoch": ca.Stochastic(0.5), "check": ca.Checkerboard()}[scheme]
    u0 = rng.integers(0, C, (n1, n2)).astype(np.int8)
    mask = rng.random((n1, n2)) < 0.85
    pd = {"p": params[0], "f": params[1]} if kind == "fire" else None
    prob = ca.CAProblem.new(rule, u0, steps, pd, space=space, seed=4, mask=mask)
    got = ca.final_state(ca.solve(prob, sch, backend=ca.GB300Backend(), save_everystep=False))
    want = o.run_array_env(P, o.Env(mask=mask), u0, 0, steps, params if kind == "fire" else None, nthreads=8)
    assert np.array_equal(got, want), f"{name}: {(got != want).sum()} cells differ"
    assert np.array_equal(got[~mask], u0[~mask]) and not np.array_equal(got, u0)


def _geometry(ca, st):
    import ctypes
    k, rows, staging = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    ca.capi.check(ca.capi.lib().gbca_geometry(st.handle, None, ctypes.byref(k), ctypes.byref(rows),
                                              ctypes.byref(staging)))
    return int(k.value), int(rows.value), int(staging.value)


BITSLICED_MASK_CASES = [
    # name, rule kind, dims, boundary kinds, scheme, steps
    ("Life on a 512 x 256 torus, three passes", "life", (512, 256), "pp", "sync", 40),
    ("Life Moore(2) on a 300 x 200 grid", "life2", (300, 200), "cc", "sync", 20),
    ("Life on a reflecting 200 x 130 lattice", "life", (200, 130), "rr", "sync", 25),
    ("Brian's Brain, Checkerboard, 256 x 128 torus", "gen", (256, 128), "pp", "check", 10),
    ("von Neumann majority, Stochastic(0.5), 320 x 96 torus", "vn", (320, 96), "pp", "stoch", 12),
]


@pytest.mark.parametrize("case", BITSLICED_MASK_CASES, ids=[c[0] for c in BITSLICED_MASK_CASES])
def test_masks_bit_sliced(ca, oracle, case):
    """Masked Life and Generations on the bit-sliced kernel (its gated form, with the mask's
    bits in shared memory): the geometry query names a fast-kernel geometry, and the state
    equals the oracle's after every step."""
    name, kind, (n1, n2), bk, scheme, steps = case
    o = oracle
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    bnd, obnd = _bnd(ca, o, bk)
    if kind == "gen":
        rule = ca.Generations(":brians_brain")
        P = o.Problem(o.RULE_GENERATIONS, n1, n2, birth=o.mask([2]), survive=0, states=3)
        C = 3
    else:
        r = 2 if kind == "life2" else 1
        birth, survive = ([3, 4], [2, 3, 4]) if kind == "vn" else ((range(5, 8), range(4, 9)) if r == 2 else
                                                                  ([3], [2, 3]))
        nb = ca.VonNeumann(1) if kind == "vn" else ca.Moore(r)
        rule = ca.Life(list(birth), list(survive), neighbourhood=nb)
        P = o.Problem(o.RULE_LIFE, n1, n2, nbhd=o.VON_NEUMANN if kind == "vn" else o.MOORE, radius=r,
                      birth=o.mask(birth), survive=o.mask(survive))
        C = 2
    P.boundary = obnd
    P.seed = 6
    if scheme == "stoch":
        P.scheme, P.scheme_p = o.STOCHASTIC, 0.5
    elif scheme == "check":
        P.scheme = o.CHECKERBOARD
    sch = {"sync": ca.Synchronous(), "stoch": ca.Stochastic(0.5), "check": ca.Checkerboard()}[scheme]
    u0 = rng.integers(0, C, (n1, n2)).astype(np.int8)
    mask = rng.random((n1, n2)) < 0.8
    prob = ca.CAProblem.new(rule, u0, steps, space=ca.Lattice((n1, n2), bnd), seed=6, mask=mask)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, sch)
    ca.set_state(B, st, u0)
    want = u0
    for t in range(steps):
        ca.advance(B, st, prob, sch, None, t)
        want = o.run_array_env(P, o.Env(mask=mask), want, t, 1, None, nthreads=8)
        if t in (0, steps // 2, steps - 1):
            got = ca.current_state(B, st)
            assert np.array_equal(got, want), f"{name}, step {t + 1}: {(got != want).sum()} cells differ"
    assert _geometry(ca, st)[0] > 0, "the masked sweep fell back to the general kernel"
    for t in range(steps, 2 * steps):  # queued steps run as whole passes
        ca.advance(B, st, prob, sch, None, t)
    want = o.run_array_env(P, o.Env(mask=mask), want, steps, steps, None, nthreads=8)
    assert np.array_equal(ca.current_state(B, st), want)
    assert np.array_equal(want[~mask], u0[~mask])
    st.close()


def test_masked_life_states_outside_range(ca, oracle):
    """Masked Life on a state holding values other than 0 and 1: a masked cell keeps its value,
    which the bit-sliced kernel's indicator bits cannot hold, so the sweep stays on the general
    kernel; the result equals the oracle's."""
    rng = np.random.default_rng(12)
    n1, n2 = 128, 96
    odd = rng.integers(-2, 4, (n1, n2)).astype(np.int8)
    mask = rng.random((n1, n2)) < 0.7
    prob = ca.CAProblem.new(ca.Life(":conway"), np.zeros((n1, n2), np.int8), 10, mask=mask)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    ca.set_state(B, st, odd)
    for t in range(10):
        ca.advance(B, st, prob, ca.Synchronous(), None, t)
    P = oracle.Problem(oracle.RULE_LIFE, n1, n2, birth=oracle.mask([3]), survive=oracle.mask([2, 3]))
    want = oracle.run_array_env(P, oracle.Env(mask=mask), odd, 0, 10, None, nthreads=8)
    assert np.array_equal(ca.current_state(B, st), want)
    assert _geometry(ca, st) == (0, 0, 0)
    st.close()
