"""The environment of a sweep on the CPU: dispersal-kernel weights, kernel fields,
covariates and masks. The oracle is pinned to the reference's own assertions
(test/test_environment.jl:3-110); the product's host-side kernel_weights must equal the
oracle's bit for bit (both call the C library's exp/pow/atan2/cos)."""
import math

import numpy as np
import pytest


def _at(o, w, off):
    """Weight of kernel offset `off` given taps (negated offsets) and weights."""
    for k, (a, b) in enumerate(o):
        if (-a, -b) == tuple(off):
            return w[k]
    raise KeyError(off)


def test_kernel_weight_pins(oracle):
    o = oracle
    # test_environment.jl:4-11
    for kind, r, a, kw in [(o.K_GAUSSIAN, 5, 1.5, {}), (o.K_EXPONENTIAL, 5, 1.0, {}), (o.K_POWERLAW, 4, 2.0, {}),
                           (o.K_UNIFORM, 2, 0.0, {}), (o.K_LENIA, 5, 0.0, {}),
                           (o.K_LENIA, 6, 0.0, dict(peaks=(0.5, 1.0)))]:
        taps, w = o.kernel_weights(kind, r, a, **kw)
        assert abs(w.sum() - 1) < 1e-12 and (w > 0).all() and len(taps) == len(w)
        assert all(math.sqrt(x * x + y * y) <= r + 1e-9 for x, y in taps)
    # :12-15
    taps, w = o.kernel_weights(o.K_UNIFORM, 1)
    assert {(-x, -y) for x, y in taps} == {(0, 0), (1, 0), (-1, 0), (0, 1), (0, -1)}
    taps, _ = o.kernel_weights(o.K_UNIFORM, 1, include_centre=False)
    assert (0, 0) not in {tuple(t) for t in taps}
    # :17-21
    taps, w = o.kernel_weights(o.K_GAUSSIAN, 3, 1.0)
    assert _at(taps, w, (0, 0)) > _at(taps, w, (0, 2))
    taps, _ = o.kernel_weights(o.K_LENIA, 4)
    assert (0, 0) not in {tuple(t) for t in taps}
    # :23-32 anisotropy: direction 0 is east (+column)
    taps, w = o.kernel_weights(o.K_ANISOTROPIC, 2, 1.0, base=o.K_GAUSSIAN, direction=0.0, strength=2.0)
    assert _at(taps, w, (0, 1)) > _at(taps, w, (-1, 0)) > _at(taps, w, (0, -1))
    taps, w = o.kernel_weights(o.K_ANISOTROPIC, 2, 1.0, base=o.K_GAUSSIAN, direction=math.pi / 2, strength=2.0)
    assert _at(taps, w, (-1, 0)) > _at(taps, w, (1, 0))
    # :34-35
    taps, w = o.kernel_weights(o.K_EMPIRICAL, 0, empirical=np.array([[0, 1, 0], [2, 4, 2], [0, 1, 0]], float))
    assert abs(_at(taps, w, (0, 0)) - 0.4) < 1e-15


def test_kernel_field_pins(oracle):
    o = oracle
    # test_environment.jl:49-53: a uniform radius-1 field, 1/5 on the cross around a live cell
    u = np.zeros((7, 7), np.int8)
    u[3, 3] = 1
    taps, w = o.kernel_weights(o.K_UNIFORM, 1)
    P = o.Problem(o.RULE_SI_FIELD, 7, 7)
    f = o.kernel_field(P, o.Env(taps=taps, weights=w, identity=True), u)
    assert abs(f[3, 3] - 0.2) < 1e-15 and abs(f[2, 3] - 0.2) < 1e-15 and abs(f[3, 4] - 0.2) < 1e-15
    assert f[2, 2] == 0
    # :55-58: beyond a Constant(1) edge cells count as 1
    P = o.Problem(o.RULE_SI_FIELD, 5, 5, boundary=(o.CONSTANT, o.CONSTANT), constant=(1, 1))
    e = o.kernel_field(P, o.Env(taps=taps, weights=w, identity=True), np.zeros((5, 5), np.int8))
    assert abs(e[0, 0] - 0.4) < 1e-15 and abs(e[0, 2] - 0.2) < 1e-15 and e[2, 2] == 0
    # :75-81: an eastward kernel carries a source's influence east; an empirical kernel with
    # all its mass at offset (-1, -1) moves the source there
    src = np.zeros((9, 9), np.int8)
    src[4, 4] = 1
    P = o.Problem(o.RULE_SI_FIELD, 9, 9)
    taps, w = o.kernel_weights(o.K_ANISOTROPIC, 3, 1.0, base=o.K_GAUSSIAN, direction=0.0, strength=3.0)
    f = o.kernel_field(P, o.Env(taps=taps, weights=w, identity=True), src)
    assert f[4, 5] > f[4, 3] and abs(f[3, 4] - f[5, 4]) < 1e-15
    taps, w = o.kernel_weights(o.K_EMPIRICAL, 0, empirical=np.array([[1, 0, 0], [0, 0, 0], [0, 0, 0]], float))
    f = o.kernel_field(P, o.Env(taps=taps, weights=w, identity=True), src)
    assert abs(f[3, 3] - 1) < 1e-15 and abs(f.sum() - 1) < 1e-15


def test_covariate_cycles_and_mask_freezes(oracle):
    """A covariate with nt slices is read at slice mod1(t + 1, nt) (test_environment.jl:84-90):
    with cov = [0, 1] cycling and a huge beta, the SI rule infects only on odd t. A masked
    cell never updates (test_environment.jl:104-108)."""
    o = oracle
    u = np.zeros((9, 9), np.int8)
    u[4, 4] = 1
    taps, w = o.kernel_weights(o.K_UNIFORM, 1)
    cov = np.stack([np.zeros((9, 9)), np.ones((9, 9))], axis=2)
    mask = np.ones((9, 9), bool)
    mask[4, 5] = False
    E = o.Env(taps=taps, weights=w, cov=cov, mask=mask)
    P = o.Problem(o.RULE_SI_FIELD, 9, 9, seed=1)
    a = o.step_reference_env(P, E, u, 0, (1e9,))
    assert np.array_equal(a, u)  # slice 1 = zeros: no infection
    b = o.step_reference_env(P, E, a, 1, (1e9,))
    assert b.sum() == 4 and b[3, 4] == b[5, 4] == b[4, 3] == 1 and b[4, 5] == 0  # masked cell stays
    assert np.array_equal(o.run_array_env(P, E, u, 0, 2, (1e9,), nthreads=3), b)


def test_array_env_matches_reference_env(oracle):
    """The oracle's two sweeps (serial ReferenceBackend, threaded ArrayBackend) agree with a
    field, a cycling covariate and a mask: the conformance battery's kernel-field case."""
    o = oracle
    rng = np.random.default_rng(2026)
    u0 = np.zeros((30, 26), np.int8)
    u0[14, 12] = 1
    taps, w = o.kernel_weights(o.K_ANISOTROPIC, 8, 1.5, base=o.K_EXPONENTIAL, direction=math.pi / 4, strength=1.0)
    mask = np.ones((30, 26), bool)
    mask[4:10, 4:20] = False
    E = o.Env(mask=mask, taps=taps, weights=w, cov=rng.random((30, 26, 3)))
    P = o.Problem(o.RULE_SI_FIELD, 30, 26, seed=9, boundary=(o.REFLECTING, o.CONSTANT))
    a = o.run_array_env(P, E, u0, 0, 12, (4.0,), nthreads=4)
    b = u0
    for t in range(12):
        b = o.step_reference_env(P, E, b, t, (4.0,))
    assert np.array_equal(a, b) and a.sum() > 20 and a[4:10, 4:20].sum() == 0
    # Life with a mask: the masked cells keep their state
    u = rng.integers(0, 2, (20, 24)).astype(np.int8)
    m = rng.random((20, 24)) < 0.8
    P = o.Problem(o.RULE_LIFE, 20, 24, birth=o.mask([3]), survive=o.mask([2, 3]))
    x = o.run_array_env(P, o.Env(mask=m), u, 0, 10, nthreads=2)
    y = u
    for t in range(10):
        y = o.step_reference_env(P, o.Env(mask=m), y, t)
    assert np.array_equal(x, y) and np.array_equal(x[~m], u[~m]) and not np.array_equal(x, u)


def test_product_kernel_weights_equal_oracle(gbca, oracle):
    ca, o = gbca, oracle
    E = np.random.default_rng(0).random((5, 7))
    cases = [(ca.GaussianKernel(1.5), (o.K_GAUSSIAN, 5, 1.5, {})),
             (ca.ExponentialKernel(1.5), (o.K_EXPONENTIAL, 8, 1.5, {})),
             (ca.PowerLawKernel(2.0, radius=4), (o.K_POWERLAW, 4, 2.0, {})),
             (ca.UniformKernel(3), (o.K_UNIFORM, 3, 0.0, {})),
             (ca.LeniaKernel(13, (1.0, 0.5)), (o.K_LENIA, 13, 0.0, dict(peaks=(1.0, 0.5)))),
             (ca.AnisotropicKernel(ca.ExponentialKernel(1.5), math.pi / 4, 1.0),
              (o.K_ANISOTROPIC, 8, 1.5, dict(base=o.K_EXPONENTIAL, direction=math.pi / 4, strength=1.0))),
             (ca.AnisotropicKernel(ca.GaussianKernel(1.5), 1.0, 1.0),
              (o.K_ANISOTROPIC, 5, 1.5, dict(base=o.K_GAUSSIAN, direction=1.0, strength=1.0))),
             (ca.EmpiricalKernel(E), (o.K_EMPIRICAL, 0, 0.0, dict(empirical=E)))]
    for k, (kind, r, a, kw) in cases:
        for centre in (True, False):
            f = ca.KernelField(k, "x == 1", include_centre=centre)
            taps, w, R = f.resolve(ca.Torus(40, 40), "f")
            ot, ow = o.kernel_weights(kind, r, a, include_centre=centre, **kw)
            assert np.array_equal(np.array(taps), ot) and np.array_equal(w, ow), type(k).__name__


def test_environment_validation(gbca):
    ca = gbca
    si = ca.KernelSI("f")
    u = np.zeros((6, 5), np.int8)
    f = {"f": ca.KernelField(ca.UniformKernel(1), "x == 1")}
    with pytest.raises(ca.StateShapeError):
        ca.CAProblem.new(si, u, 3, {"β": 1.0}, fields=f, covariates={"c": np.zeros((5, 6))})
    with pytest.raises(ca.ArgumentError):
        ca.CAProblem.new(si, u, 3, {"β": 1.0}, fields=f, mask=np.ones((6, 5)))
    with pytest.raises(ca.StateShapeError):
        ca.CAProblem.new(si, u, 3, {"β": 1.0}, fields=f, mask=np.ones((5, 5), bool))
    with pytest.raises(ca.ArgumentError):
        ca.CAProblem.new(si, u, 3, {"β": 1.0}, fields={"f": 1})
    with pytest.raises(ca.ArgumentError):
        ca.CAProblem.new(si, u, 3, {"β": 1.0}, space=ca.Grid(6, 5),
                         fields={"f": ca.KernelField(ca.UniformKernel(1), "x == 1", method="fft")})
    with pytest.raises(ca.ArgumentError):
        ca.KernelField(ca.UniformKernel(1), method="magic")
    with pytest.raises(ca.ArgumentError):
        ca.GaussianKernel(-1.0)
    with pytest.raises(ca.ArgumentError):
        ca.EmpiricalKernel(np.ones((2, 2)))
    # the rule names a field the problem lacks
    prob = ca.CAProblem.new(ca.KernelSI("g"), u, 3, {"β": 1.0}, fields=f)
    with pytest.raises(ca.ArgumentError):
        ca.check_problem(ca.GB300Backend(), prob, ca.Synchronous())
