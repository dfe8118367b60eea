"""Lenia on the GPU against the FP64 oracle (lenia.jl:42-47, environment.jl:151-169,
kernels.jl:87-104,174-189; the FFT convention of ext/CellularAutomataCoreFFTWExt.jl:17-30).

Float32 (direct and FFT): the convolution and growth run in FP32 with the weights
normalised in FP64; the per-step error (one GPU step vs one FP64 oracle step from the
same state) is held to 1e-5 max-abs. The end state after many steps is reported, not
bounded: the random-soup configuration is chaotic, and even an FP32 implementation with an
exactly rounded field drifts from the FP64 trajectory to O(1) max-abs by step 100.
Float64 (the reference's default precision): the FFT path stays within 1e-5 max-abs of the
FP64 oracle after 100 steps on the 2048 x 2048 configuration."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PER_STEP_TOL_F32 = 1e-5


@pytest.fixture(scope="module")
def ca():
    import __graft_entry__ as ge
    ge.build()
    m = ge.load_package()
    if m.capi.lib().gbca_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return m


def soup(n, patch, seed, dtype):
    """Uniform[0,1] in a central patch x patch square, 0 elsewhere (numpy PCG64(seed))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    u = np.zeros((n, n), dtype)
    c = n // 2
    u[c - patch // 2:c + patch // 2, c - patch // 2:c + patch // 2] = rng.random((patch, patch)).astype(np.float32)
    return u


def gpu_state(ca, rule, u0, space=None):
    B = ca.GB300Backend()
    prob = ca.CAProblem.new(rule, u0, 1, space=space)
    return B, prob, ca.allocate_state(B, prob, ca.Synchronous())


def gpu_step(ca, B, prob, st, u, k=1):
    ca.set_state(B, st, u)
    for t in range(k):
        ca.advance(B, st, prob, ca.Synchronous(), None, t)
    return ca.current_state(B, st)


@pytest.mark.parametrize("method", ["direct", "fft"])
def test_float32_per_step_error(ca, oracle, method):
    n = 512
    u = soup(n, 128, 4, np.float32)
    B, prob, st = gpu_state(ca, ca.Lenia(method=method, precision="Float32"), u)
    fft = oracle.LeniaFFT(n, n)
    worst = 0.0
    for _ in range(12):  # a dozen steps along the GPU's own trajectory
        nxt = gpu_step(ca, B, prob, st, u)
        want = fft.step(u.astype(np.float64))
        worst = max(worst, float(np.max(np.abs(nxt.astype(np.float64) - want))))
        u = nxt
    print(f"Float32 {method}: worst per-step max-abs error vs FP64 = {worst:.3e}")
    assert worst < PER_STEP_TOL_F32
    assert np.abs(u).sum() > 0


def test_float32_direct_matches_reference_float32_arithmetic(ca, oracle):
    """Against the oracle's Float32 restatement (precision=Float32 ArrayBackend arithmetic)
    on a Grid with Constant(0) edges: one step agrees to FP32 rounding."""
    n1, n2 = 200, 160
    rng = np.random.Generator(np.random.PCG64(9))
    u = rng.random((n1, n2)).astype(np.float32)
    space = ca.Grid(n1, n2)
    B, prob, st = gpu_state(ca, ca.Lenia(precision="Float32"), u, space)
    got = gpu_step(ca, B, prob, st, u)
    want32 = oracle.lenia_step_direct(u, f32=True, boundary=(oracle.CONSTANT, oracle.CONSTANT), nthreads=8)
    want64 = oracle.lenia_step_direct(u.astype(np.float64), boundary=(oracle.CONSTANT, oracle.CONSTANT), nthreads=8)
    assert np.max(np.abs(got - want32)) < 1e-5
    assert np.max(np.abs(got - want64)) < 1e-5


def test_other_radius_and_peaks(ca, oracle):
    """R = 6 with two rings takes the tap-list kernel; Float64 on a reflecting lattice."""
    n1, n2 = 96, 80
    rng = np.random.Generator(np.random.PCG64(2))
    u = rng.random((n1, n2))
    space = ca.Lattice((n1, n2), (ca.Reflecting(), ca.Periodic()))
    rule = ca.Lenia(R=6, peaks=(0.5, 1.0), mu=0.2, sigma=0.03, precision="Float64")
    B, prob, st = gpu_state(ca, rule, u, space)
    got = gpu_step(ca, B, prob, st, u, 3)
    want = u.copy()
    for _ in range(3):
        want = oracle.lenia_step_direct(want, R=6, peaks=(0.5, 1.0), mu=0.2, sigma=0.03,
                                        boundary=(oracle.REFLECTING, oracle.PERIODIC), nthreads=8)
    assert np.max(np.abs(got - want)) < 1e-12


def test_float64_direct_vs_fft(ca):
    """test/test_extras.jl:121-123 on the GPU: direct and FFT agree to 1e-10 after 10 steps."""
    u = soup(128, 48, 7, np.float64)
    a = gpu_step(ca, *gpu_state(ca, ca.Lenia(precision="Float64"), u), u, 10)
    b = gpu_step(ca, *gpu_state(ca, ca.Lenia(method="fft", precision="Float64"), u), u, 10)
    assert np.max(np.abs(a - b)) < 1e-10
    assert np.max(np.abs(a - u)) > 1e-3


def test_config_2048_float64_within_1e5_after_100_steps(ca, oracle):
    """Lenia on a 2048^2 torus, R = 13, mu = 0.15, sigma = 0.015, dt = 0.1, Uniform[0,1] in the
    central 256^2 patch from seed 4, 100 steps: Float64 FFT within 1e-5 max-abs of the FP64
    oracle, and the Float32 paths' end-state errors reported."""
    n = 2048
    u0 = soup(n, 256, 4, np.float32).astype(np.float64)
    fft = oracle.LeniaFFT(n, n)
    want = u0.copy()
    for _ in range(100):
        want = fft.step(want)
    got = gpu_step(ca, *gpu_state(ca, ca.Lenia(method="fft", precision="Float64"), u0), u0, 100)
    err = np.abs(got - want)
    print(f"Float64 fft after 100 steps: max-abs {err.max():.3e}, L2 {np.sqrt((err ** 2).mean()):.3e}")
    assert err.max() < 1e-5
    for method in ("direct", "fft"):
        g32 = gpu_step(ca, *gpu_state(ca, ca.Lenia(method=method, precision="Float32"), u0.astype(np.float32)),
                       u0.astype(np.float32), 100)
        e = np.abs(g32.astype(np.float64) - want)
        print(f"Float32 {method} after 100 steps: max-abs {e.max():.3e}, L2 {np.sqrt((e ** 2).mean()):.3e}")
        assert np.isfinite(e).all() and g32.min() >= 0 and g32.max() <= 1


@pytest.mark.parametrize("dims", [(360, 150), (250, 96), (135, 75), (112, 98)])
def test_fft_on_mixed_radix_and_other_sides(ca, oracle, dims):
    """The FFT field on sides that are products of 2, 3 and 5 (this library's transforms: 360 =
    2^3 3^2 5, 150 = 2 3 5^2, 250 = 2 5^3, and the odd sides 135 = 3^3 5, 75 = 3 5^2, with no
    Nyquist frequency and a last column pair of one line) and on a side with a factor 7 (98, the
    cuFFT path):
    Float64 steps within 1e-10 of the FP64 oracle's FFT, Float32 steps within the per-step
    tolerance, on a soup that fills the torus."""
    n1, n2 = dims
    rng = np.random.default_rng(n1 * 1000 + n2)
    u = rng.random((n1, n2))
    fft = oracle.LeniaFFT(n1, n2)
    space = ca.Torus(n1, n2)
    g64 = gpu_step(ca, *gpu_state(ca, ca.Lenia(method="fft", precision="Float64"), u, space), u, 3)
    want = u.copy()
    for _ in range(3):
        want = fft.step(want)
    assert np.max(np.abs(g64 - want)) < 1e-10
    u32 = u.astype(np.float32)
    g32 = gpu_step(ca, *gpu_state(ca, ca.Lenia(method="fft", precision="Float32"), u32, space), u32, 1)
    assert np.max(np.abs(g32.astype(np.float64) - fft.step(u32.astype(np.float64)))) < PER_STEP_TOL_F32


@pytest.mark.parametrize("dims", [(1024, 2048), (2048, 512), (4096, 1024), (512, 4096), (1024, 75), (360, 2048)])
def test_fft_power_of_two_sides(ca, oracle, dims):
    """Float32 FFT fields on power-of-two sides of 512 .. 4096 points, which run the transforms
    compiled for their length (a forward transform's outputs straight into the axis-2 product
    and the inverse, the growth straight into the next step's forward transform), also beside
    a mixed-radix side (1024 x 75: an odd number of axis-1 lines, the last complex line half
    empty; 360 x 2048): one step within the per-step tolerance of the FP64 oracle, and three
    steps in one run (each step's last launch also transforming the new state) bit-equal to
    three runs of one step."""
    n1, n2 = dims
    rng = np.random.default_rng(n1 + 7 * n2)
    u = rng.random((n1, n2)).astype(np.float32)
    fft = oracle.LeniaFFT(n1, n2)
    space = ca.Torus(n1, n2)
    rule = ca.Lenia(method="fft", precision="Float32")
    one = gpu_step(ca, *gpu_state(ca, rule, u, space), u, 1)
    assert np.max(np.abs(one.astype(np.float64) - fft.step(u.astype(np.float64)))) < PER_STEP_TOL_F32
    fused = gpu_step(ca, *gpu_state(ca, rule, u, space), u, 3)
    B, prob, st = gpu_state(ca, rule, u, space)
    single = u
    for _ in range(3):
        single = gpu_step(ca, B, prob, st, single, 1)
    assert np.array_equal(fused, single)
    assert 0.0 < float(fused.mean()) < 1.0
