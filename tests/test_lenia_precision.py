"""Why a Float32 Lenia state cannot meet 1e-5 max-abs against the Float64 trajectory after 100
steps of the random-soup configuration (R = 13, mu = 0.15, sigma = 0.015, dt = 0.1,
Uniform[0, 1] in a central 256 x 256 patch from seed 4; src/lenia.jl:42-47): even the best any
Float32-state implementation can do — every step computed exactly in Float64 from the Float32
state and rounded once to Float32, an error of at most 2^-25 per cell per step — leaves the Float64
trajectory past 1e-5 within 20 steps and by O(1) at step 100. The dynamics amplify the rounding,
so the end-state gap is a property of the configuration, not of a kernel.

The lattice is the 512 x 512 torus around the patch: within 100 steps the pattern does not reach
the wrap, and the 2048 x 2048 configuration gives the same errors (measured: 9.4e-6 at step 10,
4.4e-4 at step 20, 1.0 at step 100 on both). The oracle's Float64 FFT field
(ext/CellularAutomataCoreFFTWExt.jl:17-30, within 1e-10 of the direct sum) drives both runs."""
import numpy as np


def soup(n, patch, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    u = np.zeros((n, n), np.float32)
    c = n // 2
    u[c - patch // 2:c + patch // 2, c - patch // 2:c + patch // 2] = rng.random((patch, patch)).astype(np.float32)
    return u


def test_exactly_rounded_float32_state_leaves_the_float64_trajectory(oracle):
    n = 512
    fft = oracle.LeniaFFT(n, n)
    u64 = soup(n, 256, 4).astype(np.float64)
    u32 = u64.astype(np.float32)
    errs = []
    for _ in range(100):
        u64 = fft.step(u64)
        exact = fft.step(u32.astype(np.float64))
        u32 = exact.astype(np.float32)
        assert np.abs(u32 - exact).max() <= 2.0 ** -25  # one rounding per step, nothing else
        errs.append(float(np.abs(u32.astype(np.float64) - u64).max()))
    first = next(t + 1 for t, e in enumerate(errs) if e > 1e-5)
    assert errs[0] < 1e-7          # one step: the rounding alone
    assert first <= 20             # past the 1e-5 target within 20 steps
    assert errs[-1] > 0.1          # O(1) at step 100
    assert max(errs[:5]) < 1e-5 < errs[19]
