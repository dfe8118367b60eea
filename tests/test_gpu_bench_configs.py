"""The benchmarked workloads, checked against the oracle at their full size and with the tile
geometries the autotuner can pick for them: a tile-count or index error that shows only with
thousands of tiles, or with lattices of 2^26 and 2^28 cells, would be caught here.

* Larger than Life, Moore(5), B34..45/S34..58 on the 8192 x 8192 torus from the bench's own
  density-0.5 soup (src/rules.jl:385-389): 10 steps, which is one 6-step pass and one 4-step
  pass at the bench's pick (6 steps, 216-row tiles), under several pinned geometries and the
  untuned default.
* The forest fire (README.md:56-60) on the 16384 x 16384 Grid with Constant(0) edges, p = 0.03,
  f = 1e-4, seed 3: 3 steps from the bench's all-empty start, then 2 steps from a mixed state
  (40% empty, 59% trees, 1% fire), under the bench's pick (1 step per pass, TMA-staged tiles of
  the launcher's 158 rows), the persistent prefetching kernel, deeper TMA passes and vector
  loads.

Every result must equal the oracle's (the reference's ArrayBackend slab sweep,
src/backends.jl:457-479, restated in C and run on all host cores) bit for bit."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NCPU = os.cpu_count() or 1


@pytest.fixture(scope="module")
def env():
    import __graft_entry__ as ge
    ge.build()
    ca = ge.load_package()
    if ca.capi.lib().gbca_device_count() < 1:
        pytest.fail("no CUDA device visible")
    import bench
    import oracle as o
    o.build()
    return ca, bench, o


def run_pinned(ca, d, u0, t0, nsteps, geometry, params=None):
    """gbca_create / set_state / set_geometry / advance / get_state; geometry None keeps the
    kernel's default (nothing tuned or pinned)."""
    capi, lib = ca.capi, ca.capi.lib()
    lib.gbca_forget_tuning()
    h = ctypes.c_void_p()
    capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(h)))
    try:
        a = np.asfortranarray(u0, dtype=np.int8)
        capi.check(lib.gbca_set_state(h, a.ctypes.data, a.nbytes))
        if geometry is not None:
            capi.check(lib.gbca_set_geometry(h, *geometry))
        arr = (ctypes.c_double * 2)(*params) if params else None
        capi.check(lib.gbca_advance(h, t0, nsteps, arr, 2 if params else 0))
        got = np.empty_like(a, order="F")
        capi.check(lib.gbca_get_state(h, got.ctypes.data, got.nbytes))
        k, rows, staging = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        capi.check(lib.gbca_geometry(h, arr, ctypes.byref(k), ctypes.byref(rows), ctypes.byref(staging)))
        return got, (k.value, rows.value, staging.value)
    finally:
        lib.gbca_destroy(h)


@pytest.fixture(scope="module")
def ltl_case(env):
    ca, bench, o = env
    ltl0, _ = bench.initial_states()
    d1, _ = bench.descs(ca.capi)
    L = bench.LTL
    P = o.Problem(o.RULE_LIFE, L["n1"], L["n2"], radius=5, birth=o.mask(range(34, 46)), survive=o.mask(range(34, 59)),
                  seed=2)
    want = o.run_array(P, ltl0, 0, 10, None, NCPU)
    return ltl0, d1, want


@pytest.mark.parametrize("geometry", [(6, 216, 0), (5, 176, 0), (4, 128, 0), (3, 64, 0), None],
                         ids=["6x216 (bench)", "5x176", "4x128", "3x64", "default"])
def test_ltl_8192_torus_full_size(env, ltl_case, geometry):
    ca, bench, o = env
    ltl0, d1, want = ltl_case
    got, used = run_pinned(ca, d1, ltl0, 0, 10, geometry)
    if geometry is not None:
        assert used == geometry
    assert used[0] >= 1, "the bit-sliced kernel must run this problem"
    bad = int((got != want).sum())
    assert bad == 0, f"{bad} of {got.size} cells differ from the oracle after 10 steps (geometry {used})"
    # the soup is still alive and has moved: the comparison means something
    assert 0.01 < want.mean() < 0.9 and (want != ltl0).mean() > 0.05


@pytest.fixture(scope="module")
def fire_case(env):
    ca, bench, o = env
    _, fire0 = bench.initial_states()
    _, d2 = bench.descs(ca.capi)
    F = bench.FIRE
    P = o.Problem(o.RULE_FOREST_FIRE, F["n1"], F["n2"], nbhd=o.VON_NEUMANN, seed=F["seed"],
                  boundary=(o.CONSTANT, o.CONSTANT))
    params = (F["p"], F["f"])
    from_empty = o.run_array(P, fire0, 0, 3, params, NCPU)
    rng = np.random.Generator(np.random.PCG64(3))
    pct = rng.integers(0, 100, size=(F["n2"], F["n1"]), dtype=np.int8).T
    mixed = np.asfortranarray((pct >= 40).astype(np.int8) + (pct >= 99).astype(np.int8))
    from_mixed = o.run_array(P, mixed, 100, 2, params, NCPU)
    return d2, params, fire0, from_empty, mixed, from_mixed


@pytest.mark.parametrize("geometry", [(1, 0, 1), (1, 0, 2), (1, 158, 0), (4, 0, 1), (8, 0, 0)],
                         ids=["1 step, TMA (bench)", "1 step, persistent TMA", "1 step, vector loads",
                              "4 steps, TMA", "8 steps, vector loads"])
def test_fire_16384_grid_full_size(env, fire_case, geometry):
    ca, bench, o = env
    d2, params, fire0, from_empty, mixed, from_mixed = fire_case
    got, used = run_pinned(ca, d2, fire0, 0, 3, geometry, params)
    assert used[0] == geometry[0] and used[2] == geometry[2]
    bad = int((got != from_empty).sum())
    assert bad == 0, f"{bad} cells differ from the oracle after 3 steps from empty (geometry {used})"
    assert (from_empty == 1).sum() > 0.05 * from_empty.size  # trees have grown
    got, used = run_pinned(ca, d2, mixed, 100, 2, geometry, params)
    bad = int((got != from_mixed).sum())
    assert bad == 0, f"{bad} cells differ from the oracle after 2 steps from the mixed state (geometry {used})"
    assert (from_mixed == 2).sum() > 0  # fires burn
