"""gbca_advance_noalloc, the sweep for callers that cannot allocate device memory when they
need it (a device owned by a memory pool, a real-time loop, a plug-in host that forbids
allocation after start-up). Through the C ABI, two calls in a row on a state held in the
caller's own device buffer must give exactly what the allocating entry points
(gbca_create / gbca_set_state / gbca_advance / gbca_get_state) give for the same steps; Int8
results are compared bit for bit, the tolerance of every Int8 parity test here. Oversized
and misaligned states are refused. The file sorts last so that a run stopping at its first
failure has run every other test first; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import __graft_entry__ as ge
    ge.build()
    ca = ge.load_package()
    if ca.capi.lib().gbca_device_count() < 1 or not torch.cuda.is_available():
        pytest.fail("no CUDA device visible")
    return ca, torch


def desc_of(ca, prob, scheme):
    return ca.backend.make_desc(prob, scheme)


def advance_with_handle(ca, d, u, t, nsteps, params):
    """The allocating path: a handle, host state in and out."""
    lib, capi = ca.capi.lib(), ca.capi
    h = ctypes.c_void_p()
    capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(h)))
    a = np.asfortranarray(u.astype(np.int8))
    capi.check(lib.gbca_set_state(h, a.ctypes.data, a.nbytes))
    arr = (ctypes.c_double * 2)(*(params or (0.0, 0.0)))
    capi.check(lib.gbca_advance(h, t, nsteps, arr, 2 if params else 0))
    out = np.empty_like(a, order="F")
    capi.check(lib.gbca_get_state(h, out.ctypes.data, out.nbytes))
    lib.gbca_destroy(h)
    return out


CASES = [
    # rule, lattice, scheme, params, steps per call
    ("forest fire, Grid", lambda ca: ca.ForestFire(), lambda ca: ca.Grid(300, 200), "sync", (0.05, 0.001), 13),
    ("Larger than Life Moore(5), torus", lambda ca: ca.Life(range(34, 46), range(34, 59), neighbourhood=ca.Moore(5)),
     lambda ca: ca.Torus(257, 190), "sync", None, 9),
    ("Brian's Brain, Stochastic(0.6)", lambda ca: ca.Generations(":brians_brain"), lambda ca: ca.Torus(64, 80),
     "stoch", None, 7),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_allocating_path_twice(env, case):
    ca, torch = env
    name, rule_f, space_f, scheme_name, params, nsteps = case
    rule, space = rule_f(ca), space_f(ca)
    scheme = ca.Stochastic(0.6) if scheme_name == "stoch" else ca.Synchronous()
    n1, n2 = space.dims
    rng = np.random.default_rng(11)
    C = 3 if isinstance(rule, (ca.ForestFire, ca.Generations)) else 2
    u0 = rng.integers(0, C, (n1, n2)).astype(np.int8)
    pd = None if params is None else {"p": params[0], "f": params[1]}
    prob = ca.CAProblem.new(rule, u0, 2 * nsteps, pd, space=space, seed=5)
    d = desc_of(ca, prob, scheme)
    lib = ca.capi.lib()

    pitch = (n1 + 15) // 16 * 16
    dev = torch.zeros((n2, pitch), dtype=torch.int8, device="cuda")  # the caller's own buffer
    dev[:, :n1] = torch.from_numpy(np.ascontiguousarray(u0.T)).cuda()
    arr = (ctypes.c_double * 2)(*(params or (0.0, 0.0)))
    stream = torch.cuda.current_stream()
    want = u0
    for call in range(2):  # two calls in a row, the second continuing from the first
        t = call * nsteps
        rc = lib.gbca_advance_noalloc(ctypes.byref(d), ctypes.c_void_p(dev.data_ptr()), pitch, t, nsteps, arr,
                                      2 if params else 0, ctypes.c_void_p(stream.cuda_stream))
        ca.capi.check(rc)
        torch.cuda.synchronize()
        got = dev[:, :n1].cpu().numpy().T
        want = advance_with_handle(ca, d, want, t, nsteps, params)
        assert np.array_equal(got, want), f"{name}: call {call + 1} differs in {(got != want).sum()} cells"
    assert not np.array_equal(want, u0)


def test_noalloc_refuses_what_it_cannot_hold(env):
    ca, torch = env
    lib = ca.capi.lib()
    prob = ca.CAProblem.new(ca.Life(), np.zeros((8, 8), np.int8), 1)
    big = desc_of(ca, prob, ca.Synchronous())
    big.n1, big.n2 = 4096, 4097  # one column more than the scratch array holds
    dev = torch.zeros(64, dtype=torch.int8, device="cuda")
    with pytest.raises(ca.ArgumentError, match="scratch"):
        ca.capi.check(lib.gbca_advance_noalloc(ctypes.byref(big), ctypes.c_void_p(dev.data_ptr()), 4096, 0, 1, None,
                                               0, None))
    small = desc_of(ca, prob, ca.Synchronous())
    with pytest.raises(ca.ArgumentError, match="aligned"):
        ca.capi.check(lib.gbca_advance_noalloc(ctypes.byref(small), ctypes.c_void_p(dev.data_ptr() + 1), 16, 0, 1,
                                               None, 0, None))
    lenia = desc_of(ca, ca.CAProblem.new(ca.Lenia(precision="Float32"), np.zeros((8, 8), np.float32), 1),
                    ca.Synchronous())
    with pytest.raises(ca.UnsupportedCombinationError):
        ca.capi.check(lib.gbca_advance_noalloc(ctypes.byref(lenia), ctypes.c_void_p(dev.data_ptr()), 32, 0, 1, None,
                                               0, None))
    assert ca.capi.NOALLOC_SCRATCH_BYTES == 16 * 1024 * 1024
