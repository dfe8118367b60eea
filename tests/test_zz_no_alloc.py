"""gbca_advance_noalloc, the sweep for callers that cannot allocate device memory when they
need it (a device owned by a memory pool, a real-time loop, a plug-in host that forbids
allocation after start-up). Through the C ABI, two calls in a row on a state held in the
caller's own device buffer must give exactly what the allocating entry points
(gbca_create / gbca_set_state / gbca_advance / gbca_get_state) give for the same steps, and
what the oracle gives; Int8 results are compared bit for bit, the tolerance of every Int8
parity test here. The cases reach every branch of the sweep dispatch the entry point uses:
the forest-fire kernel (plain and gated), the bit-sliced kernel, and the general kernel
(Generations with more than eight states, a pitch that is not a multiple of 16, Checkerboard
Life on an unscanned state), plus a state of exactly the scratch array's size. Oversized and
misaligned states are refused. The file sorts last so that a run stopping at its first
failure has run every other test first; it also passes alone in a fresh process."""
import ctypes
import os

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
    import oracle as o
    o.build()
    return ca, torch, o


def desc_of(ca, prob, scheme):
    return ca.backend.make_desc(prob, scheme)


def oracle_problem(o, d):
    """The oracle's description of the same problem, field by field from the gbca_desc."""
    return o.Problem(int(d.rule), int(d.n1), int(d.n2), nbhd=int(d.nbhd), radius=int(d.radius), birth=int(d.birth),
                     survive=int(d.survive), states=int(d.states), boundary=(int(d.boundary[0]), int(d.boundary[1])),
                     constant=(int(d.constant[0]), int(d.constant[1])), seed=int(d.seed), scheme=int(d.scheme),
                     scheme_p=float(d.scheme_p), scheme_p_f32=bool(d.scheme_p_f32), params_f32=bool(d.params_f32))


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
    # name, rule, lattice, scheme, params, steps per call, pitch (None: n1 rounded up to 16)
    ("forest fire, Grid", lambda ca: ca.ForestFire(), lambda ca: ca.Grid(300, 200), "sync", (0.05, 0.001), 13, None),
    ("forest fire, Stochastic(0.7) gate", lambda ca: ca.ForestFire(), lambda ca: ca.Grid(128, 96), "stoch07",
     (0.05, 0.001), 5, None),
    ("Larger than Life Moore(5), torus", lambda ca: ca.Life(range(34, 46), range(34, 59), neighbourhood=ca.Moore(5)),
     lambda ca: ca.Torus(257, 190), "sync", None, 9, None),
    ("Brian's Brain, Stochastic(0.6)", lambda ca: ca.Generations(":brians_brain"), lambda ca: ca.Torus(64, 80),
     "stoch", None, 7, None),
    ("Life, Checkerboard, odd steps", lambda ca: ca.Life(), lambda ca: ca.Torus(96, 64), "check", None, 7, None),
    ("Life, pitch not a multiple of 16", lambda ca: ca.Life(), lambda ca: ca.Torus(100, 70), "sync", None, 6, 100),
    ("Generations C = 10, reflecting", lambda ca: ca.Generations("B2/S34/C10"),
     lambda ca: ca.Lattice((70, 50), (ca.Reflecting(), ca.Reflecting())), "sync", None, 5, None),
]


def run_case(ca, torch, o, rule, space, scheme, params, nsteps, pitch):
    n1, n2 = space.dims
    rng = np.random.default_rng(11)
    C = rule.states if isinstance(rule, ca.Generations) else (3 if isinstance(rule, ca.ForestFire) else 2)
    u0 = rng.integers(0, C, (n1, n2)).astype(np.int8)
    pd = None if params is None else {"p": params[0], "f": params[1]}
    prob = ca.CAProblem.new(rule, u0, 2 * nsteps, pd, space=space, seed=5)
    d = desc_of(ca, prob, scheme)
    P = oracle_problem(o, d)
    lib = ca.capi.lib()

    pitch = pitch or (n1 + 15) // 16 * 16
    buf = torch.zeros(n2 * pitch + 16, dtype=torch.int8, device="cuda")  # the caller's own buffer
    dev = buf[:n2 * pitch].view(n2, pitch)
    dev[:, :n1] = torch.from_numpy(np.ascontiguousarray(u0.T)).cuda()
    arr = (ctypes.c_double * 2)(*(params or (0.0, 0.0)))
    stream = torch.cuda.current_stream()
    want = u0
    ncpu = os.cpu_count() or 1
    for call in range(2):  # two calls in a row, the second continuing from the first
        t = call * nsteps
        rc = lib.gbca_advance_noalloc(ctypes.byref(d), ctypes.c_void_p(dev.data_ptr()), pitch, t, nsteps, arr,
                                      2 if params else 0, ctypes.c_void_p(stream.cuda_stream))
        ca.capi.check(rc)
        torch.cuda.synchronize()
        got = dev[:, :n1].cpu().numpy().T
        by_oracle = o.run_array(P, want, t, nsteps, params, ncpu)
        want = advance_with_handle(ca, d, want, t, nsteps, params)
        assert np.array_equal(want, by_oracle), f"call {call + 1}: the allocating path differs from the oracle"
        assert np.array_equal(got, want), f"call {call + 1} differs in {(got != want).sum()} cells"
    assert not np.array_equal(want, u0)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_allocating_path_twice(env, case):
    ca, torch, o = env
    name, rule_f, space_f, scheme_name, params, nsteps, pitch = case
    scheme = {"sync": ca.Synchronous(), "stoch": ca.Stochastic(0.6), "stoch07": ca.Stochastic(0.7),
              "check": ca.Checkerboard()}[scheme_name]
    run_case(ca, torch, o, rule_f(ca), space_f(ca), scheme, params, nsteps, pitch)


def test_noalloc_state_of_exactly_the_scratch_size(env):
    """A 4096 x 4096 state at pitch 4096 fills the 16 MiB scratch array to the byte."""
    ca, torch, o = env
    assert 4096 * 4096 == ca.capi.NOALLOC_SCRATCH_BYTES
    run_case(ca, torch, o, ca.Life(), ca.Torus(4096, 4096), ca.Synchronous(), None, 5, 4096)


def test_noalloc_refuses_what_it_cannot_hold(env):
    ca, torch, o = env
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
