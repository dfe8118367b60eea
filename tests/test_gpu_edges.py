"""Edge cases of the sweep on the GPU: degenerate and ragged lattices (1 x 1, single rows and
columns, sides just off the kernels' word and tile sizes), zero-step advances, and a lattice of
more than 2^32 cells, whose cell ids need the Philox counter's high word
(src/random.jl:102-107: ctr = (id % 2^32, id >> 32, t, k))."""
import ctypes
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


SHAPES = [(1, 1), (1, 50), (50, 1), (2, 2), (31, 33), (33, 31), (32, 1), (257, 129), (1025, 3)]


def _pair(ca, o, kind, n1, n2, bnd):
    kinds = {"p": (ca.Periodic(), o.PERIODIC), "r": (ca.Reflecting(), o.REFLECTING), "c": (ca.Constant(0), o.CONSTANT)}
    space = ca.Lattice((n1, n2), (kinds[bnd[0]][0], kinds[bnd[1]][0]))
    ob = (kinds[bnd[0]][1], kinds[bnd[1]][1])
    if kind == "life":
        return ca.Life(":highlife"), space, o.Problem(o.RULE_LIFE, n1, n2, birth=o.mask([3, 6]),
                                                    survive=o.mask([2, 3]), boundary=ob), 2, None
    if kind == "ltl":
        r = ca.Life(list(range(5, 9)), list(range(4, 10)), neighbourhood=ca.Moore(3))
        return r, space, o.Problem(o.RULE_LIFE, n1, n2, radius=3, birth=o.mask(range(5, 9)),
                                   survive=o.mask(range(4, 10)), boundary=ob), 2, None
    if kind == "gen":
        return ca.Generations(":star_wars"), space, o.Problem(o.RULE_GENERATIONS, n1, n2, birth=o.mask([2]),
                                                             survive=o.mask([3, 4, 5]), states=4, boundary=ob), 4, None
    return (ca.ForestFire(), space, o.Problem(o.RULE_FOREST_FIRE, n1, n2, nbhd=o.VON_NEUMANN, boundary=ob, seed=5),
            3, (0.2, 0.01))


@pytest.mark.parametrize("kind", ["life", "ltl", "gen", "fire"])
@pytest.mark.parametrize("shape", SHAPES, ids=[f"{a}x{b}" for a, b in SHAPES])
def test_degenerate_and_ragged_lattices(ca, oracle, kind, shape):
    n1, n2 = shape
    for bnd in ("pp", "rc"):
        rule, space, P, C, params = _pair(ca, oracle, kind, n1, n2, bnd)
        P.seed = 5
        rng = np.random.default_rng(zlib.crc32(f"{kind}{shape}{bnd}".encode()))
        u0 = rng.integers(0, C, (n1, n2)).astype(np.int8)
        pd = None if params is None else {"p": params[0], "f": params[1]}
        prob = ca.CAProblem.new(rule, u0, 13, pd, space=space, seed=5)
        sol = ca.solve(prob, ca.Synchronous(), backend=ca.GB300Backend(), saveat=13)
        want = oracle.run_array(P, u0, 0, 13, params)
        assert np.array_equal(sol.u[-1], want), (kind, shape, bnd)


def test_zero_steps_and_repeated_reads(ca):
    u0 = np.random.default_rng(1).integers(0, 2, (40, 30)).astype(np.int8)
    prob = ca.CAProblem.new(ca.Life(":conway"), u0, 0)
    sol = ca.solve(prob, ca.Synchronous(), backend=ca.GB300Backend())
    assert sol.t == [0] and np.array_equal(sol.u[0], u0)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    capi = ca.capi
    capi.check(capi.lib().gbca_advance(st.handle, 0, 0, None, 0))
    assert np.array_equal(ca.current_state(B, st), u0) and np.array_equal(ca.current_state(B, st), u0)
    st.close()


def test_more_than_2_to_32_cells(ca, oracle):
    """A forest fire on a 65541 x 65539 grid (4.295e9 cells, ids past 2^32): the general
    kernel's 64-bit ids. The state is a device soup; chosen cells and their neighbours are
    read before one step, and each cell's next state is checked against the rule with the
    oracle's draws for its 64-bit id."""
    n1, n2 = 65541, 65539
    assert n1 * n2 > 2 ** 32
    # the problem without a host u0 (4.3 GB): only its shape and element type reach the library
    prob = ca.CAProblem(rule=ca.ForestFire(), u0=np.zeros(0, np.int8), tspan=(0, 1), p={"p": 0.4, "f": 0.3},
                        space=ca.Grid(n1, n2), seed=77, neighbours=ca.VonNeumann(1))
    B = ca.GB300Backend()
    d = ca.backend.make_desc(prob, ca.Synchronous())
    st = ca.GB300State(d, np.int8)
    capi = ca.capi
    # a soup of trees (1) and empty cells (0); then a few fires (2) written near the chosen cells
    capi.check(capi.lib().gbca_set_state_soup(st.handle, 0.6, 12345))
    cells = [(1, 1), (n1, n2), (n1 // 2, n2 - 1), (n1 - 7, n2 - 2), (5, n2), (n1 - 1, 65536), (300, 65535)]
    for i, j in cells[:3]:
        if j + 1 <= n2:
            ca.write_cell(B, st, (i, j + 1), 2)

    def read(i, j):
        if 1 <= i <= n1 and 1 <= j <= n2:
            return int(ca.read_cell(B, st, (i, j)))
        return 0  # Constant(0) edge

    before = {c: (read(*c), [read(c[0] + di, c[1] + dj) for di, dj in ((0, -1), (-1, 0), (1, 0), (0, 1))])
              for c in cells}
    capi.check(capi.lib().gbca_advance(st.handle, 0, 1, (ctypes.c_double * 2)(0.4, 0.3), 2))
    for (i, j), (c, nb) in before.items():
        cid = (i - 1) + (j - 1) * n1 + 1
        if c == 2:
            want = 0
        elif c == 0:
            want = 1 if oracle.uniform(77, cid, 0, 1) < 0.4 else 0
        elif 2 in nb:
            want = 2
        else:
            want = 2 if oracle.uniform(77, cid, 0, 2) < 0.3 else 1
        assert read(i, j) == want, ((i, j), cid, c, nb)
    assert any((i - 1) + (j - 1) * n1 + 1 > 2 ** 32 for i, j in cells)
    st.close()


class _DeviceBytes:
    """A device byte range as a (rows, pitch) int8 array for torch.as_tensor."""

    def __init__(self, ptr, rows, pitch):
        self.__cuda_array_interface__ = {"shape": (rows, pitch), "typestr": "|i1", "data": (ptr, False),
                                         "version": 3, "strides": None, "stream": None}


@pytest.mark.parametrize("kind", ["life", "ltl"])
def test_bit_sliced_past_2_to_32_cells(ca, kind):
    """Life B3/S23 on Moore(1) (3 steps) and Larger than Life
    B34..45/S34..58 on Moore(5) (2 steps) on a 65541 x 65539 torus: 4.295e9 cells, so the
    bit-sliced kernel's column offsets (column x pitch) pass 2^32 bytes and its tiles wrap at
    both far edges. The state is a density-0.5 device soup; the (2 r K + 1)^2 window around each
    chosen cell is read from device memory before the advance (wrapped periodically,
    src/spaces.jl:46-51), stepped by the oracle, and its centre compared with the cell after
    the advance."""
    import torch

    import oracle as o
    o.build()
    n1, n2 = 65541, 65539
    if kind == "life":
        rule, r, nsteps, birth, survive = ca.Life([3], [2, 3]), 1, 3, [3], [2, 3]
    else:
        birth, survive = list(range(34, 46)), list(range(34, 59))
        rule, r, nsteps = ca.Life(birth, survive, neighbourhood=ca.Moore(5)), 5, 2
    prob = ca.CAProblem(rule=rule, u0=np.zeros(0, np.int8), tspan=(0, nsteps), p=None,
                        space=ca.Lattice((n1, n2), (ca.Periodic(), ca.Periodic())), seed=3,
                        neighbours=ca.Moore(r))
    d = ca.backend.make_desc(prob, ca.Synchronous())
    st = ca.GB300State(d, np.int8)
    capi, lib = ca.capi, ca.capi.lib()
    try:
        capi.check(lib.gbca_set_state_soup(st.handle, 0.5, 2024))

        def device_columns():
            ptr, pitch = ctypes.c_void_p(), ctypes.c_int64()
            capi.check(lib.gbca_device_state(st.handle, ctypes.byref(ptr), ctypes.byref(pitch)))
            assert pitch.value >= n1 and pitch.value * n2 > 2 ** 32
            torch.cuda.synchronize()
            return torch.as_tensor(_DeviceBytes(ptr.value, n2, pitch.value), device="cuda")

        cells = [(1, 1), (n1, n2), (n1 // 2, n2 - 1), (n1 - 7, n2 - 2), (5, n2), (n1 - 1, 65536), (300, 65535),
                 (40000, 65538), (n1, 1), (1, n2)]
        R = r * nsteps
        cols = device_columns()
        windows = {}
        for i, j in cells:
            ii = torch.tensor([(i - 1 + a) % n1 for a in range(-R, R + 1)], device="cuda")
            jj = torch.tensor([(j - 1 + a) % n2 for a in range(-R, R + 1)], device="cuda")
            windows[(i, j)] = np.asfortranarray(cols[jj][:, ii].cpu().numpy().T)  # [i, j] like the lattice
        del cols
        capi.check(lib.gbca_advance(st.handle, 0, nsteps, None, 0))
        k, rows, staging = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        capi.check(lib.gbca_geometry(st.handle, None, ctypes.byref(k), ctypes.byref(rows), ctypes.byref(staging)))
        assert k.value >= 1, "the bit-sliced kernel must run this problem"
        cols = device_columns()
        w = 2 * R + 1
        P = o.Problem(o.RULE_LIFE, w, w, radius=r, birth=o.mask(birth), survive=o.mask(survive))
        live = 0
        for (i, j), win in windows.items():
            # the centre of a (2 R + 1)^2 window after R / r steps depends only on the window
            want = int(o.run_array(P, win, 0, nsteps)[R, R])
            got = int(cols[j - 1, i - 1].item())
            assert got == want, ((i, j), (i - 1) + (j - 1) * n1 + 1, got, want)
            live += int(win.sum())
        assert 0.3 < live / (len(cells) * w * w) < 0.7  # the soup is a soup
    finally:
        st.close()


def test_async_state_copies(ca):
    """gbca_set_state_async / gbca_get_state_async from pinned host memory, queued on the
    handle's stream around an advance, give the states the synchronous calls give; a second
    handle's copies and sweep run meanwhile on its own stream."""
    import torch

    capi, lib = ca.capi, ca.capi.lib()
    rng = np.random.default_rng(11)
    states = [(rng.random((300, 200)) < 0.4).astype(np.int8), (rng.random((257, 130)) < 0.5).astype(np.int8)]
    rules = [ca.Life(":highlife"), ca.Life([3], [2, 3])]
    got, want = [], []
    handles = []
    try:
        pins = []
        for u0, rule in zip(states, rules):
            prob = ca.CAProblem.new(rule, u0, 7, space=ca.Torus(*u0.shape))
            d = ca.backend.make_desc(prob, ca.Synchronous())
            h = ctypes.c_void_p()
            capi.check(lib.gbca_create(ctypes.byref(d), ctypes.byref(h)))
            handles.append(h)
            hin = torch.from_numpy(np.asfortranarray(u0).ravel(order="F").copy()).pin_memory()
            hout = torch.empty_like(hin).pin_memory()
            pins.append((hin, hout))
        for h, (hin, hout) in zip(handles, pins):
            capi.check(lib.gbca_set_state_async(h, ctypes.c_void_p(hin.data_ptr()), hin.numel()))
            capi.check(lib.gbca_advance(h, 0, 7, None, 0))
            capi.check(lib.gbca_get_state_async(h, ctypes.c_void_p(hout.data_ptr()), hout.numel()))
        for h, (hin, hout), u0 in zip(handles, pins, states):
            capi.check(lib.gbca_sync(h))
            got.append(hout.numpy().reshape(u0.shape, order="F").copy())
            a = np.asfortranarray(u0)
            capi.check(lib.gbca_set_state(h, a.ctypes.data, a.nbytes))
            capi.check(lib.gbca_advance(h, 0, 7, None, 0))
            w = np.empty_like(a, order="F")
            capi.check(lib.gbca_get_state(h, w.ctypes.data, w.nbytes))
            want.append(w)
        with pytest.raises(ca.errors.StateShapeError):  # a buffer of the wrong size
            capi.check(lib.gbca_get_state_async(handles[0], ctypes.c_void_p(pins[0][1].data_ptr()), 5))
    finally:
        for h in handles:
            lib.gbca_destroy(h)
    for g, w, u0 in zip(got, want, states):
        assert np.array_equal(g, w) and not np.array_equal(w, u0)
