"""Host-side checks that need no GPU: the C-ABI library loads and exports every symbol
include/gbca.h declares; the FP64/FP32 uniform-vs-p compares equal their integer
thresholds; descriptions are checked with the reference's error types; the rule
parser matches the reference's presets; problems validate like src/problem.jl."""
import json
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ca():
    import __graft_entry__ as ge
    ge.build()
    return ge.load_package()


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            with open(os.path.join(ROOT, "include", name)) as f:
                src = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
            syms |= set(re.findall(r"\b(gbca_[a-z0-9_]+)\s*\(", src))
    return syms


def test_library_exports_every_declared_symbol(ca):
    lib = ca.capi.lib()
    syms = declared_symbols()
    assert "gbca_advance" in syms and "gbca_create" in syms
    for s in syms:
        assert hasattr(lib, s), s
    assert set(ca.capi.SIGNATURES) <= syms | {"gbca_last_error"}
    assert lib.gbca_version() >= 100


def declared_parameter_counts():
    """{function: number of parameters} from the prototypes in include/*.h."""
    counts = {}
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            with open(os.path.join(ROOT, "include", name)) as f:
                src = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
            for fn, params in re.findall(r"\b(gbca_[a-z0-9_]+)\s*\(([^;{)]*)\)\s*;", src):
                params = params.strip()
                counts[fn] = 0 if params in ("", "void") else params.count(",") + 1
    return counts


def test_bindings_match_prototypes(ca):
    """Every function the Python binding calls takes as many arguments as include/gbca.h
    declares (a changed prototype without a changed binding would pass garbage through ctypes)."""
    counts = declared_parameter_counts()
    assert len(counts) >= 40
    assert set(counts) == declared_symbols()  # every prototype parsed
    for fn, (_, argtypes) in ca.capi.SIGNATURES.items():
        assert len(argtypes) == counts[fn], (fn, len(argtypes), counts[fn])


def test_thresholds_equal_float_compares(ca, oracle):
    """uniform < p (random.jl:116-120, FP64; :109-114, FP32) <=> x < T for the draw's integer x."""
    rng = np.random.default_rng(7)
    ps = list(rng.random(200)) + [0.0, -0.0, 1.0, 1.5, -2.0, 1e-300, 5e-324, 0.5, 0.03, 1e-4, 2.0 ** -53,
                                  1 - 2.0 ** -53, math.nextafter(0.5, 1), float("nan"), float("inf")]
    for p in ps:
        T = ca.capi.threshold(p, False)
        c = p * 2.0 ** 53
        xs = {0, 1, 2 ** 53 - 1}
        if math.isfinite(c):
            base = int(min(max(math.floor(c), 0), 2 ** 53 - 1))
            xs |= {max(0, min(2 ** 53 - 1, base + d)) for d in range(-3, 4)}
        for x in xs:
            assert (x * 2.0 ** -53 < p) == (x < T), (p, x, T)
        p32 = np.float32(p) if math.isfinite(p) else np.float32(p)
        T32 = ca.capi.threshold(float(p32), True)
        c32 = float(p32) * 2.0 ** 24
        ys = {0, 1, 2 ** 24 - 1}
        if math.isfinite(c32):
            b32 = int(min(max(math.floor(c32), 0), 2 ** 24 - 1))
            ys |= {max(0, min(2 ** 24 - 1, b32 + d)) for d in range(-3, 4)}
        for y in ys:
            assert bool(np.float32(y) * np.float32(2.0 ** -24) < p32) == (y < T32), (p, y, T32)
    # and on real draws from the oracle
    for i in range(1, 400):
        u = oracle.uniform(3, i, 5, 1)
        assert (u < 0.37) == (int(u * 2 ** 53) < ca.capi.threshold(0.37, False))


def desc_for(ca, **kw):
    d = ca.capi.Desc()
    d.rule, d.nbhd, d.radius, d.states, d.n1, d.n2 = ca.capi.RULE_LIFE, ca.capi.MOORE, 1, 2, 8, 8
    d.lenia_R, d.lenia_npeaks, d.lenia_sigma, d.lenia_dt = 13, 1, 0.015, 0.1
    for k, v in kw.items():
        if k in ("boundary", "constant"):
            for a in range(2):
                getattr(d, k)[a] = v[a]
        else:
            setattr(d, k, v)
    return d


def test_check_maps_errors(ca):
    import ctypes
    lib, E = ca.capi.lib(), ca.errors
    ok = desc_for(ca)
    assert lib.gbca_check(ctypes.byref(ok)) == 0
    cases = [
        (dict(n1=0), E.ArgumentError),
        (dict(rule=9), E.ArgumentError),
        (dict(radius=0), E.ArgumentError),
        (dict(nbhd=5), E.ArgumentError),
        (dict(boundary=(2, 2), constant=(300.0, 0.0)), E.IncompatibleSpaceError),
        (dict(boundary=(2, 2), constant=(0.5, 0.0)), E.IncompatibleSpaceError),
        (dict(scheme=7), E.UnsupportedCombinationError),
        (dict(scheme=1, scheme_p=0.0), E.ArgumentError),
        (dict(rule=ca.capi.RULE_GENERATIONS, states=1), E.ArgumentError),
        (dict(rule=ca.capi.RULE_LENIA, lenia_method=ca.capi.FFT, boundary=(2, 0)), E.ArgumentError),
        (dict(rule=ca.capi.RULE_LENIA, lenia_sigma=0.0), E.ArgumentError),
        (dict(rule=ca.capi.RULE_LENIA, scheme=2), E.UnsupportedCombinationError),
    ]
    for kw, exc in cases:
        d = desc_for(ca, **kw)
        with pytest.raises(exc):
            ca.capi.check(lib.gbca_check(ctypes.byref(d)))
        assert lib.gbca_last_error()  # a message came with it


def test_rule_parsing_matches_presets(ca):
    """src/rules.jl:249-265,316-330; test/test_rules.jl:89-106."""
    with open(os.path.join(ROOT, "tests", "golden", "rule_strings.json")) as f:
        presets = json.load(f)
    assert presets["life"] == ca.LIFE_PRESETS and presets["generations"] == ca.GENERATIONS_PRESETS
    for name, s in presets["life"].items():
        assert ca.Life(name).rulestring() == s
    for name, s in presets["generations"].items():
        assert ca.Generations(name).rulestring() == s
    assert ca.Life("23/36").rulestring() == "B36/S23"
    assert ca.Life("b3s23").rulestring() == "B3/S23"
    assert ca.Generations("345/2/4").rulestring() == "B2/S345/C4"
    assert ca.Generations("B2/S/3").rulestring() == "B2/S/C3"
    assert ca.Life(range(34, 46), range(34, 59)).rulestring() == "B34..45/S34..58"
    for bad in ("B9/S23", "hello", "B3/S23/C3"):
        with pytest.raises(ca.RuleParseError):
            ca.Life(bad)
    with pytest.raises(ca.RuleParseError):
        ca.Generations("B3/S23")
    with pytest.raises(ca.ArgumentError):
        ca.Life([64], [2])
    with pytest.raises(ca.ArgumentError):
        ca.Life(":nonsense")


def test_problem_validation(ca):
    u = np.zeros((8, 8), np.int8)
    with pytest.raises(ca.InvalidStateError):
        ca.CAProblem.new(ca.Life(), np.full((8, 8), 2, np.int8), 1)
    with pytest.raises(ca.StateShapeError):
        ca.CAProblem.new(ca.Life(), u, 1, space=ca.Torus(8, 9))
    with pytest.raises(ca.ArgumentError):
        ca.CAProblem.new(ca.Life(), u, (5, 1))
    with pytest.raises(ca.IncompatibleSpaceError):
        ca.CAProblem.new(ca.Life(), u, 1, space=ca.Grid(8, 8, boundary=ca.Constant(500)))
    with pytest.raises(ca.InvalidStateError):
        ca.CAProblem.new(ca.Generations("brians_brain"), np.full((8, 8), 3, np.int8), 1)
    p = ca.CAProblem.new(ca.Life(), u, 10, seed=1)
    assert [ca.seed_trajectory(p, i).seed for i in range(1, 5)] == [2, 3, 4, 5]  # test_sciml.jl:118
    assert ca.neighbourhood_offsets(ca.VonNeumann(1)) == [(0, -1), (-1, 0), (1, 0), (0, 1)]
    assert len(ca.neighbourhood_offsets(ca.Moore(5))) == 120
    # the backend refuses what it cannot run, with the reference's error types
    B = ca.GB300Backend()
    assert ca.supports(B, ca.Synchronous()) and ca.supports(B, ca.Stochastic(0.5)) and ca.supports(B, ca.Checkerboard())
    with pytest.raises(ca.ArgumentError):
        ca.check_problem(B, ca.CAProblem.new(ca.Life(), np.zeros((8, 8), np.int32), 1), ca.Synchronous())
    with pytest.raises(ca.ArgumentError):  # a Float32 rule on a Float64 state
        ca.check_problem(B, ca.CAProblem.new(ca.Lenia(precision="Float32"), np.zeros((8, 8)), 1), ca.Synchronous())
    with pytest.raises(ca.ArgumentError):
        ca.check_problem(B, ca.CAProblem.new(ca.Lenia(method="fft", precision="Float32"), np.zeros((8, 8), np.float32), 1,
                                             space=ca.Grid(8, 8)), ca.Synchronous())


def test_no_device_fails_loudly(ca):
    """Without a visible GPU the library refuses to create a handle (a CUDA error naming the
    missing device) instead of running anywhere else, and the no-alloc entry point refuses a
    sweep it cannot run; its argument checks come first and touch no memory."""
    import ctypes
    lib = ca.capi.lib()
    if lib.gbca_device_count() > 0:
        pytest.skip("a GPU is visible: the refusal applies to machines without one")
    h = ctypes.c_void_p()
    rc = lib.gbca_create(ctypes.byref(desc_for(ca)), ctypes.byref(h))
    assert rc == ca.capi.ERR_CUDA and not h.value
    assert "device" in lib.gbca_last_error().decode()
    buf = np.zeros(8 * 1024 + 64, np.int8)
    addr = buf.ctypes.data + (-buf.ctypes.data) % 16  # a 16-byte aligned host address, never written
    big = desc_for(ca, n1=4096, n2=4097)  # one column more than the scratch array holds
    with pytest.raises(ca.ArgumentError, match="scratch"):
        ca.capi.check(lib.gbca_advance_noalloc(ctypes.byref(big), ctypes.c_void_p(addr), 4096, 0, 1, None, 0, None))
    with pytest.raises(ca.ArgumentError, match="aligned"):
        ca.capi.check(lib.gbca_advance_noalloc(ctypes.byref(desc_for(ca)), ctypes.c_void_p(addr + 1), 16, 0, 1, None,
                                               0, None))
    with pytest.raises(ca.ArgumentError):
        ca.capi.check(lib.gbca_advance_noalloc(ctypes.byref(desc_for(ca)), ctypes.c_void_p(addr), 4, 0, 1, None, 0,
                                               None))  # pitch below n1
    with pytest.raises(ca.UnsupportedCombinationError):
        ca.capi.check(lib.gbca_advance_noalloc(ctypes.byref(desc_for(ca, rule=ca.capi.RULE_LENIA)),
                                               ctypes.c_void_p(addr), 32, 0, 1, None, 0, None))
    assert lib.gbca_advance_noalloc(ctypes.byref(desc_for(ca)), ctypes.c_void_p(addr), 16, 0, 0, None, 0,
                                    None) == ca.capi.OK  # zero steps: nothing to run
    rc = lib.gbca_advance_noalloc(ctypes.byref(desc_for(ca)), ctypes.c_void_p(addr), 16, 0, 1, None, 0, None)
    assert rc == ca.capi.ERR_CUDA and not buf.any()
    # the reference-facing call raises too
    prob = ca.CAProblem.new(ca.Life(), np.zeros((8, 8), np.int8), 2)
    with pytest.raises(ca.errors.GPUError, match="no CUDA device"):
        ca.solve(prob, backend=ca.GB300Backend())
