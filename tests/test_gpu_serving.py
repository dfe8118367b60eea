"""Serving with continuous batching: every request's result (state counts and Moran's I,
src/measures.jl) is the same alone and in a mix of rules, sizes, step counts, small and large
requests, staggered arrivals and an HBM budget that makes requests wait for admission; and
equal to the single-handle path for requests given an explicit initial state."""
import time

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


def mixed_requests(ca, n=40, seed=3):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        side = int(np.round(np.exp(rng.uniform(np.log(16), np.log(700)))))
        steps = int(rng.integers(10, 90))
        kind = i % 3
        if kind == 0:
            rule, space, p = ca.Life("B3/S23"), ca.Torus(side, side), None
        elif kind == 1:
            rule, space, p = ca.Generations(":brians_brain"), ca.Torus(side, side), None
        else:
            rule, space = ca.ForestFire(), ca.Grid(side, side)
            p = {"p": float(rng.uniform(0.01, 0.1)), "f": float(np.exp(rng.uniform(np.log(1e-5), np.log(1e-3))))}
        explicit = i % 2 == 0
        C = 2 if kind == 0 else 3
        u0 = rng.integers(0, C, (side, side)).astype(np.int8) if explicit else np.zeros((side, side), np.int8)
        prob = ca.CAProblem.new(rule, u0, steps, p, space=space, seed=1000 + i)
        reqs.append((prob, None if explicit else 0.4, 77 + i))
    return reqs


def key(r):
    return (tuple(r["counts"]), r["other"], None if np.isnan(r["morans"]) else r["morans"], r["status"])


def test_same_alone_and_in_the_mix(ca):
    reqs = mixed_requests(ca)
    # the mix: a small budget (forces admission waits), small chunks (large requests too: a 1 us
    # chunk target leaves chunk_steps steps per chunk, so they interleave and resume), a low
    # large-request threshold
    with ca.serving.Server(hbm_budget=6 << 20, chunk_steps=16, big_cells=40000, max_big=3, big_chunk_us=1) as srv:
        ids = []
        for k, (prob, dens, s) in enumerate(reqs):
            ids.append(srv.submit(prob, density=dens, init_seed=s))
            if k % 7 == 3:
                time.sleep(0.003)  # staggered arrivals join running iterations
        mix = srv.wait(ids)
        occ = srv.stats()
    assert all(mix[i]["status"] == 0 for i in ids)
    big = [p for p, _, _ in reqs if p.space.dims[0] * p.space.dims[1] > 40000]
    assert occ["chunks"] > len(big) > 0  # large requests ran in several chunks each
    assert len(occ["lane_busy_s"]) == 3 and all(0.0 <= b <= occ["wall_s"] for b in occ["lane_busy_s"])
    # each request alone in its own server
    for (prob, dens, s), i in zip(reqs, ids):
        with ca.serving.Server(hbm_budget=8 << 20, chunk_steps=1000, big_cells=40000, max_big=1) as one:
            j = one.submit(prob, density=dens, init_seed=s)
            alone = one.wait([j])[j]
        assert key(alone) == key(mix[i]), (prob.rule, prob.space.dims)
    # and the single-handle path for requests with an explicit initial state
    B = ca.GB300Backend()
    for (prob, dens, s), i in list(zip(reqs, ids))[::2]:
        st = ca.allocate_state(B, prob, ca.Synchronous())
        for t in range(prob.tspan[1]):
            ca.advance(B, st, prob, ca.Synchronous(), prob.p, t)
        counts, other, mi = ca.device_summaries(st, 8)
        st.close()
        assert mix[i]["counts"] == counts and mix[i]["other"] == other
        assert (mix[i]["morans"] == mi) or (np.isnan(mi) and np.isnan(mix[i]["morans"]))


def test_oversized_request_is_refused(ca):
    with ca.serving.Server(hbm_budget=1 << 20, chunk_steps=8) as srv:
        big = ca.CAProblem.new(ca.Life(), np.zeros((1024, 1024), np.int8), 5)
        small = ca.CAProblem.new(ca.Life(), np.zeros((64, 64), np.int8), 5)
        i, j = srv.submit(big), srv.submit(small)
        got = srv.wait([i, j])
    assert got[i]["status"] == ca.capi.ERR_OOM and got[j]["status"] == 0
    assert got[j]["counts"][0] == 64 * 64


def test_served_mix_against_the_oracle(ca, oracle):
    """Twelve requests of the served stream's three rules (Life B3/S23 and Generations B2/S/C3
    from the server's device soups, the forest fire from empty, p ~ U(0.01, 0.1),
    f ~ LogU(1e-5, 1e-3)), sides log-uniform in 64..1024 and 50..400 steps, submitted together
    to a server with the bench's configuration: each result's state counts equal the oracle's
    and its Moran's I agrees to 1e-12 (src/measures.jl:14-20,91-107), the oracle running the
    same soup (seed; id, 0, 0xFFFFFFFF, 0xFFFFFFFE) through the reference's ArrayBackend sweep."""
    import os

    o = oracle
    rng = np.random.Generator(np.random.PCG64(1212))
    reqs, want = [], []
    for k in range(12):
        kind = k % 3
        side = int(np.round(np.exp(rng.uniform(np.log(64), np.log(1024)))))
        steps = int(rng.integers(50, 401))
        seed, init_seed = int(rng.integers(1, 2 ** 62)), int(rng.integers(1, 2 ** 62))
        if kind == 0:
            rule, space, p, dens = ca.Life("B3/S23"), ca.Torus(side, side), None, 0.5
            P = o.Problem(o.RULE_LIFE, side, side, birth=o.mask([3]), survive=o.mask([2, 3]), seed=seed)
        elif kind == 1:
            rule, space, p, dens = ca.Generations("B2/S/C3"), ca.Torus(side, side), None, 0.5
            P = o.Problem(o.RULE_GENERATIONS, side, side, birth=o.mask([2]), survive=0, states=3, seed=seed)
        else:
            rule, space, dens = ca.ForestFire(), ca.Grid(side, side), None
            p = {"p": float(rng.uniform(0.01, 0.1)), "f": float(np.exp(rng.uniform(np.log(1e-5), np.log(1e-3))))}
            P = o.Problem(o.RULE_FOREST_FIRE, side, side, nbhd=o.VON_NEUMANN, seed=seed,
                          boundary=(o.CONSTANT, o.CONSTANT))
        prob = ca.CAProblem.new(rule, np.zeros((side, side), np.int8), steps, p, space=space, seed=seed)
        reqs.append((prob, dens, init_seed))
        u0 = o.soup(init_seed, side, side, dens) if dens else np.zeros((side, side), np.int8)
        u = o.run_array(P, u0, 0, steps, (p["p"], p["f"]) if p else None, os.cpu_count() or 1)
        want.append((o.state_counts(u, 8), o.morans_i(P, u)))
    with ca.serving.Server(hbm_budget=8 << 30, chunk_steps=100, big_cells=1 << 16, max_big=16) as srv:
        ids = [srv.submit(prob, density=dens, init_seed=s) for prob, dens, s in reqs]
        got = srv.wait(ids)
    for (prob, dens, s), i, ((counts, other), mi) in zip(reqs, ids, want):
        r = got[i]
        assert r["status"] == 0
        assert r["counts"] == counts and r["other"] == other, (prob.rule, prob.space.dims)
        if np.isnan(mi):
            assert np.isnan(r["morans"])
        else:
            assert r["morans"] == pytest.approx(mi, rel=1e-12, abs=1e-15), (prob.rule, prob.space.dims)
