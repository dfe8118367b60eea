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
    # the mix: a small budget (forces admission waits), small chunks, a low large-request threshold
    with ca.serving.Server(hbm_budget=6 << 20, chunk_steps=16, big_cells=40000, max_big=3) as srv:
        ids = []
        for k, (prob, dens, s) in enumerate(reqs):
            ids.append(srv.submit(prob, density=dens, init_seed=s))
            if k % 7 == 3:
                time.sleep(0.003)  # staggered arrivals join running iterations
        mix = srv.wait(ids)
    assert all(mix[i]["status"] == 0 for i in ids)
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
