"""The device-side save path: gbca_snapshot stages a state on the device and copies it out on
a second stream while the sweep goes on. Saved states equal the oracle's; tickets can be
fetched in any order; the integrator's saves (which use the path) keep the reference's
save times and states, also with callbacks that read and change integ.u."""
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


def test_snapshots_in_any_order(ca, oracle):
    u0 = np.random.default_rng(5).integers(0, 2, (300, 200)).astype(np.int8)
    prob = ca.CAProblem.new(ca.Life(":highlife"), u0, 60)
    B = ca.GB300Backend()
    st = ca.allocate_state(B, prob, ca.Synchronous())
    tickets = []
    for t in range(60):
        if t % 10 == 0:
            tickets.append((t, ca.backend.snapshot(st)))
        ca.advance(B, st, prob, ca.Synchronous(), None, t)
    tickets.append((60, ca.backend.snapshot(st)))
    P = oracle.Problem(oracle.RULE_LIFE, 300, 200, birth=oracle.mask([3, 6]), survive=oracle.mask([2, 3]))
    want = {0: u0}
    u = u0
    for t in range(0, 60, 10):
        u = oracle.run_array(P, u, t, 10, nthreads=8)
        want[t + 10] = u
    for t, k in reversed(tickets):
        assert np.array_equal(ca.backend.snapshot_fetch(st, k), want[t]), t
    with pytest.raises(ca.ArgumentError):
        ca.backend.snapshot_fetch(st, tickets[0][1])  # already fetched
    st.close()


def test_snapshot_limit(ca):
    prob = ca.CAProblem.new(ca.Life(":conway"), np.zeros((16, 16), np.int8), 1)
    st = ca.allocate_state(ca.GB300Backend(), prob, ca.Synchronous())
    ks = [ca.backend.snapshot(st) for _ in range(64)]
    with pytest.raises(ca.errors.Busy):
        ca.backend.snapshot(st)
    for k in ks:
        ca.backend.snapshot_fetch(st, k)
    ca.backend.snapshot_fetch(st, ca.backend.snapshot(st))
    st.close()


def test_save_everystep_and_callbacks(ca, oracle):
    """Every step saved (201 saves through the device path), and a run whose callback reads
    integ.u at every step and changes it at t = 7."""
    u0 = np.random.default_rng(6).integers(0, 3, (64, 48)).astype(np.int8)
    prob = ca.CAProblem.new(ca.Generations(":brians_brain"), u0, 200)
    sol = ca.solve(prob, ca.Synchronous(), backend=ca.GB300Backend())
    P = oracle.Problem(oracle.RULE_GENERATIONS, 64, 48, birth=oracle.mask([2]), survive=0, states=3)
    ts, us = oracle.solve(P, u0, 200, nthreads=4)
    assert sol.t == ts and all(np.array_equal(a, b) for a, b in zip(sol.u, us))

    def affect(integ):
        u = integ.u.copy()
        u[0:5, 0:5] = 1
        integ.u = u

    cb = ca.DiscreteCallback(lambda u, t, integ: t == 7, affect)
    sol = ca.solve(prob.remake(tspan=20), ca.Synchronous(), backend=ca.GB300Backend(), saveat=5, callback=cb)
    u = u0
    u = oracle.run_array(P, u, 0, 7)
    u[0:5, 0:5] = 1
    u = oracle.run_array(P, u, 7, 13)
    assert sol.t == [0, 5, 10, 15, 20] and np.array_equal(sol.u[-1], u)


def test_bounded_wait_reports_timeout(ca):
    """The failure path of the device-side waits, without a fault: a kernel waits (at most
    256 polls) on a barrier nothing completes; the host reads GBCA_ERR_TIMEOUT and the context
    stays usable."""
    with pytest.raises(ca.errors.DeviceTimeout):
        ca.capi.check(ca.capi.lib().gbca_selftest_wait(256))
    u0 = np.random.default_rng(2).integers(0, 2, (64, 64)).astype(np.int8)
    prob = ca.CAProblem.new(ca.Life(":conway"), u0, 5)
    sol = ca.solve(prob, ca.Synchronous(), backend=ca.GB300Backend())
    assert len(sol.u) == 6
