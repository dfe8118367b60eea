"""update_cell (src/backends.jl:281-307): the new state of one cell under a synchronous update of
the whole state at time t, without changing the state. Over every cell it is one synchronous
step (test/test_backend_interface.jl:35-67), here checked against the oracle's ReferenceBackend
step on a masked forest fire with Constant(1) and Reflecting edges at two times, and on
Larger-than-Life on a torus; a masked cell keeps its state; kernel-field problems are refused,
as in the reference (the refusals need no GPU)."""
import numpy as np
import pytest


def test_update_cell_refuses_kernel_fields_and_bad_indices(gbca):
    ca = gbca
    u0 = np.zeros((12, 10), np.int8)
    field = ca.KernelField(ca.GaussianKernel(1.5), source="x == 1")
    prob = ca.CAProblem.new(ca.KernelSI(field="pressure"), u0, 3, {"β": 0.5}, fields={"pressure": field})
    with pytest.raises(ca.ArgumentError, match="kernel fields"):
        ca.update_cell(prob, u0, (1, 1), 0)
    lenia = ca.CAProblem.new(ca.Lenia(precision="Float32"), np.zeros((8, 8), np.float32), 1)
    with pytest.raises(ca.ArgumentError, match="kernel fields"):
        ca.update_cell(lenia, lenia.u0, (1, 1), 0)
    life = ca.CAProblem.new(ca.Life(), u0, 3)
    with pytest.raises(ca.ArgumentError):
        ca.update_cell(life, u0, (13, 1), 0)
    with pytest.raises(ca.ArgumentError):
        ca.update_cell(life, u0, 121, 0)
    with pytest.raises(ca.StateShapeError):
        ca.update_cell(life, np.zeros((5, 5), np.int8), (1, 1), 0)


@pytest.mark.gpu
def test_update_cell_over_every_cell_is_one_synchronous_step(gbca, oracle):
    ca, o = gbca, oracle
    if ca.capi.lib().gbca_device_count() < 1:
        pytest.fail("no CUDA device visible")
    rng = np.random.default_rng(3)
    n1, n2 = 12, 10
    mask = np.ones((n1, n2), bool)
    mask[0:3, :] = False
    u0 = rng.integers(0, 3, (n1, n2)).astype(np.int8)
    space = ca.Lattice((n1, n2), (ca.Constant(1), ca.Reflecting()))
    params = {"p": 0.3, "f": 0.05}
    prob = ca.CAProblem.new(ca.ForestFire(), u0, 8, params, space=space, seed=4, mask=mask)
    P = o.Problem(o.RULE_FOREST_FIRE, n1, n2, nbhd=o.VON_NEUMANN, seed=4, boundary=(o.CONSTANT, o.REFLECTING),
                  constant=(1, 0))
    env = o.Env(mask=mask)
    u = u0
    states = [u0]
    for t in range(4):
        u = o.step_reference_env(P, env, u, t, (0.3, 0.05))
        states.append(u)
    for t in (0, 3):
        stepped = np.array([[ca.update_cell(prob, states[t], (i, j), t) for j in range(1, n2 + 1)]
                            for i in range(1, n1 + 1)], dtype=np.int8)
        assert np.array_equal(stepped, states[t + 1]), t
        assert not np.array_equal(states[t + 1], states[t])
    assert ca.update_cell(prob, u0, (2, 5), 0) == u0[1, 4]  # masked: unchanged
    k = 8 + 4 * n1  # the 1-based linear index of (8, 5)
    assert ca.update_cell(prob, u0, k, 0) == ca.update_cell(prob, u0, (8, 5), 0)
    assert ca.update_cell(prob, u0, (8, 5), 0, {"p": 0.3, "f": 0.05}) == states[1][7, 4]

    ltl = ca.CAProblem.new(ca.Life(range(34, 46), range(34, 59), neighbourhood=ca.Moore(5)),
                           rng.integers(0, 2, (40, 33)).astype(np.int8), 3)
    PL = o.Problem(o.RULE_LIFE, 40, 33, radius=5, birth=o.mask(range(34, 46)), survive=o.mask(range(34, 59)))
    want = o.step_reference(PL, ltl.u0, 0)
    got = np.array([[ca.update_cell(ltl, ltl.u0, (i, j), 0) for j in range(1, 34)] for i in range(1, 41)], np.int8)
    assert np.array_equal(got, want)
