"""The CPU oracle checked on its own: the reference fixture, finite
differences, dense linear algebra, and the generator's inputs."""
import numpy as np
import pytest
import scipy.sparse as sp

from grids import ieee14, observable_ieee14, state_index, synthetic_state
from oracle.binding import Oracle
from state_estimation_with_cuda_gb300 import workloads
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid


def dense_h(o, g, v, th, z, exact=True):
    ev = o.evaluate(v, th, z, exact=exact)
    H = np.zeros((g.n_meas, 2 * g.n_bus - 1))
    for q in range(g.n_meas):
        for x in range(ev["h_ptr"][q], ev["h_ptr"][q + 1]):
            H[q, ev["h_col"][x]] += ev["h_val"][x]
    return ev, H


def test_ieee14_fixture_loads_and_is_unobservable():
    g = ieee14()
    assert (g.n_bus, g.n_branch, g.n_meas) == (14, 20, 31)
    assert g.slack == 0
    o = Oracle(g)
    v, th, res, r = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20)
    assert res.status == 3  # singular gain: buses 10..14 carry only |V|
    # rank deficiency of G equals the number of unobserved angles
    ev, H = dense_h(o, g, g.v_setpoint, np.zeros(g.n_bus), g.z)
    G = H.T @ np.diag(ev["w_eff"]) @ H
    assert np.linalg.matrix_rank(G, tol=1e-8 * np.abs(G).max()) < 2 * g.n_bus - 1


@pytest.mark.parametrize("which", ["grid14", "ieee14obs", "grid300"])
def test_exact_jacobian_matches_finite_differences(which):
    if which == "grid14":
        g = workloads.make("grid14")
    elif which == "ieee14obs":
        g = observable_ieee14()
    else:
        g = SyntheticGrid(300, 420, 77)
    o = Oracle(g)
    v, th = synthetic_state(g)
    z = np.zeros(g.n_meas)
    ev, H = dense_h(o, g, v, th, z, exact=True)
    eps = 1e-6
    for i in range(g.n_bus):
        for which_state in (0, 1):
            c = state_index(g, i, which_state)
            if c < 0:
                continue
            vp, tp, vm, tm = v.copy(), th.copy(), v.copy(), th.copy()
            if which_state == 0:
                tp[i] += eps
                tm[i] -= eps
            else:
                vp[i] += eps
                vm[i] -= eps
            hp = o.evaluate(vp, tp, z)["hx"]
            hm = o.evaluate(vm, tm, z)["hx"]
            fd = (hp - hm) / (2 * eps)
            assert np.allclose(H[:, c], fd, rtol=1e-6, atol=1e-6), (i, which_state, np.abs(H[:, c] - fd).max())


def test_reference_jacobian_differs_only_at_documented_defects():
    g = SyntheticGrid(120, 168, 5)
    o = Oracle(g)
    v, th = synthetic_state(g)
    z = np.zeros(g.n_meas)
    _, He = dense_h(o, g, v, th, z, exact=True)
    _, Hr = dense_h(o, g, v, th, z, exact=False)
    diff = np.argwhere(np.abs(He - Hr) > 1e-12)
    for q, c in diff:
        t, loc = int(g.m_type[q]), int(g.m_loc[q])
        if t in (2, 3, 7, 8):  # A1: injection angle-diagonal
            assert c == state_index(g, loc, 0)
        elif t == 4:  # A2: P flow at the TO end, angle columns
            assert g.m_end[q] == 1
            assert c in (state_index(g, g.br_from[loc], 0), state_index(g, g.br_to[loc], 0))
        elif t == 5:  # A3: Q flow, V column of the measured end (charging term dropped)
            end_bus = g.br_to[loc] if g.m_end[q] else g.br_from[loc]
            assert c == state_index(g, end_bus, 1)
        else:
            raise AssertionError("unexpected difference in row type %d" % t)
    assert len(diff) > 0


def test_oracle_gain_and_solve_match_dense_numpy():
    g = workloads.make("grid14")
    o = Oracle(g)
    v, th = synthetic_state(g)
    ev, H = dense_h(o, g, v, th, g.z)
    G = H.T @ np.diag(ev["w_eff"]) @ H
    rows, cols, vals = o.gain()
    Gs = sp.coo_matrix((vals, (rows, cols)), shape=G.shape).toarray()
    assert np.allclose(np.tril(G), Gs, rtol=1e-12, atol=1e-9)
    b = H.T @ (ev["w_eff"] * ev["r"])
    assert np.allclose(ev["rhs"], b, rtol=1e-12, atol=1e-9)
    st, x = o.solve_gain(ev["rhs"])
    assert st == 0
    assert np.allclose(x, np.linalg.solve(G, b), rtol=1e-9, atol=1e-12)


def test_oracle_symbolic_matches_dense_elimination():
    g = SyntheticGrid(60, 84, 11)
    o = Oracle(g)
    perm = o.ordering()
    assert sorted(perm.tolist()) == list(range(g.n_bus))
    parent, cc = o.symbolic(perm)
    # dense check: pattern of the Cholesky factor of a random SPD matrix with the bus-graph pattern
    ev, H = dense_h(o, g, *synthetic_state(g), g.z)
    A = (np.abs(H.T) > 0).astype(float) @ (np.abs(H) > 0).astype(float)
    # bus-level pattern: collapse states to buses
    bus_of = np.array([(c if c < g.slack else c + 1) if c < g.n_bus - 1 else c - (g.n_bus - 1)
                       for c in range(2 * g.n_bus - 1)])
    B = np.zeros((g.n_bus, g.n_bus))
    for a in range(A.shape[0]):
        for b in np.nonzero(A[a])[0]:
            B[bus_of[a], bus_of[b]] = 1
    P = B[np.ix_(perm, perm)] + g.n_bus * np.eye(g.n_bus)
    L = np.linalg.cholesky(P + 0.0)
    pattern = np.abs(L) > 1e-14
    for j in range(g.n_bus):
        below = np.nonzero(pattern[j + 1:, j])[0] + j + 1
        assert cc[j] == len(below) + 1 or cc[j] >= len(below) + 1
        if len(below):
            assert parent[j] == below[0]


def test_generator_is_deterministic_and_observable():
    a = SyntheticGrid(400, 560, 123)
    b = SyntheticGrid(400, 560, 123)
    for f in ("br_from", "br_to", "br_r", "br_x", "br_tap", "m_type", "m_loc", "z", "v_true", "theta_true"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    c = SyntheticGrid(400, 560, 124)
    assert not np.array_equal(a.z, c.z)
    o = Oracle(a)
    v, th, res, r = o.wls(a.z, a.v_setpoint, np.zeros(a.n_bus), max_iterations=20)
    assert res.status == 0 and res.iterations <= 8
    # renoise touches 1 % of the rows
    z0 = a.z.copy()
    z1 = a.renoise(0, 0.01)
    assert (z0 != z1).sum() == round(0.01 * a.n_meas)


def test_workload_counts():
    g = workloads.make("grid14")
    assert (g.n_bus, g.n_branch, g.n_meas) == (14, 20, 67)
    assert (g.br_tap != 1.0).sum() == 3
    g = workloads.make("grid10k")
    assert (g.n_bus, g.n_branch) == (10000, 14000)
    base = 3000 + 2 * 6000 + 4 * 9800
    assert g.n_meas >= base and g.n_meas - base < 0.02 * base  # pseudo flows restore observability


def test_bad_data_flags_follow_normalized_residual():
    g = workloads.make("grid14")
    o = Oracle(g)
    r = np.linspace(-0.05, 0.05, g.n_meas)
    idx = o.bad_data(r, 3.0)
    exp = np.nonzero(np.abs(r) / g.m_sigma > 3.0)[0]
    assert np.array_equal(idx, exp)
