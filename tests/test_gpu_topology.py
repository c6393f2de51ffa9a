"""GPU: the single-grid device topology processor against the CPU FP64
oracle loaded with the edited network.

The reference queues breaker changes and applies them before the next solve
(sle_engine.cu:1712-1773, sle_api.h:1063-1084) and forces a re-upload on tap
and impedance edits (sle_api.h:709-749).  Here a switched branch stays in the
uploaded pattern, so opening or closing it, and changing any branch's r, x,
charging, tap or phase shift, are value edits on the device: the branch
arrays are copied, admittances and Ybus recomputed, the factor invalidated
-- no new symbolic analysis and no new device arena.

Tolerances as the other parity tests: states 1e-8 pu / rad with the oracle's
iteration count (flat start, tol 1e-6).
"""
import numpy as np
import pytest

from conftest import gpu_available
from grids import copy_grid
from oracle.binding import Oracle
from state_estimation_with_cuda_gb300 import Estimator
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-8


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.fail("GPU tests need a CUDA device; the product has no CPU fallback")


def base():
    return SyntheticGrid(2000, 2800, 0x5E61)


def switched_branches(g, count):
    """Non-bridge branches without flow rows whose opening (all together)
    keeps the grid observable in the oracle."""
    metered = set(int(k) for k in g.m_loc[np.isin(g.m_type, (4, 5, 6))])
    out = []
    for d in range(5000):
        k = int(g._lib.segen_pick_nonbridge(g._h, d))
        if k < 0 or k in out or k in metered:
            continue
        trial = copy_grid(g)
        trial.br_status[out + [k]] = 0
        _, _, res, _ = Oracle(trial).wls(trial.z, trial.v_setpoint, np.zeros(trial.n_bus), max_iterations=20,
                                         tolerance=1e-6)
        if res.status == 0:
            out.append(k)
        if len(out) == count:
            return out
    raise RuntimeError("not enough switchable branches")


def solve_both(e, g_edit):
    """GPU flat start on the handle against the oracle on the edited grid."""
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    v, th = e.voltages()
    o = Oracle(g_edit)
    ov, oth, ores, orr = o.wls(g_edit.z, g_edit.v_setpoint, np.zeros(g_edit.n_bus), max_iterations=20,
                               tolerance=1e-6)
    return res, (v, th), ores, (ov, oth), e.bad_data(3.0), o.bad_data(orr, 3.0)


def check(res, st, ores, ost, flags, oflags):
    assert res.status == ores.status == 0
    assert res.iterations == ores.iterations
    assert max(np.abs(st[0] - ost[0]).max(), np.abs(st[1] - ost[1]).max()) < STATE_TOL
    assert np.array_equal(flags, oflags)


def test_switch_open_close_on_the_device_matches_oracle():
    g = base()
    ks = switched_branches(g, 3)
    e = Estimator()
    e.load_network(g)
    for i, k in enumerate(ks):
        e.add_switch("SW%d" % i, "BR%d" % k, closed=True)
    e.upload_model()
    check(*solve_both(e, copy_grid(g)))
    st0 = e.stats()
    # open two breakers: value edits applied at the next solve
    e.set_switch("SW0", False)
    e.set_switch("SW2", False)
    edited = copy_grid(g)
    edited.br_status[ks[0]] = 0
    edited.br_status[ks[2]] = 0
    check(*solve_both(e, edited))
    st1 = e.stats()
    assert st1.analyses == st0.analyses and st1.uploads == st0.uploads
    assert st1.branch_edits == st0.branch_edits + 1
    # islands on the device see the open branches (still one island: non-bridges)
    assert e.check_observability()[1] == 1
    # close one again, applied explicitly
    e.set_switch("SW0", True)
    e.apply_switch_changes()
    edited.br_status[ks[0]] = 1
    check(*solve_both(e, edited))
    st2 = e.stats()
    assert st2.analyses == st0.analyses and st2.uploads == st0.uploads
    assert st2.branch_edits == st0.branch_edits + 2
    e.close()


def test_tap_shift_and_impedance_edits_on_the_device_match_oracle():
    g = base()
    e = Estimator()
    e.load_network(g)
    e.upload_model()
    e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    st0 = e.stats()
    edited = copy_grid(g)
    taps = np.nonzero(g.br_tap != 1.0)[0][:2]
    for k in taps:
        e.set_transformer_tap("BR%d" % k, 1.02)
        edited.br_tap[k] = 1.02
    e.set_phase_shift("BR%d" % taps[0], 0.03)
    edited.br_shift[taps[0]] = 0.03
    k = 17
    e.set_branch_impedance("BR%d" % k, 0.02, 0.11, 0.03, 0.0)
    edited.br_r[k], edited.br_x[k], edited.br_b[k] = 0.02, 0.11, 0.03
    check(*solve_both(e, edited))
    st1 = e.stats()
    assert st1.analyses == st0.analyses and st1.uploads == st0.uploads
    assert st1.branch_edits == st0.branch_edits + 1
    # the device Ybus is the edited one
    ptr, col, gv, bv = e.ybus()
    optr, ocol, ogv, obv = Oracle(edited).ybus()
    assert np.array_equal(ptr, optr) and np.array_equal(col, ocol)
    assert np.allclose(gv, ogv, rtol=1e-13, atol=1e-12) and np.allclose(bv, obv, rtol=1e-13, atol=1e-12)
    e.close()


def test_opening_a_leaf_breaker_splits_the_islands_on_the_device():
    g = base()
    deg = np.bincount(np.concatenate([g.br_from, g.br_to]), minlength=g.n_bus)
    leaf = [k for k in range(g.n_branch) if deg[g.br_from[k]] == 1 or deg[g.br_to[k]] == 1][0]
    e = Estimator()
    e.load_network(g)
    e.add_switch("SWL", "BR%d" % leaf, closed=True)
    e.upload_model()
    assert e.check_observability() == (True, 1)
    e.set_switch("SWL", False)
    obs, islands = e.check_observability()
    assert islands == 2 and not obs
    assert e.stats().uploads == 1  # the edit went to the device, no new arena
    e.close()
