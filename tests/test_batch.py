"""Batched form: many grids in one handle, solved together by the same kernels.

Each grid's result must equal solving it alone (same iteration count; states
within 1e-12, same arithmetic in both), and the FP64 batch must match the
oracle (states within 1e-8, same iteration counts).  The Gauss-Newton loop
runs on the device (a CUDA graph's conditional while node) and gives the same
bits as the host loop it replaces.
"""
import numpy as np
import pytest

from conftest import gpu_available
from oracle.binding import Oracle
from state_estimation_with_cuda_gb300 import BatchEstimator, Estimator, SLEError
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid, batch_sizes, grid_seed

pytestmark = pytest.mark.gpu

SAME = 1e-12


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.fail("GPU tests need a CUDA device; the product has no CPU fallback")


def small_batch(count=16, hi=1500):
    sizes = batch_sizes(count, seed=0x5E13, lo=30, hi=hi)
    return [SyntheticGrid(n, int(round(1.4 * n)), grid_seed(0x5E13, i)) for i, n in enumerate(sizes)]


def alone(g, mixed, z=None, z0=None, flat=True, robust=False):
    """Solve g on its own; with flat=False, first a flat start on z0 (the
    telemetry the batch's previous solve used), then a hot start on z."""
    e = Estimator()
    e.set_option("use_double_precision", 0 if mixed else 1)
    e.load_network(g, z=z0 if not flat else z)
    e.upload_model()
    if not flat:
        e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True, robust=robust)
        e.update_telemetry(z)
    rc, r = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=flat, robust=robust)
    out = (r.status, r.iterations, *e.voltages())
    e.close()
    return out


@pytest.mark.parametrize("mixed", [True, False])
def test_batch_equals_each_grid_alone(mixed):
    grids = small_batch()
    b = BatchEstimator(mixed=mixed)
    for g in grids:
        b.add_grid(g)
    res = b.solve(flat_start=True, max_iterations=20, tolerance=1e-6)
    for i, g in enumerate(grids):
        st, its, v, th = alone(g, mixed)
        bv, bth = b.state(i)
        assert res[i].status == st == 0, (i, res[i].status, st)
        assert res[i].iterations == its, (i, res[i].iterations, its)
        assert max(np.abs(bv - v).max(), np.abs(bth - th).max()) <= SAME, i
    b.close()


def test_fp64_batch_matches_oracle():
    grids = small_batch(6, hi=800)
    b = BatchEstimator(mixed=False)
    for g in grids:
        b.add_grid(g)
    res = b.solve(flat_start=True, max_iterations=20, tolerance=1e-6)
    for i, g in enumerate(grids):
        ov, oth, ores, _ = Oracle(g).wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
        v, th = b.state(i)
        assert res[i].status == ores.status == 0
        assert res[i].iterations == ores.iterations
        assert max(np.abs(v - ov).max(), np.abs(th - oth).max()) < 1e-8
        assert res[i].objective == pytest.approx(ores.objective, rel=1e-8)
    b.close()


def test_subset_hot_start_and_untouched_grids():
    grids = small_batch(10, hi=1000)
    b = BatchEstimator(mixed=True)
    for g in grids:
        b.add_grid(g)
    b.solve(flat_start=True)
    before = [b.state(i) for i in range(len(grids))]
    z0 = [g.z.copy() for g in grids]
    pick = [1, 4, 7]
    for i in pick:
        b.set_telemetry(i, grids[i].renoise(0))
    res = b.solve(grids=pick, flat_start=False)
    for k, i in enumerate(pick):
        st, its, v, th = alone(grids[i], True, z=grids[i].z, z0=z0[i], flat=False)
        bv, bth = b.state(i)
        assert res[k].status == st == 0 and res[k].iterations == its
        assert max(np.abs(bv - v).max(), np.abs(bth - th).max()) <= SAME
    for i in range(len(grids)):
        if i not in pick:
            v, th = b.state(i)
            assert np.array_equal(v, before[i][0]) and np.array_equal(th, before[i][1])
    b.close()


def test_breaker_edit_changes_values_only():
    g = SyntheticGrid(600, 840, 77)
    k = g._lib.segen_pick_nonbridge(g._h, 3)
    assert k >= 0
    b = BatchEstimator(mixed=False)
    b.add_grid(SyntheticGrid(200, 280, 5))
    gid = b.add_grid(g)
    b.solve(flat_start=True)
    # open branch k: the generator re-evaluates the true flows, fresh telemetry
    g._lib.segen_set_status(g._h, int(k), 0)
    z = g.renoise(1, 1.0)
    b.set_branch_status(gid, int(k), 0)
    b.set_telemetry(gid, z)
    res = b.solve(grids=[gid], flat_start=True)
    # reference: the same grid loaded with the branch open (pattern without it)
    status = g.br_status.copy()
    status[k] = 0
    g.br_status = status
    st, its, v, th = alone(g, False, z=z)
    bv, bth = b.state(gid)
    assert res[0].status == st == 0 and res[0].iterations == its
    assert max(np.abs(bv - v).max(), np.abs(bth - th).max()) < 1e-9
    b.close()


# ------------------------------------------- Gauss-Newton loop on the device
def run_batch(grids, mixed, device_loop, max_iterations=20, hot=None):
    b = BatchEstimator(mixed=mixed)
    b.set_option("device_loop", device_loop)
    for g in grids:
        b.add_grid(g)
    b.solve(flat_start=True, max_iterations=max_iterations)
    if hot is not None:
        for i, z in hot.items():
            b.set_telemetry(i, z)
    b.reset_stats()
    res = b.solve(flat_start=hot is None, max_iterations=max_iterations)
    st = b.stats()
    out = ([(r.status, r.iterations, r.max_mismatch, r.objective) for r in res],
           [np.concatenate(b.state(i)) for i in range(len(grids))], st.iterations, st.step_waits)
    b.close()
    return out


@pytest.mark.parametrize("mixed", [True, False])
def test_device_loop_equals_host_loop(mixed):
    """The conditional-node loop runs the same steps as the host loop and
    stops on the same test: identical per-grid results, bit for bit, with no
    host wait between steps."""
    grids = small_batch(12, hi=1200)
    hot = {i: grids[i].renoise(0).copy() for i in (0, 3, 5, 8)}
    for kw in ({}, {"hot": hot}, {"max_iterations": 2}):
        r_dev, s_dev, it_dev, w_dev = run_batch(grids, mixed, 1, **kw)
        r_host, s_host, it_host, w_host = run_batch(grids, mixed, 0, **kw)
        assert r_dev == r_host, kw
        assert all(np.array_equal(a, b) for a, b in zip(s_dev, s_host)), kw
        assert it_dev == it_host == max(r[1] for r in r_dev)
        assert w_dev == 0 and w_host == it_host
    # the step limit holds: every grid stops after two steps, none converged
    r2 = run_batch(grids, mixed, 1, max_iterations=2)[0]
    assert all(r[0] == 1 and r[1] == 2 for r in r2)


def test_device_loop_stops_on_a_timed_out_wait():
    """A dataflow wait that runs out inside the device loop ends the loop
    after that step and the solve reports it; the handle then solves again."""
    grids = small_batch(6, hi=1500)
    b = BatchEstimator(mixed=True)
    for g in grids:
        b.add_grid(g)
    par = b.symbolic()["sn_parent"]
    roots = np.nonzero(par < 0)[0]
    nchild = np.bincount(par[par >= 0], minlength=len(par))
    root = int(roots[np.argmax(nchild[roots])])
    assert nchild[root] > 0
    b.set_option("spin_limit", 1000)
    b.set_option("hold_front", root)
    b.reset_stats()
    with pytest.raises(SLEError) as err:
        b.solve(flat_start=True)
    assert "timed out" in str(err.value)
    assert b.stats().iterations == 1 and b.stats().step_waits == 0
    b.set_option("hold_front", -1)
    b.set_option("spin_limit", 1 << 22)
    res = b.solve(flat_start=True)
    for i, g in enumerate(grids):
        st, its, v, th = alone(g, True)
        bv, bth = b.state(i)
        assert res[i].status == st == 0 and res[i].iterations == its
        assert max(np.abs(bv - v).max(), np.abs(bth - th).max()) <= SAME
    b.close()
