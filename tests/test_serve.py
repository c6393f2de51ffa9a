"""Serving form: requests for many grids in flight at once, continuous
batching across size units, breaker edits and memory-budget admission.

Each served result must equal the same grid solved alone through the same
sequence of snapshots (same iteration count, states within 1e-12: the same
kernels run the same arithmetic), however the requests were batched.
"""
import numpy as np
import pytest

from conftest import gpu_available
from state_estimation_with_cuda_gb300 import Estimator, Server
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid, grid_seed

pytestmark = pytest.mark.gpu

SAME = 1e-12
SIZES = [40, 75, 120, 260, 300, 520, 900, 1400, 2100, 2600, 3300, 60]


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.fail("GPU tests need a CUDA device; the product has no CPU fallback")


def fleet():
    return [SyntheticGrid(n, int(round(1.4 * n)), grid_seed(0x5E24, i)) for i, n in enumerate(SIZES)]


def server_for(grids, **kw):
    s = Server(mixed=True, bucket_bus=(150, 1000, 0, 0), own_unit_bus=2500, **kw)
    for g in grids:
        s.add_grid(g)
    s.start()
    return s


def chain_alone(g, z0, snaps):
    """Flat start on z0, then one hot start per snapshot; returns (iters, V, theta) per snapshot."""
    e = Estimator()
    e.set_option("use_double_precision", 0)
    e.load_network(g, z=z0)
    e.upload_model()
    e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    out = []
    for z in snaps:
        e.update_telemetry(z)
        rc, r = e.solve_with(max_iterations=20, tolerance=1e-6)
        out.append((r.status, r.iterations, *e.voltages()))
    e.close()
    return out


def test_served_results_equal_alone():
    grids = fleet()
    z0 = [g.z.copy() for g in grids]
    s = server_for(grids)
    st = s.stats()
    assert st.units == 5 and st.admitted_units == 5  # 3 shared size units + 2 own units
    # three snapshots per grid, all submitted at once: a grid's later snapshots
    # queue behind its earlier ones and join later passes
    snaps = [[g.renoise(u).copy() for u in range(3)] for g in grids]
    tickets = [[s.submit(i, snaps[i][u]) for u in range(3)] for i in range(len(grids))]
    results = [[s.wait(t, 60000.0) for t in row] for row in tickets]
    batched = 0
    for i, g in enumerate(grids):
        ref = chain_alone(g, z0[i], snaps[i])
        for u in range(3):
            r = results[i][u]
            assert r is not None and r.admitted == 1
            assert r.status == ref[u][0] == 0
            assert r.iterations == ref[u][1], (i, u, r.iterations, ref[u][1])
            batched += r.batch_size > 1
            assert r.t_submit_ns <= r.t_start_ns <= r.t_done_ns
        v, th = s.state(i)
        assert max(np.abs(v - ref[2][2]).max(), np.abs(th - ref[2][3]).max()) <= SAME, i
    assert batched > 0  # requests of different grids shared passes
    st = s.stats()
    assert st.completed == st.submitted == 3 * len(grids) and st.rejected == 0
    s.close()


def test_breaker_request():
    grids = fleet()[:4]
    z0 = [g.z.copy() for g in grids]
    s = server_for(grids)
    g = grids[3]
    k = g._lib.segen_pick_nonbridge(g._h, 11)
    assert k >= 0
    g._lib.segen_set_status(g._h, int(k), 0)
    z = g.renoise(2, 1.0)
    t = s.submit(3, z, branch=int(k), closed=0)
    r = s.wait(t, 60000.0)
    assert r.status == 0
    # alone: hot start from the estimate of z0 with the branch open
    e = Estimator()
    e.set_option("use_double_precision", 0)
    e.load_network(g, z=z0[3])
    e.upload_model()
    e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    v0, th0 = e.voltages()
    e.close()
    status = g.br_status.copy()
    status[k] = 0
    g.br_status = status
    e = Estimator()
    e.set_option("use_double_precision", 0)
    e.load_network(g, z=z)
    e.upload_model()
    e.lib.sle_ApplyFlatStart(e.h)
    rc, ra = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    va, tha = e.voltages()
    e.close()
    v, th = s.state(3)
    # both converge to the same estimate of the edited topology (different
    # start points and patterns, so within the convergence tolerance)
    assert ra.status == 0
    assert max(np.abs(v - va).max(), np.abs(th - tha).max()) < 1e-5
    s.close()


def fleet_bytes(grids):
    s = server_for(grids)
    b = s.stats().device_bytes
    s.close()
    return b


def test_unit_larger_than_the_budget_is_not_admitted():
    grids = fleet()
    total = fleet_bytes(grids)
    s = server_for(grids, memory_budget=total // 12)
    st = s.stats()
    assert 0 < st.admitted_units < st.units  # the largest units alone exceed the budget
    assert st.device_bytes <= st.budget_bytes
    outcomes = []
    for i, g in enumerate(grids):
        r = s.wait(s.submit(i, g.z), 60000.0)
        outcomes.append(r.admitted)
        if r.admitted:
            assert r.status == 0
        else:
            assert r.status == 4  # NOT_OBSERVABLE: no unit can hold the grid
    assert 0 in outcomes and 1 in outcomes
    st = s.stats()
    assert st.rejected == outcomes.count(0)
    assert st.device_bytes <= st.budget_bytes
    s.close()


def test_budget_smaller_than_the_fleet_serves_every_request():
    """Units are brought in as requests arrive and idle ones are evicted to
    make room; a grid's states survive eviction on the host, so every result
    equals the grid solved alone through the same snapshots."""
    grids = fleet()
    z0 = [g.z.copy() for g in grids]
    total = fleet_bytes(grids)
    s = server_for(grids, memory_budget=int(0.55 * total))
    st = s.stats()
    assert st.admitted_units == st.units and st.resident_units < st.units
    snaps = [[g.renoise(u).copy() for u in range(2)] for g in grids]
    outs = [[(np.full(g.n_bus, np.nan), np.full(g.n_bus, np.nan)) for _ in range(2)] for g in grids]
    # round-robin over the grids: every unit is needed again after the others
    for u in range(2):
        tickets = [s.submit(i, snaps[i][u], out=outs[i][u]) for i in range(len(grids))]
        for i, t in enumerate(tickets):
            r = s.wait(t, 120000.0)
            assert r is not None and r.admitted == 1 and r.status == 0, (i, u)
    st = s.stats()
    assert st.evictions > 0 and st.admissions > 0
    assert st.device_bytes <= st.budget_bytes
    assert st.completed == st.submitted == 2 * len(grids) and st.rejected == 0
    for i, g in enumerate(grids):
        ref = chain_alone(g, z0[i], snaps[i])
        for u in range(2):
            v, th = outs[i][u]
            assert max(np.abs(v - ref[u][2]).max(), np.abs(th - ref[u][3]).max()) <= SAME, (i, u)
    s.close()


def test_submit_with_state_buffers_returns_the_served_state():
    grids = fleet()[:5]
    s = server_for(grids)
    outs = [(np.empty(g.n_bus), np.empty(g.n_bus)) for g in grids]
    tickets = [s.submit(i, g.renoise(7), out=outs[i]) for i, g in enumerate(grids)]
    for i, t in enumerate(tickets):
        r = s.wait(t, 60000.0)
        assert r.status == 0
        v, th = s.state(i)
        assert np.array_equal(v, outs[i][0]) and np.array_equal(th, outs[i][1])
    s.close()
