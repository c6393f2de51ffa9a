"""GPU parity at the sizes whose factorisation runs the tiled multi-CTA front
kernels, against the CPU FP64 oracle (flat start, tol 1e-6).

  grid20k   20,000 buses / 28,000 branches: eight fronts wider than the
            single-CTA limit, so the FP32 tiled kernels (panel, trailing
            update, assembly) and the FP64 tiled kernels both run.
  grid200k  the 200,000-bus / 280,000-branch workload (1.09 M rows, 2 % gross
            errors on telemetry rows), plain WLS as the reference runs it
            with robust estimation off.

Tolerances: plain FP64 states 1e-8 pu / rad with the oracle's iteration
count and bad-data flags; mixed precision (FP32 H, G and L, FP64 residual,
gradient and state) 1e-6 pu / rad, iterations within one of the oracle's.
The mixed pipeline's tiled fronts run as a panel and an update launch per
step by default; the dataflow form (option tile_flow = 1, one persistent
launch per level) computes the same arithmetic, so both give the same bits.
"""
import numpy as np
import pytest

from conftest import gpu_available
from oracle.binding import Oracle
from state_estimation_with_cuda_gb300 import Estimator, workloads
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.fail("GPU tests need a CUDA device; the product has no CPU fallback")


def engine(g, mixed, **options):
    e = Estimator()
    if mixed:
        e.set_option("use_double_precision", 0)
    for k, v in options.items():
        e.set_option(k, v)
    e.load_network(g)
    return e


def state_err(e, ov, oth):
    v, th = e.voltages()
    return max(np.abs(v - ov).max(), np.abs(th - oth).max())


@pytest.fixture(scope="module")
def grid20k():
    g = SyntheticGrid(20000, 28000, 0x5E77)
    o = Oracle(g)
    ov, oth, ores, orr = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    return g, o, (ov, oth, ores, orr)


@pytest.mark.parametrize("mixed", [False, True])
def test_tiled_fronts_grid20k_flat_start(grid20k, mixed):
    g, o, (ov, oth, ores, orr) = grid20k
    e = engine(g, mixed)
    si = e.schedule_info()
    assert si.n_sync > 0 and si.panel_steps > 0  # tiled fronts are on the path
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    assert rc == 0 and res.status == ores.status == 0
    if mixed:
        assert abs(res.iterations - ores.iterations) <= 1
        assert state_err(e, ov, oth) < 1e-6
    else:
        assert res.iterations == ores.iterations
        assert state_err(e, ov, oth) < 1e-8
        assert np.array_equal(e.bad_data(3.0), o.bad_data(orr, 3.0))
    e.close()


def tile_flow_bits(g, tile_flow, hot):
    """Flat start then hot starts on re-noised telemetry; the states and
    results of every solve, and the factor's own G x = b at the end."""
    e = engine(g, True, tile_flow=tile_flow)
    si = e.schedule_info()
    out = [si.tile_tasks]
    rc, r = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    out.append((rc, r.status, r.iterations, r.max_mismatch, *map(np.copy, e.voltages())))
    for z in hot:
        e.update_telemetry(z)
        rc, r = e.solve_with(max_iterations=20, tolerance=1e-6)
        out.append((rc, r.status, r.iterations, r.max_mismatch, *map(np.copy, e.voltages())))
    e.close()
    return out


def same(a, b):
    if isinstance(a, np.ndarray):
        return np.array_equal(a, b)
    if isinstance(a, tuple):
        return all(same(x, y) for x, y in zip(a, b))
    return a == b


def test_tile_dataflow_equals_per_step_launches(grid20k):
    g, _, _ = grid20k
    z0 = g.z.copy()
    hot = [g.renoise(u).copy() for u in range(2)]
    g.z = z0
    on = tile_flow_bits(g, 1, hot)
    off = tile_flow_bits(g, 0, hot)
    assert on[0] > 0 and off[0] == 0
    for a, b in zip(on[1:], off[1:]):
        assert a[0] == 0 and a[1] == 0
        assert same(a, b)


def test_tile_dataflow_batch_equals_alone():
    """Tiled fronts of several grids share a level's dataflow launch; each
    grid's result equals the grid alone (a frozen grid's items publish
    without computing)."""
    from state_estimation_with_cuda_gb300 import BatchEstimator
    grids = [SyntheticGrid(n, int(round(1.4 * n)), 0x5E90 + i) for i, n in enumerate((20000, 12000, 16000))]
    b = BatchEstimator(mixed=True)
    b.set_option("tile_flow", 1)
    for g in grids:
        b.add_grid(g)
    assert b.schedule_info().tile_tasks > 0
    res = b.solve(flat_start=True, max_iterations=20, tolerance=1e-6)
    for i, g in enumerate(grids):
        e = engine(g, True)
        rc, r = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
        v, th = e.voltages()
        e.close()
        bv, bth = b.state(i)
        assert res[i].status == r.status == 0 and res[i].iterations == r.iterations
        assert max(np.abs(bv - v).max(), np.abs(bth - th).max()) <= 1e-12
    b.close()


def test_tiled_fronts_grid20k_mixed_hot_start_sequence(grid20k):
    g, o, (ov, oth, _, _) = grid20k
    e = engine(g, True)
    e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    z0 = g.z.copy()
    for u in range(3):
        z = g.renoise(u)
        e.update_telemetry(z)
        rc, res = e.solve_with(max_iterations=20, tolerance=1e-6)
        ov, oth, ores, _ = o.wls(z, ov, oth, max_iterations=20, tolerance=1e-6, flat_start=False)
        assert res.status == 0
        assert state_err(e, ov, oth) < 1e-6
    g.z = z0
    e.close()


@pytest.fixture(scope="module")
def grid200k():
    g = workloads.make("grid200k")
    o = Oracle(g)
    ov, oth, ores, orr = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    flags = o.bad_data(orr, 3.0)
    o.close()
    return g, (ov, oth, ores, flags)


def test_grid200k_fp64_flat_start_matches_oracle(grid200k):
    g, (ov, oth, ores, flags) = grid200k
    e = engine(g, False)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    assert rc == 0 and res.status == ores.status == 0
    assert res.iterations == ores.iterations
    assert state_err(e, ov, oth) < 1e-8
    assert res.objective == pytest.approx(ores.objective, rel=1e-9)
    assert np.array_equal(e.bad_data(3.0), flags)
    e.close()


def test_grid200k_mixed_flat_start_within_1e6(grid200k):
    g, (ov, oth, ores, _) = grid200k
    e = engine(g, True)
    si = e.schedule_info()
    assert si.n_sync > 0 and si.panel_steps > 0
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    assert rc == 0 and res.status == 0
    assert abs(res.iterations - ores.iterations) <= 1
    assert state_err(e, ov, oth) < 1e-6
    e.close()
