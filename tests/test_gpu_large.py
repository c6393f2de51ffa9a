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


def engine(g, mixed):
    e = Estimator()
    if mixed:
        e.set_option("use_double_precision", 0)
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
