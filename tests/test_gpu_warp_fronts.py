"""Warp phase: fronts whose whole subtree is at most 32 wide are factorised
and solved one front per warp.  By default every grid with such fronts
uses it; here it is forced on and off.

* FP64 with the warp phase matches the oracle with the parity tolerances
  (G x = b within 1e-9, same iteration counts, states within 1e-8);
* the mixed pipeline stays within 1e-6 of the oracle;
* on and off agree with each other within the same tolerances (different
  summation orders, same mathematics);
* the phase is decided per grid, so a grid inside a batch runs the kernels
  it runs alone: same iterations, states within 1e-12.
"""
import numpy as np
import pytest

from conftest import gpu_available
from grids import synthetic_state
from oracle.binding import Oracle
from state_estimation_with_cuda_gb300 import BatchEstimator, Estimator, workloads
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid, batch_sizes, grid_seed

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-8
SAME = 1e-12


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.fail("GPU tests need a CUDA device; the product has no CPU fallback")


def grid(name):
    if name == "grid2k":
        return SyntheticGrid(2000, 2800, 0x5E01)
    return workloads.make(name)


def engine(g, warp, mixed=False, z=None):
    e = Estimator()
    e.set_option("use_double_precision", 0 if mixed else 1)
    e.set_option("warp_fronts", warp)
    e.load_network(g, z=z)
    e.upload_model()
    return e


@pytest.mark.parametrize("name", ["grid2k", "grid10k"])
def test_warp_phase_factor_solve_matches_oracle(name):
    g = grid(name)
    e, o = engine(g, 1), Oracle(g)
    v, th = synthetic_state(g)
    e.evaluate_at(v, th, exact=True)
    ref = o.evaluate(v, th, g.z, exact=True)
    st, xo = o.solve_gain(ref["rhs"])
    assert st == 0
    xg = e.factor_solve(ref["rhs"])
    assert np.abs(xg - xo).max() <= 1e-9 * max(np.abs(xo).max(), 1e-30)
    e.close()


@pytest.mark.parametrize("name", ["grid2k", "grid10k"])
@pytest.mark.parametrize("mixed", [False, True])
def test_warp_phase_flat_start_matches_oracle(name, mixed):
    g = grid(name)
    o = Oracle(g)
    ov, oth, ores, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    e = engine(g, 1, mixed)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    v, th = e.voltages()
    e.close()
    assert rc == 0 and res.status == ores.status == 0
    err = max(np.abs(v - ov).max(), np.abs(th - oth).max())
    if mixed:
        assert abs(res.iterations - ores.iterations) <= 1
        assert err < 1e-6
    else:
        assert res.iterations == ores.iterations
        assert err < STATE_TOL


@pytest.mark.parametrize("mixed", [False, True])
def test_warp_phase_on_and_off_agree(mixed):
    g = grid("grid10k")
    z0 = g.z.copy()
    snaps = [g.renoise(u).copy() for u in range(2)]  # renoise accumulates: draw once
    out = []
    for warp in (0, 1):
        e = engine(g, warp, mixed, z=z0)
        e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
        seq = []
        for z in snaps:
            e.update_telemetry(z)
            rc, r = e.solve_with(max_iterations=20, tolerance=1e-6)
            seq.append((r.status, r.iterations))
        out.append((seq, np.concatenate(e.voltages())))
        e.close()
    if mixed:
        assert all(abs(a[1] - b[1]) <= 1 and a[0] == b[0] == 0 for a, b in zip(out[0][0], out[1][0]))
        assert np.abs(out[0][1] - out[1][1]).max() < 1e-6
    else:
        assert out[0][0] == out[1][0]
        assert np.abs(out[0][1] - out[1][1]).max() < STATE_TOL


def test_batch_with_warp_phase_equals_alone_with_it():
    sizes = batch_sizes(12, seed=0x5E31, lo=30, hi=1200)
    grids = [SyntheticGrid(n, int(round(1.4 * n)), grid_seed(0x5E31, i)) for i, n in enumerate(sizes)]
    b = BatchEstimator(mixed=True)
    b.set_option("warp_fronts", 1)
    for g in grids:
        b.add_grid(g)
    res = b.solve(flat_start=True, max_iterations=20, tolerance=1e-6)
    for i, g in enumerate(grids):
        e = engine(g, 1, mixed=True)
        rc, r = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
        v, th = e.voltages()
        e.close()
        bv, bth = b.state(i)
        assert res[i].status == r.status == 0
        assert res[i].iterations == r.iterations, (i, res[i].iterations, r.iterations)
        assert max(np.abs(bv - v).max(), np.abs(bth - th).max()) <= SAME, i
    b.close()
