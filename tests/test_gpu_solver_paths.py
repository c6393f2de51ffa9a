"""GPU: the Gauss-Newton driver's non-happy paths and the reference's own
solver policies, against the CPU FP64 oracle, through the C ABI.

Reference behaviour covered (wls_solver.cu / kernels.cu of the reference):
  NaN / Inf in the step -> DIVERGED, <= 2 flat-start retries outside REALTIME
                                        wls_solver.cu:326-332, kernels.cu:926-941
  REALTIME time limit   -> MAX_ITERATIONS  wls_solver.cu:313-323
  fixed-gain policy (G kept until invalidated)  wls_solver.cu:416-419
  the reference's Jacobian formulas (defects A1-A4 kept)  sparse_matrix.cu:1627-2147
  sigma = 0 rows: weight 1/max(sigma, eps)^2 (network_model.cu:142-143), never
  flagged as bad data (sle_engine.cu:959-977)
  I_MAG rows (kernels.cu:335-375), result accessors (sle_engine.cu:841-977)
plus the bounded dataflow wait of the solves, made to run out on purpose.

Tolerances: states 1e-8 pu / rad (relative to max(1, |x|) where the reference
formulas throw the state far from 1 pu), same status and iteration count;
stage values rtol 1e-12; accessor values 1e-12 of their scale.
"""
import numpy as np
import pytest

from conftest import gpu_available
from grids import copy_grid, with_current_rows
from oracle.binding import Oracle
from state_estimation_with_cuda_gb300 import Estimator, SLEError, api, workloads
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-8


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.fail("GPU tests need a CUDA device; the product has no CPU fallback")


def grid2k():
    return SyntheticGrid(2000, 2800, 0x5E01)


def engine(g, **options):
    e = Estimator()
    for k, v in options.items():
        e.set_option(k, v)
    e.load_network(g)
    e.upload_model()
    return e


def state_err(v, th, ov, oth, relative=False):
    if relative:
        return max((np.abs(v - ov) / np.maximum(1.0, np.abs(ov))).max(),
                   (np.abs(th - oth) / np.maximum(1.0, np.abs(oth))).max())
    return max(np.abs(v - ov).max(), np.abs(th - oth).max())


# ---------------------------------------------------------------- divergence
@pytest.mark.parametrize("mode", [api.MODE_PRECISION, api.MODE_REALTIME])
def test_nan_telemetry_diverges_with_flat_start_retries(mode):
    g = grid2k()
    e, o = engine(g), Oracle(g)
    z = g.z.copy()
    z[17] = np.nan
    e.update_telemetry(z)
    e.set_config(max_precision_iterations=20, max_realtime_iterations=20, realtime_time_limit_ms=0.0,
                 use_flat_start_default=1)
    it0 = e.stats().iterations
    rc, res = e.solve(mode)
    runs = e.stats().iterations - it0
    ov, oth, ores, _ = o.wls(z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6,
                             realtime=(mode == api.MODE_REALTIME))
    assert ores.status == 2 and res.status == 2
    assert rc == api.ERROR_DIVERGED
    assert res.iterations == ores.iterations == 1
    # the step of every attempt is non-finite: 1 attempt in REALTIME, 1 + 2 retries otherwise
    assert runs == (1 if mode == api.MODE_REALTIME else 3)
    # the handle stays usable: finite telemetry and a flat start converge like the oracle
    e.update_telemetry(g.z)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    v, th = e.voltages()
    ov, oth, ores, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    assert rc == 0 and res.status == ores.status == 0 and res.iterations == ores.iterations
    assert state_err(v, th, ov, oth) < STATE_TOL
    e.close()


def test_realtime_time_limit_ends_with_max_iterations():
    g = grid2k()
    e, o = engine(g), Oracle(g)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True, mode=api.MODE_REALTIME,
                           time_limit_ms=1e-6)
    assert rc == api.ERROR_MAX_ITERATIONS and res.status == 1 and res.iterations == 1
    v, th = e.voltages()
    ov, oth, ores, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=1, tolerance=1e-6, realtime=True)
    assert ores.status == 1 and ores.iterations == 1
    assert state_err(v, th, ov, oth) < STATE_TOL  # the one step taken is the oracle's
    # sle_Solve(REALTIME) takes the limit and the iteration cap from the handle's configuration
    e.set_config(realtime_time_limit_ms=1e-6, max_realtime_iterations=20, use_flat_start_default=1)
    rc, res = e.solve(api.MODE_REALTIME)
    assert rc == api.ERROR_MAX_ITERATIONS and res.status == 1 and res.iterations == 1
    # without a limit the same configuration converges
    e.set_config(realtime_time_limit_ms=0.0)
    rc, res = e.solve(api.MODE_REALTIME)
    ov, oth, ores, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6, realtime=True)
    assert rc == 0 and res.status == ores.status == 0 and res.iterations == ores.iterations
    e.close()


# ----------------------------------------------------------- reference policies
@pytest.mark.parametrize("name", ["grid14", "grid2k", "grid10k"])
def test_fixed_gain_policy_hot_start_sequence_matches_oracle(name):
    """gain_policy = 1: the factor of G stays valid across iterations and
    solves until the model changes, as in the reference's realtime operation
    (wls_solver.cu:416-419).  A flat-start estimate leaves the factor of its
    last iteration; the hot starts that follow reuse it.  (From a flat start
    the fixed-gain iteration does not converge, in the oracle and on the GPU
    alike, so the sequence starts from the estimate.)"""
    g = grid2k() if name == "grid2k" else workloads.make(name)
    e, o = engine(g), Oracle(g)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    ov, oth, ores, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    assert res.status == ores.status == 0 and res.iterations == ores.iterations
    e.set_option("gain_policy", 1)
    before = e.stats().launches[1]
    for u in range(3):
        z = g.renoise(u)
        e.update_telemetry(z)
        rc, res = e.solve_with(max_iterations=30, tolerance=1e-6, flat_start=False)
        ov, oth, ores, _ = o.wls(z, ov, oth, max_iterations=30, tolerance=1e-6, gain_policy=1, flat_start=False)
        v, th = e.voltages()
        assert res.status == ores.status == 0, (u, res.status, ores.status)
        assert res.iterations == ores.iterations, (u, res.iterations, ores.iterations)
        assert state_err(v, th, ov, oth) < STATE_TOL, u
    assert e.stats().launches[1] == before  # no factorisation ran in the sequence
    e.close()


@pytest.mark.parametrize("name", ["grid14", "grid2k"])
@pytest.mark.parametrize("gain_policy", [0, 1])
@pytest.mark.parametrize("steps", [1, 2])
def test_reference_jacobian_steps_match_oracle(name, gain_policy, steps):
    """exact_jacobian = 0 runs the reference's own formulas (defects A1-A4
    kept).  They do not converge on these grids (the oracle agrees), so the
    check is step by step: the state after k flat-start steps.  Two steps at
    most: after the second the angles run to 1e3-1e4 rad, where the sine and
    cosine of either side amplify last-place differences past 1e-8."""
    g = grid2k() if name == "grid2k" else workloads.make(name)
    e, o = engine(g, exact_jacobian=0, gain_policy=gain_policy), Oracle(g)
    rc, res = e.solve_with(max_iterations=steps, tolerance=1e-6, flat_start=True)
    v, th = e.voltages()
    ov, oth, ores, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=steps, tolerance=1e-6,
                             exact=False, gain_policy=gain_policy)
    assert res.status == ores.status == 1 and res.iterations == ores.iterations == steps
    assert state_err(v, th, ov, oth, relative=True) < STATE_TOL
    e.close()


def test_reference_jacobian_from_the_estimate_matches_oracle():
    g = grid2k()
    o = Oracle(g)
    ev, eth, _, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    e = engine(g, exact_jacobian=0)
    e.evaluate_at(ev, eth, exact=False)
    rc, res = e.solve_with(max_iterations=3, tolerance=1e-6, flat_start=False)
    v, th = e.voltages()
    ov, oth, ores, _ = o.wls(g.z, ev, eth, max_iterations=3, tolerance=1e-6, exact=False, flat_start=False)
    assert res.status == ores.status and res.iterations == ores.iterations
    assert state_err(v, th, ov, oth, relative=True) < STATE_TOL
    e.close()


def test_zero_sigma_rows_weight_and_bad_data():
    g = copy_grid(grid2k())
    vrows = np.nonzero(g.m_type == 0)[0][:3]
    g.m_sigma[vrows] = 0.0
    e, o = engine(g), Oracle(g)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    v, th = e.voltages()
    ov, oth, ores, orr = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    assert res.status == ores.status == 0 and res.iterations == ores.iterations
    assert state_err(v, th, ov, oth) < STATE_TOL
    # the zero-sigma rows are held (weight 1e24) and never flagged
    assert np.abs(v[g.m_loc[vrows]] - g.z[vrows]).max() < 1e-9
    flagged = e.bad_data(3.0)
    assert np.array_equal(flagged, o.bad_data(orr, 3.0))
    assert not np.isin(vrows, flagged).any()
    e.close()


# ------------------------------------------------------------ bounded waits
def test_dataflow_wait_timeout_is_reported_not_hung():
    """The backward sweep waits (bounded) on each front's parent.  With the
    root's completion withheld, its children's waits run out after
    spin_limit polls: the call returns an error instead of hanging, and the
    handle works again once the hook is off."""
    g = grid2k()
    e, o = engine(g), Oracle(g)
    sym = e.symbolic()
    par = sym["sn_parent"]
    roots = np.nonzero(par < 0)[0]
    nchild = np.bincount(par[par >= 0], minlength=len(par))
    root = int(roots[np.argmax(nchild[roots])])
    assert nchild[root] > 0
    v, th = g.v_true, g.theta_true
    ref = o.evaluate(v, th, g.z, exact=True)
    st, xo = o.solve_gain(ref["rhs"])
    e.set_option("spin_limit", 1000)
    e.set_option("hold_front", root)
    e.evaluate_at(v, th, exact=True)
    with pytest.raises(SLEError) as err:
        e.factor_solve(ref["rhs"])
    assert err.value.code == api.ERROR_CUDA_FAILURE and "timed out" in str(err.value)
    rc, res = e.solve_with(max_iterations=5, tolerance=1e-6, flat_start=True)
    assert rc == api.ERROR_MAX_ITERATIONS and res.status == 3  # SINGULAR_MATRIX, like any in-iteration failure
    assert "timed out" in e.last_error()
    e.set_option("hold_front", -1)
    e.set_option("spin_limit", 1 << 22)
    e.evaluate_at(v, th, exact=True)
    x = e.factor_solve(ref["rhs"])
    assert np.abs(x - xo).max() <= 1e-9 * np.abs(xo).max()
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    assert rc == 0 and res.status == 0
    e.close()


# ---------------------------------------------------------- outputs and rows
def test_result_accessors_match_oracle():
    g = grid2k()
    e, o = engine(g), Oracle(g)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    assert rc == 0
    v, th = e.voltages()
    p, q = e.injections()
    pf, qf, pt, qt = e.branch_flows()
    got = [p, q, pf, qf, pt, qt]
    at_gpu_state = o.results(v, th)
    for a, b in zip(got, at_gpu_state):
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())
    ov, oth, _, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    for a, b in zip(got, o.results(ov, oth)):
        assert np.abs(a - b).max() < 1e-6 * max(1.0, np.abs(b).max())
    e.close()


@pytest.mark.parametrize("exact", [True, False])
def test_current_magnitude_rows_stage_values(exact):
    g = with_current_rows(grid2k(), 150)
    e, o = engine(g), Oracle(g)
    rng = np.random.default_rng(3)
    v = g.v_true + 0.01 * rng.standard_normal(g.n_bus)
    th = g.theta_true + 0.01 * rng.standard_normal(g.n_bus)
    th[g.slack] = 0.0
    got = e.evaluate_at(v, th, exact=exact)
    ref = o.evaluate(v, th, g.z, exact=exact)
    assert np.array_equal(got["h_ptr"], ref["h_ptr"]) and np.array_equal(got["h_col"], ref["h_col"])
    assert np.allclose(got["hx"], ref["hx"], rtol=1e-12, atol=1e-12)
    scale = np.abs(ref["h_val"]).max()
    assert np.allclose(got["h_val"], ref["h_val"], rtol=1e-12, atol=1e-12 * scale)
    rs = np.abs(ref["rhs"]).max()
    assert np.allclose(got["rhs"], ref["rhs"], rtol=1e-10, atol=1e-10 * rs)
    e.close()


def test_current_magnitude_rows_solve_matches_oracle():
    g = with_current_rows(grid2k(), 150)
    e, o = engine(g), Oracle(g)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    v, th = e.voltages()
    ov, oth, ores, orr = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    assert res.status == ores.status == 0 and res.iterations == ores.iterations
    assert state_err(v, th, ov, oth) < STATE_TOL
    assert np.array_equal(e.bad_data(3.0), o.bad_data(orr, 3.0))
    e.close()


def test_huber_stall_option_matches_oracle():
    """Robust (Huber) solves with the reference's reweighting creep when gross
    errors sit on critical measurement pairs; the huber_stall option also
    stops when an iteration lowers the Huber objective by no more than that
    fraction.  Same stopping iteration and state as the oracle with the same
    rule; without it both run to the iteration cap."""
    g = SyntheticGrid(600, 840, 0x5E02, gross=0.02)
    e, o = engine(g, huber_stall=1e-5), Oracle(g)
    rc, res = e.solve_with(max_iterations=100, tolerance=1e-6, flat_start=True, robust=True, huber_gamma=1.5)
    v, th = e.voltages()
    ov, oth, ores, orr = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=100, tolerance=1e-6,
                               robust=True, gamma=1.5, huber_stall=1e-5)
    assert res.status == ores.status == 0
    assert res.iterations == ores.iterations < 100
    assert state_err(v, th, ov, oth) < STATE_TOL
    assert np.array_equal(e.bad_data(3.0), o.bad_data(orr, 3.0))
    e.set_option("huber_stall", 0.0)
    rc, res = e.solve_with(max_iterations=100, tolerance=1e-6, flat_start=True, robust=True, huber_gamma=1.5)
    ov, oth, ores, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=100, tolerance=1e-6, robust=True,
                             gamma=1.5)
    assert res.status == ores.status == 1 and res.iterations == ores.iterations == 100
    e.close()


def test_host_phase_times_in_stats():
    """SLE_ExStats carries the host time of the analysis, the schedule, the
    arena build with its copies and the graph captures (taken by the first
    solve); a reset clears them."""
    g = grid2k()
    e = engine(g)
    s = e.stats()
    assert s.analyses == 1 and s.analysis_ms > 0 and s.schedule_ms > 0 and s.upload_ms > 0
    assert s.capture_ms == 0
    e.solve_with(max_iterations=10, tolerance=1e-6, flat_start=True)
    s2 = e.stats()
    assert s2.capture_ms > 0 and s2.analysis_ms == s.analysis_ms
    e.reset_stats()
    s3 = e.stats()
    assert s3.analysis_ms == s3.schedule_ms == s3.upload_ms == s3.capture_ms == 0
    e.close()
