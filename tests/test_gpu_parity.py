"""GPU parity: every stage of the sm_103a pipeline, called through the C ABI,
against the CPU FP64 oracle on the same seeded inputs.

Tolerances (FP64 both sides; the GPU contracts multiply-adds and uses its own
sincos, so bits may differ in the last places):
  Ybus, h(x), Jacobian values     rtol 1e-12 (atol 1e-12 x row scale)
  gain entries, b = H^T W r       rtol 1e-10 of the largest entry
  G x = b                         rtol 1e-9 (relative to |x|_inf)
  converged |V|, theta            1e-8 pu / rad, identical iteration counts
  patterns, bad-data flags        bit-exact
"""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import gpu_available
from grids import ieee14, observable_ieee14, synthetic_state
from oracle.binding import Oracle
from state_estimation_with_cuda_gb300 import Estimator, workloads
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-8


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.fail("GPU tests need a CUDA device; the product has no CPU fallback")


def grid(name):
    if name == "ieee14obs":
        g = observable_ieee14()
        v, th = synthetic_state(g, seed=3)
        o = Oracle(g)
        g.z = o.evaluate(v, th, g.z)["hx"] + 0.001 * np.random.default_rng(0).standard_normal(g.n_meas)
        return g
    if name == "grid2k":
        return SyntheticGrid(2000, 2800, 0x5E01)
    return workloads.make(name)


def engine(g, **options):
    e = Estimator()
    for k, v in options.items():
        e.set_option(k, v)
    e.load_network(g)
    e.upload_model()
    return e


@pytest.mark.parametrize("name", ["grid14", "ieee14obs", "grid2k"])
def test_ybus_values(name):
    g = grid(name)
    e, o = engine(g), Oracle(g)
    ptr, col, gv, bv = e.ybus()
    optr, ocol, ogv, obv = o.ybus()
    assert np.array_equal(ptr, optr) and np.array_equal(col, ocol)
    assert np.allclose(gv, ogv, rtol=1e-13, atol=1e-12)
    assert np.allclose(bv, obv, rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("name", ["grid14", "ieee14obs", "grid2k"])
@pytest.mark.parametrize("exact", [True, False])
def test_measurement_function_and_jacobian(name, exact):
    g = grid(name)
    e, o = engine(g), Oracle(g)
    v, th = synthetic_state(g)
    got = e.evaluate_at(v, th, exact=exact)
    ref = o.evaluate(v, th, g.z, exact=exact)
    assert np.array_equal(got["h_ptr"], ref["h_ptr"]) and np.array_equal(got["h_col"], ref["h_col"])
    assert np.allclose(got["hx"], ref["hx"], rtol=1e-12, atol=1e-12)
    scale = np.abs(ref["h_val"]).max()
    assert np.allclose(got["h_val"], ref["h_val"], rtol=1e-12, atol=1e-12 * scale)
    rs = np.abs(ref["rhs"]).max()
    assert np.allclose(got["rhs"], ref["rhs"], rtol=1e-10, atol=1e-10 * rs)


@pytest.mark.parametrize("name", ["grid14", "grid2k"])
@pytest.mark.parametrize("exact", [True, False])
def test_paired_evaluation_matches_oracle(name, exact):
    """P rows evaluated with their Q twins (one thread per pair, shared angle
    and admittance terms; the default from 2^18 rows on), forced here on small
    grids: the same h(x), H and gradient as the oracle, and as the row-per-
    thread evaluation within rounding."""
    g = grid(name)
    e, e1, o = engine(g, eval_pair_rows=0), engine(g), Oracle(g)
    v, th = synthetic_state(g)
    got = e.evaluate_at(v, th, exact=exact)
    single = e1.evaluate_at(v, th, exact=exact)
    ref = o.evaluate(v, th, g.z, exact=exact)
    assert np.array_equal(got["h_ptr"], ref["h_ptr"]) and np.array_equal(got["h_col"], ref["h_col"])
    assert np.allclose(got["hx"], ref["hx"], rtol=1e-12, atol=1e-12)
    scale = np.abs(ref["h_val"]).max()
    assert np.allclose(got["h_val"], ref["h_val"], rtol=1e-12, atol=1e-12 * scale)
    assert np.allclose(got["h_val"], single["h_val"], rtol=1e-14, atol=1e-14 * scale)
    rs = np.abs(ref["rhs"]).max()
    assert np.allclose(got["rhs"], ref["rhs"], rtol=1e-10, atol=1e-10 * rs)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    ov, oth, ores, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    v2, th2 = e.voltages()
    assert rc == 0 and res.status == ores.status == 0 and res.iterations == ores.iterations
    assert max(np.abs(v2 - ov).max(), np.abs(th2 - oth).max()) < 1e-8
    e.close()
    e1.close()


@pytest.mark.parametrize("name", ["grid14", "grid2k", "grid10k"])
def test_gain_and_factor_solve(name):
    g = grid(name)
    e, o = engine(g), Oracle(g)
    v, th = synthetic_state(g)
    e.evaluate_at(v, th, exact=True)
    ref = o.evaluate(v, th, g.z, exact=True)
    n = 2 * g.n_bus - 1
    r, c, val = e.gain()
    orr, oc, oval = o.gain()
    # the GPU stores the lower triangle in its elimination order; compare as
    # lower triangles in state order
    lo, hi = np.minimum(r, c), np.maximum(r, c)
    Gp = sp.coo_matrix((val, (hi, lo)), shape=(n, n)).tocsr()
    Go = sp.coo_matrix((oval, (orr, oc)), shape=(n, n)).tocsr()
    Gp.sort_indices()
    Go.sort_indices()
    assert np.array_equal(Gp.indptr, Go.indptr) and np.array_equal(Gp.indices, Go.indices)  # same stored pattern
    d = abs(Gp - Go).max()
    assert d <= 1e-10 * abs(Go).max(), d
    st, xo = o.solve_gain(ref["rhs"])
    assert st == 0
    xg = e.factor_solve(ref["rhs"])
    assert np.abs(xg - xo).max() <= 1e-9 * max(np.abs(xo).max(), 1e-30)


@pytest.mark.parametrize("name", ["grid14", "ieee14obs", "grid2k", "grid10k"])
def test_flat_start_solve_matches_oracle(name):
    g = grid(name)
    e, o = engine(g), Oracle(g)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    v, th = e.voltages()
    ov, oth, ores, orr = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    assert res.status == ores.status == 0
    assert rc == 0
    assert res.iterations == ores.iterations
    assert np.abs(v - ov).max() < STATE_TOL
    assert np.abs(th - oth).max() < STATE_TOL
    assert res.objective == pytest.approx(ores.objective, rel=1e-9)
    assert np.allclose(e.residuals(), orr, rtol=1e-8, atol=1e-9)
    assert np.array_equal(e.bad_data(3.0), o.bad_data(orr, 3.0))


def test_hot_start_sequence_grid10k():
    g = grid("grid10k")
    e, o = engine(g), Oracle(g)
    e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    ov, oth, _, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    for u in range(4):
        z = g.renoise(u)
        e.update_telemetry(z)
        rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=False)
        ov, oth, ores, _ = o.wls(z, ov, oth, max_iterations=20, tolerance=1e-6, flat_start=False)
        v, th = e.voltages()
        assert res.status == ores.status == 0
        assert res.iterations == ores.iterations
        assert max(np.abs(v - ov).max(), np.abs(th - oth).max()) < STATE_TOL


def test_robust_huber_matches_oracle():
    g = SyntheticGrid(600, 840, 2024, gross=0.02)
    e, o = engine(g), Oracle(g)
    rc, res = e.solve_with(max_iterations=30, tolerance=1e-6, flat_start=True, robust=True, huber_gamma=1.5)
    v, th = e.voltages()
    ov, oth, ores, orr = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=30, tolerance=1e-6, robust=True,
                               gamma=1.5)
    assert res.status == ores.status
    assert res.iterations == ores.iterations
    assert max(np.abs(v - ov).max(), np.abs(th - oth).max()) < STATE_TOL
    flagged = e.bad_data(3.0)
    assert np.array_equal(flagged, o.bad_data(orr, 3.0))
    # most injected gross errors are among the flagged rows
    gross = np.nonzero(g.gross)[0]
    assert np.isin(gross, flagged).mean() > 0.8


def test_reference_fixture_is_singular_on_gpu():
    g = ieee14()
    e = Estimator()
    e.load_ieee14()
    e.update_telemetry(g.z)
    rc, res = e.solve()
    assert rc == -7 and res.status == 3  # SLE_ERROR_SINGULAR_MATRIX, like the oracle


def test_solve_is_deterministic():
    g = grid("grid2k")
    out = []
    for _ in range(2):
        e = engine(g)
        e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
        out.append(np.concatenate(e.voltages()))
        e.close()
    assert np.array_equal(out[0], out[1])


def mixed_engine(g, refine=0):
    e = Estimator()
    e.set_option("use_double_precision", 0)
    e.set_option("refine_steps", refine)
    e.load_network(g)
    e.upload_model()
    return e


@pytest.mark.parametrize("name", ["grid14", "ieee14obs", "grid2k", "grid10k"])
def test_mixed_precision_flat_start_within_1e6(name):
    g = grid(name)
    e, o = mixed_engine(g), Oracle(g)
    rc, res = e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    v, th = e.voltages()
    ov, oth, ores, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    assert res.status == ores.status == 0
    assert abs(res.iterations - ores.iterations) <= 1
    assert max(np.abs(v - ov).max(), np.abs(th - oth).max()) < 1e-6


@pytest.mark.parametrize("refine", [0, 1])
def test_mixed_precision_hot_start_sequence_grid10k(refine):
    g = grid("grid10k")
    e, o = mixed_engine(g, refine), Oracle(g)
    e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
    ov, oth, _, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    for u in range(4):
        z = g.renoise(u)
        e.update_telemetry(z)
        rc, res = e.solve_with(max_iterations=20, tolerance=1e-6)
        ov, oth, ores, _ = o.wls(z, ov, oth, max_iterations=20, tolerance=1e-6, flat_start=False)
        v, th = e.voltages()
        assert res.status == 0
        assert max(np.abs(v - ov).max(), np.abs(th - oth).max()) < 1e-6


def _degree_one_branches(g, count):
    deg = np.bincount(np.concatenate([g.br_from, g.br_to]), minlength=g.n_bus)
    leaves = [k for k in range(g.n_branch) if deg[g.br_from[k]] == 1 or deg[g.br_to[k]] == 1]
    return leaves[:count]


@pytest.mark.parametrize("n_open", [0, 1, 5])
def test_islands_on_device_match_host(n_open):
    """Opening n branches that each isolate a leaf bus leaves n + 1 islands;
    the device labelling (uploaded model) agrees with the host check."""
    g = SyntheticGrid(3000, 4200, 0x5E31)
    status = np.ones(g.n_branch, np.int32)
    for k in _degree_one_branches(g, n_open):
        status[k] = 0
    g.br_status = status
    e = Estimator()
    e.load_network(g)
    host = e.check_observability()
    e.upload_model()
    dev = e.check_observability()
    assert dev == host
    assert dev[1] == n_open + 1
    e.close()
