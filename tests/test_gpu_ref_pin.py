"""GPU: the CPU oracle and this library pinned to the reference's own code.

The reference's element kernels -- computeBranchAdmittanceKernel /
countYbusNonzerosKernel / initYbusDiagonalKernel / fillYbusKernel
(sparse_matrix.cu:321-492, orchestrated as buildYbus, :498-626),
computePowerInjectionsKernel / computeBranchFlowsKernel /
computeBranchCurrentsKernel / computeMeasurementFunctionKernel
(kernels.cu:129-489) and computeJacobianValuesKernel
(sparse_matrix.cu:1627-2147) -- are compiled unchanged from its sources
(oracle/build_ref.py, the reference's FP32 build: its FP64 switch does not
compile) and run on the GPU by oracle/refpin.cpp.  Their Ybus, h(x) and
Jacobian rows are compared with the CPU FP64 oracle's `ref` mode and with
this library's stage outputs at the same state.

Grids: every bus has at most four branches and no parallel branches, so no
injection row overflows the reference's fixed 10 Jacobian slots (its rows
for buses of degree >= 5 are silently truncated, sparse_matrix.cu:1574-1595).
The reference's Ybus rows come in atomic arrival order; entries are matched
by column.

Tolerances (the reference computes in FP32; a formula difference -- a sign,
a dropped shunt, the 1/a^4 from-end charging quirk -- moves values by 1e-3
or more at these states):
  Ybus entries    1e-5 relative to the largest |Y| entry
  h(x)            1e-4 pu
  Jacobian        1e-5 relative to the row's largest |value|, plus 1e-5
"""
import numpy as np
import pytest

from conftest import gpu_available
from grids import bounded_degree_grid
from oracle.binding import Oracle, RefPin
from state_estimation_with_cuda_gb300 import Estimator

pytestmark = pytest.mark.gpu

Y_TOL = 1e-5
H_TOL = 1e-4
J_TOL = 1e-5


@pytest.fixture(scope="module")
def ref():
    if not gpu_available():
        pytest.fail("GPU tests need a CUDA device; the product has no CPU fallback")
    if not RefPin.available():
        pytest.skip("the reference's kernels are not built (oracle/build_ref.py needs the reference sources)")
    return RefPin()


GRIDS = {"deg4_300": (300, 1), "deg4_2000": (2000, 2)}


def grid(name):
    n, seed = GRIDS[name]
    return bounded_degree_grid(n, seed)


def state(g, seed=9):
    rng = np.random.default_rng(seed)
    v = g.v_true + 0.01 * rng.standard_normal(g.n_bus)
    th = g.theta_true + 0.01 * rng.standard_normal(g.n_bus)
    th[g.slack] = 0.0
    return v, th


def rows_by_column(ptr, col, *vals):
    out = []
    for i in range(len(ptr) - 1):
        out.append({int(col[e]): tuple(float(v[e]) for v in vals) for e in range(ptr[i], ptr[i + 1])})
    return out


@pytest.mark.parametrize("name", list(GRIDS))
def test_ybus_matches_reference_kernels(ref, name):
    g = grid(name)
    rptr, rcol, rg, rb = ref.ybus(g)
    optr, ocol, og, ob = Oracle(g).ybus()
    assert np.array_equal(rptr, optr)  # diagonal + one entry per closed branch end
    assert np.array_equal(rcol[rptr[:-1]], np.arange(g.n_bus))  # diagonal first in every row
    scale = max(np.abs(og).max(), np.abs(ob).max())
    R, O = rows_by_column(rptr, rcol, rg, rb), rows_by_column(optr, ocol, og, ob)
    for i in range(g.n_bus):
        assert R[i].keys() == O[i].keys(), i
        for c in O[i]:
            assert abs(R[i][c][0] - O[i][c][0]) <= Y_TOL * scale, (i, c)
            assert abs(R[i][c][1] - O[i][c][1]) <= Y_TOL * scale, (i, c)
    # the library's device Ybus, same pattern in canonical order
    e = Estimator()
    e.load_network(g)
    e.upload_model()
    eptr, ecol, eg, eb = e.ybus()
    E = rows_by_column(eptr, ecol, eg, eb)
    for i in range(g.n_bus):
        assert E[i].keys() == R[i].keys(), i
        for c in R[i]:
            assert abs(E[i][c][0] - R[i][c][0]) <= Y_TOL * scale and abs(E[i][c][1] - R[i][c][1]) <= Y_TOL * scale
    e.close()


@pytest.mark.parametrize("name", list(GRIDS))
def test_measurement_function_and_reference_jacobian_match_reference_kernels(ref, name):
    g = grid(name)
    v, th = state(g)
    rh, rcol, rval = ref.evaluate(g, v, th)
    o = Oracle(g).evaluate(v, th, g.z, exact=False)
    e = Estimator()
    e.load_network(g)
    e.upload_model()
    lib = e.evaluate_at(v, th, exact=False)
    e.close()
    # h(x): injections, flows at both ends, |I|, |V|
    assert np.abs(rh - o["hx"]).max() <= H_TOL
    assert np.abs(rh - lib["hx"]).max() <= H_TOL
    assert np.array_equal(lib["h_ptr"], o["h_ptr"]) and np.array_equal(lib["h_col"], o["h_col"])
    for q in range(g.n_meas):
        got = {}
        for c, x in zip(rcol[q], rval[q]):
            if c >= 0:
                got[int(c)] = got.get(int(c), 0.0) + float(x)
        a, b = o["h_ptr"][q], o["h_ptr"][q + 1]
        want = dict(zip(o["h_col"][a:b].tolist(), o["h_val"][a:b].tolist()))
        mine = dict(zip(lib["h_col"][a:b].tolist(), lib["h_val"][a:b].tolist()))
        assert got.keys() == want.keys(), (q, g.m_type[q], sorted(got), sorted(want))
        scale = max(abs(x) for x in want.values()) if want else 0.0
        for c in want:
            assert abs(got[c] - want[c]) <= J_TOL * scale + J_TOL, (q, int(g.m_type[q]), c, got[c], want[c])
            assert abs(got[c] - mine[c]) <= J_TOL * scale + J_TOL, (q, int(g.m_type[q]), c, got[c], mine[c])
