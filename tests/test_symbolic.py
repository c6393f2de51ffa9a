"""Symbolic analysis of the product (host C++ behind the C ABI) against the
oracle's independent definitions: bit-exact patterns, ordering validity,
elimination tree and supernode row structures."""
import numpy as np
import pytest

from grids import ieee14
from oracle.binding import Oracle
from state_estimation_with_cuda_gb300 import Estimator, workloads
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid


def load(g):
    e = Estimator()
    e.load_network(g)
    return e


def cases():
    return {
        "ieee14": ieee14(),
        "grid14": workloads.make("grid14"),
        "grid2k": SyntheticGrid(2000, 2800, 0x5E01),
        "open_branches": _with_open(SyntheticGrid(300, 420, 9)),
        "grid20k_open": _with_open(SyntheticGrid(20000, 28000, 0x5E77)),
        "islands": _with_open(SyntheticGrid(400, 560, 21), step=3),
    }


def _with_open(g, step=17):
    g.br_status = g.br_status.copy()
    g.br_status[::step] = 0
    return g


@pytest.fixture(scope="module", params=["ieee14", "grid14", "grid2k", "open_branches", "grid20k_open", "islands"])
def case(request):
    g = cases()[request.param]
    return g, load(g), Oracle(g)


def test_ybus_pattern_bit_exact(case):
    g, e, o = case
    ptr, col, _, _ = o.ybus()
    info = e.plan_info()
    p_ptr = np.empty(g.n_bus + 1, np.int32)
    p_col = np.empty(info.nnz_ybus, np.int32)
    e._check(e.lib.sle_ExGetYbus(e.h, p_ptr.ctypes.data_as(e.lib.sle_ExGetYbus.argtypes[1]),
                                 p_col.ctypes.data_as(e.lib.sle_ExGetYbus.argtypes[2]), None, None))
    assert np.array_equal(ptr, p_ptr)
    assert np.array_equal(col, p_col)


def test_jacobian_pattern_bit_exact(case):
    g, e, o = case
    ev = o.evaluate(g.v_setpoint, np.zeros(g.n_bus), g.z)
    info = e.plan_info()
    ptr = np.empty(g.n_meas + 1, np.int32)
    col = np.empty(info.nnz_h, np.int32)
    f = e.lib.sle_ExGetJacobian
    e._check(f(e.h, ptr.ctypes.data_as(f.argtypes[1]), col.ctypes.data_as(f.argtypes[2]), None, None, None))
    assert np.array_equal(ev["h_ptr"], ptr)
    assert np.array_equal(ev["h_col"], col)


def test_ordering_etree_and_supernodes(case):
    g, e, o = case
    s = e.symbolic()
    n = g.n_bus
    perm = s["bus_perm"]
    assert sorted(perm.tolist()) == list(range(n))
    # states expand bus by bus: theta then V, slack only V
    sop = s["state_of_ps"]
    assert sorted(sop.tolist()) == list(range(2 * n - 1))
    parent, colcount = o.symbolic(perm)
    pos = np.empty(n, np.int64)
    pos[perm] = np.arange(n)
    ps_start = np.zeros(n + 1, np.int64)
    for k in range(n):
        ps_start[k + 1] = ps_start[k] + (1 if perm[k] == g.slack else 2)
    c0 = s["sn_c0"]
    ns = len(c0) - 1
    bus_of_ps = np.repeat(np.arange(n), np.diff(ps_start))
    for sn in range(ns):
        b0, b1 = bus_of_ps[c0[sn]], bus_of_ps[c0[sn + 1] - 1] + 1
        rows = s["sn_rows"][s["sn_rows_off"][sn]:s["sn_rows_off"][sn + 1]]
        rbus = np.unique(bus_of_ps[rows])
        # own columns first, ascending rows
        assert np.all(np.diff(rows) > 0)
        assert np.array_equal(rows[:c0[sn + 1] - c0[sn]], np.arange(c0[sn], c0[sn + 1]))
        # every column's true structure is inside the supernode's rows
        last = b1 - 1
        assert len(rbus) == (b1 - b0 - 1) + colcount[last]  # rows = own cols + structure of the last col
        # parent supernode holds the etree parent of the last column
        p = parent[last]
        psn = s["sn_parent"][sn]
        if p < 0:
            assert psn == -1
        else:
            assert bus_of_ps[c0[psn]] <= p < bus_of_ps[c0[psn + 1] - 1] + 1
        for j in range(b0, b1 - 1):  # interior columns' parents stay inside the supernode
            assert j < parent[j] < b1


def test_plan_is_deterministic():
    g = SyntheticGrid(1500, 2100, 3)
    a = load(g).symbolic()
    b = load(g).symbolic()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_plan_statistics_grid10k():
    g = workloads.make("grid10k")
    info = load(g).plan_info()
    assert info.n_state == 19999
    assert info.nnz_l < 2_000_000  # fill-reducing ordering
    assert info.n_levels < 64
