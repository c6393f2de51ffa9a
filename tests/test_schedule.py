"""Kernel schedule (host logic, no GPU): which fronts each factorisation phase
takes, the per-grid warp-phase decision, and the order of the
level-synchronous part.  sle_ExGetScheduleInfo builds the schedule on the
host before the first upload.

* By default every grid with fronts whose subtree is at most 32 wide runs
  them in the warp phase (one front per warp); the option forces it on or
  off.
* In a batch the decision is per grid: the batch's warp fronts are exactly
  those of its grids that use the phase alone (each grid runs the kernels it
  runs alone).
* Every front belongs to exactly one phase and one backward sweep.
* The mixed pipeline's tiled fronts (wider than 224) become dataflow items:
  per 32-column step, one panel item per 128 rows below the diagonal block
  and one update item per 32 x 32 tile of the trailing lower triangle.
* The synchronous levels are ordered by depth or by height, whichever needs
  fewer launches; in a batch, depth lines up the grids' tiled fronts so the
  union needs far fewer panel steps than its grids one after another.
"""
import pytest

from state_estimation_with_cuda_gb300 import BatchEstimator, Estimator
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid, grid_seed

def schedule(grids, warp=None, mixed=True, **options):
    if len(grids) == 1:
        e = Estimator()
        e.set_option("use_double_precision", 0 if mixed else 1)
    else:
        e = BatchEstimator(mixed=mixed)
    if warp is not None:
        e.set_option("warp_fronts", warp)
    for k, v in options.items():
        e.set_option(k, v)
    if len(grids) == 1:
        e.load_network(grids[0])
    else:
        for g in grids:
            e.add_grid(g)
    si, pi = e.schedule_info(), e.plan_info()
    e.close()
    return si, pi


def check_partition(si, pi):
    assert si.n_warp + si.n_phase_a + si.n_phase_b + si.n_sync == pi.n_super
    assert si.down_n + si.down_warp_n == pi.n_super
    assert si.down_warp_n == si.n_warp
    assert si.warp_ready <= si.n_warp and si.a_ready <= si.n_phase_a and si.b_ready <= si.n_phase_b


@pytest.fixture(scope="module")
def grids():
    small = SyntheticGrid(2000, 2800, grid_seed(0x5E51, 0))
    big = SyntheticGrid(20000, 28000, grid_seed(0x5E51, 1))
    return small, big


def test_warp_phase_default_and_option(grids):
    small, big = grids
    s0, sp = schedule([small])
    b0, bp = schedule([big])
    for si, pi in ((s0, sp), (b0, bp)):
        check_partition(si, pi)
    # on by default for any grid with warp-able fronts
    assert s0.n_warp > 0 and s0.warp_ready > 0
    assert b0.n_warp > s0.n_warp
    s1, _ = schedule([small], warp=1)
    s_off, _ = schedule([small], warp=0)
    b_off, _ = schedule([big], warp=0)
    assert s1.n_warp == s0.n_warp and s1.warp_ready == s0.warp_ready
    assert s_off.n_warp == 0 and s_off.n_phase_a > s0.n_phase_a
    assert b_off.n_warp == 0 and b_off.n_phase_a > b0.n_phase_a
    # switching the phase moves fronts between the dataflow phases only
    assert s_off.n_sync == s0.n_sync and b_off.n_sync == b0.n_sync


def test_batch_decides_the_warp_phase_per_grid(grids):
    small, big = grids
    s0, _ = schedule([small])
    b0, _ = schedule([big])
    u, up = schedule([small, big])
    check_partition(u, up)
    assert u.n_warp == b0.n_warp + s0.n_warp
    assert u.n_phase_a == b0.n_phase_a + s0.n_phase_a
    assert u.warp_ready == b0.warp_ready + s0.warp_ready
    # forced off, no grid's fronts join
    s_off, _ = schedule([small], warp=0)
    b_off, _ = schedule([big], warp=0)
    u_off, _ = schedule([small, big], warp=0)
    assert u_off.n_warp == 0
    assert u_off.n_phase_a == s_off.n_phase_a + b_off.n_phase_a


def test_synchronous_order_is_the_cheaper_and_aligns_a_batch():
    h1 = SyntheticGrid(60000, 84000, grid_seed(0x5E51, 2))
    h2 = SyntheticGrid(50000, 70000, grid_seed(0x5E51, 3))
    a, _ = schedule([h1])
    b, _ = schedule([h2])
    u, up = schedule([h1, h2])
    check_partition(u, up)
    for si in (a, b, u):
        assert si.panel_steps > 0
        assert si.by_depth == (si.launches_by_depth < si.launches_by_height)
        assert min(si.launches_by_depth, si.launches_by_height) > 0
    # both grids' tiled fronts sit just below their roots: by depth they share
    # panel steps instead of running one after the other
    assert u.by_depth == 1
    assert u.panel_steps < a.panel_steps + b.panel_steps
    assert u.panel_steps <= max(a.panel_steps, b.panel_steps) + min(a.panel_steps, b.panel_steps) // 2


def expected_tile_tasks(est):
    """Panel chunks and update tiles of every front wider than 224."""
    sym = est.symbolic()
    c0, off = sym["sn_c0"], sym["sn_rows_off"]
    n = 0
    for s in range(len(c0) - 1):
        f, nc = int(off[s + 1] - off[s]), int(c0[s + 1] - c0[s])
        if f <= 224:
            continue
        ut = (f + 31) // 32
        for p in range((nc + 31) // 32):
            q0 = 32 * p + min(32, nc - 32 * p)
            n += max(1, (f - q0 + 127) // 128)
            if q0 < f:
                n += sum(ut - tj for tj in range(q0 // 32, ut))
    return n


def test_tiled_fronts_as_dataflow_items(grids):
    _, big = grids
    e = Estimator()
    e.set_option("use_double_precision", 0)
    e.set_option("tile_flow", 1)
    e.load_network(big)
    want = expected_tile_tasks(e)
    si = e.schedule_info()
    e.close()
    assert want > 0 and si.tile_tasks == want  # -1 would mean an out-of-order dependency
    off, _ = schedule([big])  # the default: per-step launches
    fp64, _ = schedule([big], mixed=False, tile_flow=1)
    assert off.tile_tasks == 0 and fp64.tile_tasks == 0
    # the same fronts, the same steps: only how they are launched changes
    assert off.panel_steps == si.panel_steps
