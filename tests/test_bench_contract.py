"""bench.py's roofline arithmetic and its link to the committed ncu summary
(host logic; no GPU): the object carries the contract's keys, frac is
achieved / peak, achieved is the stage's algorithmic bytes over its time, and
the loaded-pass roofline finds its DRAM traffic in profiles/."""
import argparse
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def fake_info(n_bus):
    return argparse.Namespace(n_meas=5 * n_bus, n_bus=n_bus, n_state=2 * n_bus - 1, nnz_h=20 * n_bus,
                              nnz_ybus=4 * n_bus, n_gain_pairs=40 * n_bus, n_gain_targets=8 * n_bus,
                              lx_size=30 * n_bus, u_size=10 * n_bus)


@pytest.mark.parametrize("n_bus", [10000, 475607])
def test_roofline_object(n_bus):
    info = fake_info(n_bus)
    g = argparse.Namespace(m_type=np.array([2, 3, 4, 5, 1, 0] * (info.n_meas // 6), np.int32))
    leg = {"info": info,
           "stage_ms": {"evaluate": 0.5, "factor": 4.0, "rhs": 0.1, "solve": 2.0, "update": 0.05, "final": 0.02},
           "stage_calls": {"evaluate": 1, "factor": 1, "rhs": 1, "solve": 1, "update": 1, "final": 1}}
    r = bench.roofline(leg, g, True)
    for key in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert key in r
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    sb = bench.stage_bytes(info, g, 4)
    assert r["algorithmic_bytes_per_call"] == int(sb["factor"])  # the dominant stage here
    assert r["achieved"] == pytest.approx(sb["factor"] / 4.0e-3 / 1e9, rel=1e-3)
    assert abs(r["frac"] - r["achieved"] / r["peak"]) <= 1e-5  # frac is rounded to 5 decimals
    if n_bus > 100000:  # the batch union's stage reads its committed capture
        assert r["kernel"] == "union_front_factorisation"
        assert r["traffic"] == bench.profile_traffic("union_front_factorisation") > 0


def test_committed_traffic_close_to_algorithmic_bytes():
    # the capture of the loaded pass moved about the algorithmic bytes of the
    # stage (860 MB): nothing is re-read
    t = bench.profile_traffic("union_front_factorisation")
    assert t is not None and 0.8e9 < t < 0.9e9
