"""Seeded synthetic workloads (the generator lives in csrc/gen/segen.cpp).

Named workloads (seed = 0x5E00 + index):
  grid14      14 buses / 20 branches (spanning tree + 7 chords), taps on 3
              branches, |V| at 5 buses, P+Q injection at 9, both-end P+Q flow
              on 11 branches (67 rows); flat start, tol 1e-6, <= 20 iterations.
  grid10k     10,000 buses / 14,000 branches, |V| at 30 % of buses, P+Q
              injection at 60 %, both-end P+Q flows on 70 % of branches
              (54,200 rows), taps on 15 % of branches; flat start, then
              hot-start updates that re-noise 1 % of the rows each.
  grid200k    200,000 buses / 280,000 branches, same mix (1,084,000 rows),
              2 % gross errors of +-(10..30) sigma on telemetry rows, Huber
              gamma = 1.5.
  batch512    512 independent grids, n = round(30 (5000/30)^U) buses
              (log-uniform), round(1.4 n) branches, the grid10k mix; grid i
              seeded 0x5E03 ^ (i * 0x9E3779B97F4A7C15).
  fleet200    200 grids with n ~ Zipf(1.2) truncated to [30, 200000], the
              grid10k mix; grid i seeded 0x5E04 ^ (i * 0x9E3779B97F4A7C15).
"""
import ctypes

import numpy as np

from .native import SEGenParams, segen_lib

WORKLOADS = {
    "grid14": dict(index=0, n_bus=14, n_branch=20, n_vmag=5, n_inj=9, n_flow=11, n_tap=3, gross=0.0),
    "grid10k": dict(index=1, n_bus=10000, n_branch=14000, gross=0.0),
    "grid200k": dict(index=2, n_bus=200000, n_branch=280000, gross=0.02),
}


class SyntheticGrid:
    """One generated grid; arrays are numpy copies owned by this object."""

    def __init__(self, n_bus, n_branch, seed, n_vmag=-1, n_inj=-1, n_flow=-1, n_tap=-1, gross=0.0):
        self._lib = segen_lib()
        p = SEGenParams()
        self._lib.segen_default_params(ctypes.byref(p), int(n_bus), int(n_branch), ctypes.c_uint64(seed))
        p.n_vmag, p.n_inj, p.n_flow, p.n_tap = n_vmag, n_inj, n_flow, n_tap
        p.gross_frac = gross
        self._h = self._lib.segen_create(ctypes.byref(p))
        if not self._h:
            raise ValueError("invalid synthetic grid parameters")
        L = self._lib
        h = self._h
        self.seed = seed
        self.n_bus = L.segen_n_bus(h)
        self.n_branch = L.segen_n_branch(h)
        self.n_meas = L.segen_n_meas(h)
        self.slack = L.segen_slack(h)

        def arr(fn, n, dt):
            return np.ctypeslib.as_array(fn(h), shape=(n,)).astype(dt).copy() if n > 0 else np.zeros(0, dt)

        self.bus_type = arr(L.segen_bus_type, self.n_bus, np.int32)
        self.v_setpoint = arr(L.segen_v_setpoint, self.n_bus, np.float64)
        self.v_true = arr(L.segen_v_true, self.n_bus, np.float64)
        self.theta_true = arr(L.segen_theta_true, self.n_bus, np.float64)
        self.br_from = arr(L.segen_br_from, self.n_branch, np.int32)
        self.br_to = arr(L.segen_br_to, self.n_branch, np.int32)
        self.br_r = arr(L.segen_br_r, self.n_branch, np.float64)
        self.br_x = arr(L.segen_br_x, self.n_branch, np.float64)
        self.br_b = arr(L.segen_br_b, self.n_branch, np.float64)
        self.br_tap = arr(L.segen_br_tap, self.n_branch, np.float64)
        self.br_shift = arr(L.segen_br_shift, self.n_branch, np.float64)
        self.br_status = arr(L.segen_br_status, self.n_branch, np.int32)
        self.m_type = arr(L.segen_meas_type, self.n_meas, np.int32)
        self.m_loc = arr(L.segen_meas_loc, self.n_meas, np.int32)
        self.m_end = arr(L.segen_meas_end, self.n_meas, np.int32)
        self.m_sigma = arr(L.segen_meas_sigma, self.n_meas, np.float64)
        self.z = arr(L.segen_meas_z, self.n_meas, np.float64)
        self.gross = arr(L.segen_meas_gross, self.n_meas, np.int32)
        self.h_true = arr(L.segen_meas_htrue, self.n_meas, np.float64)

    def renoise(self, update, frac=0.01):
        """Hot-start telemetry update `update`: redraw the noise of a seeded
        fraction of rows; returns the full new z (also kept in self.z)."""
        out = np.empty(self.n_meas, np.float64)
        self._lib.segen_renoise(self._h, int(update), float(frac), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        self.z = out
        return out

    def close(self):
        if self._h:
            self._lib.segen_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


GOLDEN = 0x9E3779B97F4A7C15
MASK64 = (1 << 64) - 1


def grid_seed(base, i):
    return (base ^ ((i * GOLDEN) & MASK64)) & MASK64


def batch_sizes(count=512, seed=0x5E03, lo=30, hi=5000):
    L = segen_lib()
    return [L.segen_draw_loguniform(seed, i, lo, hi) for i in range(count)]


def fleet_sizes(count=200, seed=0x5E04, s=1.2, lo=30, hi=200000):
    L = segen_lib()
    return [L.segen_draw_zipf(seed, i, s, lo, hi) for i in range(count)]


def batch_grids(count=512, seed=0x5E03, lo=30, hi=5000):
    """The batched-form workload: `count` independent grids of log-uniform size."""
    return [SyntheticGrid(n, int(round(1.4 * n)), grid_seed(seed, i)) for i, n in enumerate(batch_sizes(count, seed, lo, hi))]


def fleet_grids(count=200, seed=0x5E04):
    """The serving-form fleet: `count` grids of Zipf(1.2) size in [30, 200000]."""
    return [SyntheticGrid(n, int(round(1.4 * n)), grid_seed(seed, i)) for i, n in enumerate(fleet_sizes(count, seed))]


def make(name):
    w = WORKLOADS[name]
    return SyntheticGrid(w["n_bus"], w["n_branch"], 0x5E00 + w["index"], n_vmag=w.get("n_vmag", -1),
                         n_inj=w.get("n_inj", -1), n_flow=w.get("n_flow", -1), n_tap=w.get("n_tap", -1),
                         gross=w.get("gross", 0.0))
