"""Python mirror of the SLE Engine C interface (reference include/sle_api.h).

`Estimator` wraps one SLE_Handle of libsle_gb300.so; method names follow the
sle_* functions (sle_AddBus -> add_bus, sle_Solve -> solve, ...), arguments
keep their meaning, and a non-OK status raises SLEError carrying the status
code and sle_GetLastError() text.  solve() returns the status and result
instead of raising, because MAX_ITERATIONS / DIVERGED / SINGULAR are
outcomes, not misuse.
"""
import ctypes

import numpy as np

from . import native as N

OK = 0
ERROR_INVALID_HANDLE = -1
ERROR_NOT_INITIALIZED = -2
ERROR_CUDA_FAILURE = -3
ERROR_INVALID_ARGUMENT = -4
ERROR_MODEL_INCOMPLETE = -5
ERROR_NOT_OBSERVABLE = -6
ERROR_SINGULAR_MATRIX = -7
ERROR_DIVERGED = -8
ERROR_MAX_ITERATIONS = -9
ERROR_OUT_OF_MEMORY = -10
ERROR_ELEMENT_NOT_FOUND = -11
ERROR_DUPLICATE_ID = -12
ERROR_CONFIG_FILE = -13

MODE_REALTIME, MODE_PRECISION = 0, 1
BUS_PQ, BUS_PV, BUS_SLACK = 0, 1, 2
MEAS_V_MAG, MEAS_V_ANGLE, MEAS_P_INJ, MEAS_Q_INJ, MEAS_P_FLOW, MEAS_Q_FLOW, MEAS_I_MAG, MEAS_P_PSEUDO, MEAS_Q_PSEUDO = range(9)


class SLEError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


def _b(s):
    return None if s is None else (s if isinstance(s, bytes) else s.encode())


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class Estimator:
    def __init__(self, config=None):
        self.lib = N.sle_lib()
        self.h = ctypes.c_void_p()
        if config is None:
            rc = self.lib.sle_Create(ctypes.byref(self.h))
        else:
            rc = self.lib.sle_CreateWithConfig(ctypes.byref(self.h), ctypes.byref(config))
        self._check(rc)

    # -- helpers -------------------------------------------------------------
    def _check(self, rc):
        if rc != OK:
            err = self.lib.sle_GetLastError(self.h)
            raise SLEError(rc, err.decode() if err else "error")
        return rc

    def close(self):
        if self.h:
            self.lib.sle_Destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- configuration ---------------------------------------------------------
    def get_config(self):
        c = N.SLE_Config()
        self._check(self.lib.sle_GetConfig(self.h, ctypes.byref(c)))
        return c

    def set_config(self, **kw):
        c = self.get_config()
        for k, v in kw.items():
            setattr(c, k, v)
        self._check(self.lib.sle_SetConfig(self.h, ctypes.byref(c)))

    def set_option(self, key, value):
        self._check(self.lib.sle_ExSetOption(self.h, _b(key), float(value)))

    def initialize(self):
        self._check(self.lib.sle_Initialize(self.h))

    # -- model -------------------------------------------------------------------
    def add_bus(self, id, base_kv=1.0, type=BUS_PQ, v_setpoint=1.0, p=0.0, q=0.0):
        self._check(self.lib.sle_AddBus(self.h, ctypes.byref(N.SLE_BusInfo(_b(id), base_kv, type, v_setpoint, p, q))))

    def add_branch(self, id, from_bus, to_bus, r, x, b=0.0, g=0.0, tap=1.0, shift=0.0, is_transformer=0, sd_id=None):
        info = N.SLE_BranchInfo(_b(id), _b(from_bus), _b(to_bus), r, x, b, g, tap, shift, is_transformer, _b(sd_id))
        self._check(self.lib.sle_AddBranch(self.h, ctypes.byref(info)))

    def add_measurement(self, id, type, location, sigma, branch_end=0, pt=1.0, ct=1.0, pseudo=0):
        info = N.SLE_MeasurementInfo(_b(id), type, _b(location), branch_end, sigma, pt, ct, pseudo)
        self._check(self.lib.sle_AddMeasurement(self.h, ctypes.byref(info)))

    def add_switch(self, id, branch_id, closed=True):
        self._check(self.lib.sle_AddSwitch(self.h, ctypes.byref(N.SLE_SwitchInfo(_b(id), _b(branch_id), int(bool(closed))))))

    def load_network(self, grid, z=None):
        """Bulk-load a SyntheticGrid (or any object with the same arrays)."""
        L = self.lib
        i32, f64 = np.int32, np.float64
        self._arrays = [np.ascontiguousarray(a, dt) for a, dt in (  # no copy when already contiguous and typed
            (grid.bus_type, i32), (grid.v_setpoint, f64), (grid.br_from, i32), (grid.br_to, i32), (grid.br_r, f64),
            (grid.br_x, f64), (grid.br_b, f64), (grid.br_tap, f64), (grid.br_shift, f64), (grid.br_status, i32),
            (grid.m_type, i32), (grid.m_loc, i32), (grid.m_end, i32), (grid.m_sigma, f64),
            (grid.z if z is None else z, f64))]
        a = self._arrays
        self._check(L.sle_ExLoadNetwork(self.h, grid.n_bus, _ip(a[0]), _dp(a[1]), grid.n_branch, _ip(a[2]), _ip(a[3]),
                                        _dp(a[4]), _dp(a[5]), _dp(a[6]), _dp(a[7]), _dp(a[8]), _ip(a[9]), grid.n_meas,
                                        _ip(a[10]), _ip(a[11]), _ip(a[12]), _dp(a[13]), _dp(a[14])))

    def load_ieee14(self):
        self._check(self.lib.sle_LoadIEEE14Bus(self.h))

    def upload_model(self):
        self._check(self.lib.sle_UploadModel(self.h))

    # -- telemetry -----------------------------------------------------------------
    def update_telemetry(self, z):
        z = np.ascontiguousarray(z, np.float64)
        self._check(self.lib.sle_UpdateTelemetry(self.h, _dp(z), len(z)))

    def update_measurement(self, id, value):
        self._check(self.lib.sle_UpdateMeasurement(self.h, _b(id), float(value)))

    def set_switch(self, sd_id, closed):
        self._check(self.lib.sle_SetSwitchStatus(self.h, _b(sd_id), int(bool(closed))))

    def apply_switch_changes(self):
        self._check(self.lib.sle_ApplySwitchChanges(self.h))

    def set_transformer_tap(self, branch_id, tap):
        self._check(self.lib.sle_SetTransformerTap(self.h, _b(branch_id), float(tap)))

    def set_phase_shift(self, branch_id, shift):
        self._check(self.lib.sle_SetTransformerPhaseShift(self.h, _b(branch_id), float(shift)))

    def set_branch_impedance(self, branch_id, r, x, b=0.0, g=0.0):
        self._check(self.lib.sle_SetBranchImpedance(self.h, _b(branch_id), float(r), float(x), float(b), float(g)))

    # -- estimation ------------------------------------------------------------------
    def solve(self, mode=MODE_PRECISION):
        r = N.SLE_Result()
        rc = self.lib.sle_Solve(self.h, mode, ctypes.byref(r))
        return rc, r

    def solve_with(self, max_iterations=20, tolerance=1e-6, flat_start=False, robust=False, huber_gamma=1.5,
                   mode=MODE_PRECISION, time_limit_ms=0.0):
        c = N.SLE_SolverConfig(mode, max_iterations, tolerance, huber_gamma, int(robust), int(flat_start), time_limit_ms)
        r = N.SLE_Result()
        rc = self.lib.sle_SolveWithConfig(self.h, ctypes.byref(c), ctypes.byref(r))
        return rc, r

    def flat_start(self):
        self._check(self.lib.sle_ApplyFlatStart(self.h))

    def check_observability(self):
        """(observable, islands): topological check, on the device once uploaded."""
        obs = ctypes.c_int32()
        isl = ctypes.c_int32()
        self._check(self.lib.sle_CheckObservability(self.h, ctypes.byref(obs), ctypes.byref(isl)))
        return bool(obs.value), isl.value

    # -- results ------------------------------------------------------------------------
    def counts(self):
        return (self.lib.sle_GetBusCount(self.h), self.lib.sle_GetBranchCount(self.h),
                self.lib.sle_GetMeasurementCount(self.h))

    def voltages(self):
        n = self.lib.sle_GetBusCount(self.h)
        v = np.empty(n, np.float64)
        t = np.empty(n, np.float64)
        self._check(self.lib.sle_GetVoltageMagnitudes(self.h, _dp(v), n))
        self._check(self.lib.sle_GetVoltageAngles(self.h, _dp(t), n))
        return v, t

    def residuals(self):
        m = self.lib.sle_GetMeasurementCount(self.h)
        r = np.empty(m, np.float64)
        self._check(self.lib.sle_GetResiduals(self.h, _dp(r), m))
        return r

    def injections(self):
        n = self.lib.sle_GetBusCount(self.h)
        p = np.empty(n, np.float64)
        q = np.empty(n, np.float64)
        self._check(self.lib.sle_GetPowerInjections(self.h, _dp(p), _dp(q), n))
        return p, q

    def branch_flows(self):
        nb = self.lib.sle_GetBranchCount(self.h)
        out = [np.empty(nb, np.float64) for _ in range(4)]
        self._check(self.lib.sle_GetBranchFlows(self.h, *[_dp(a) for a in out], nb))
        return out

    def objective(self):
        return self.lib.sle_GetObjective(self.h)

    def bad_data(self, threshold=0.0):
        m = self.lib.sle_GetMeasurementCount(self.h)
        idx = np.empty(max(m, 1), np.int32)
        cnt = ctypes.c_int32()
        self._check(self.lib.sle_IdentifyBadData(self.h, threshold, _ip(idx), m, ctypes.byref(cnt)))
        return idx[:cnt.value].copy()

    def last_error(self):
        err = self.lib.sle_GetLastError(self.h)
        return err.decode() if err else ""

    def stats(self):
        """Per-stage launch counts, Gauss-Newton iterations and solves of this
        handle (sle_ExGetStats)."""
        st = N.SLE_ExStats()
        self._check(self.lib.sle_ExGetStats(self.h, ctypes.byref(st)))
        return st

    def reset_stats(self):
        self._check(self.lib.sle_ExResetStats(self.h))

    # -- stage-level access (sle_ex.h) ------------------------------------------------------
    def schedule_info(self):
        """Kernel schedule of the current model and options (host-only before
        the first upload): fronts per phase, ready lists, panel steps."""
        info = N.SLE_ExScheduleInfo()
        self._check(self.lib.sle_ExGetScheduleInfo(self.h, ctypes.byref(info)))
        return info

    def plan_info(self):
        info = N.SLE_ExPlanInfo()
        self._check(self.lib.sle_ExGetPlanInfo(self.h, ctypes.byref(info)))
        return info

    def ybus(self):
        info = self.plan_info()
        ptr = np.empty(info.n_bus + 1, np.int32)
        col = np.empty(info.nnz_ybus, np.int32)
        g = np.empty(info.nnz_ybus, np.float64)
        b = np.empty(info.nnz_ybus, np.float64)
        self._check(self.lib.sle_ExGetYbus(self.h, _ip(ptr), _ip(col), _dp(g), _dp(b)))
        return ptr, col, g, b

    def evaluate_at(self, v, theta, exact=True):
        v = np.ascontiguousarray(v, np.float64)
        theta = np.ascontiguousarray(theta, np.float64)
        self._check(self.lib.sle_ExEvaluateAt(self.h, _dp(v), _dp(theta), int(exact)))
        info = self.plan_info()
        ptr = np.empty(info.n_meas + 1, np.int32)
        col = np.empty(info.nnz_h, np.int32)
        val = np.empty(info.nnz_h, np.float64)
        hx = np.empty(info.n_meas, np.float64)
        rhs = np.empty(info.n_state, np.float64)
        self._check(self.lib.sle_ExGetJacobian(self.h, _ip(ptr), _ip(col), _dp(val), _dp(hx), _dp(rhs)))
        return dict(h_ptr=ptr, h_col=col, h_val=val, hx=hx, rhs=rhs)

    def gain(self):
        info = self.plan_info()
        n = info.n_gain_targets
        rows = np.empty(n, np.int32)
        cols = np.empty(n, np.int32)
        vals = np.empty(n, np.float64)
        self._check(self.lib.sle_ExGetGain(self.h, _ip(rows), _ip(cols), _dp(vals)))
        return rows, cols, vals

    def factor_solve(self, rhs):
        rhs = np.ascontiguousarray(rhs, np.float64)
        x = np.empty_like(rhs)
        self._check(self.lib.sle_ExFactorSolve(self.h, _dp(rhs), _dp(x)))
        return x

    def symbolic(self):
        info = self.plan_info()
        bus_perm = np.empty(info.n_bus, np.int32)
        sop = np.empty(info.n_state, np.int32)
        c0 = np.empty(info.n_super + 1, np.int32)
        par = np.empty(info.n_super, np.int32)
        off = np.empty(info.n_super + 1, np.int64)
        self._check(self.lib.sle_ExGetSymbolic(self.h, _ip(bus_perm), _ip(sop), _ip(c0), _ip(par),
                                               off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None))
        rows = np.empty(int(off[-1]), np.int32)
        self._check(self.lib.sle_ExGetSymbolic(self.h, None, None, None, None, None, _ip(rows)))
        return dict(bus_perm=bus_perm, state_of_ps=sop, sn_c0=c0, sn_parent=par, sn_rows_off=off, sn_rows=rows)


class BatchEstimator(Estimator):
    """Many independent grids on one handle, solved together
    (sle_ExBatch*; no reference counterpart).  Grid i's result and iteration
    count equal those of solving grid i alone."""

    def __init__(self, config=None, mixed=True):
        super().__init__(config)
        if mixed:
            self.set_option("use_double_precision", 0)
        self._grid_arrays = []
        self.sizes = []

    def add_grid(self, grid, z=None):
        a = [np.ascontiguousarray(x) for x in (
            grid.bus_type.astype(np.int32), grid.v_setpoint.astype(np.float64), grid.br_from.astype(np.int32),
            grid.br_to.astype(np.int32), grid.br_r, grid.br_x, grid.br_b, grid.br_tap, grid.br_shift,
            grid.br_status.astype(np.int32), grid.m_type.astype(np.int32), grid.m_loc.astype(np.int32),
            grid.m_end.astype(np.int32), grid.m_sigma, np.asarray(grid.z if z is None else z, np.float64))]
        gid = ctypes.c_int32()
        self._check(self.lib.sle_ExBatchAddGrid(self.h, grid.n_bus, _ip(a[0]), _dp(a[1]), grid.n_branch, _ip(a[2]),
                                                _ip(a[3]), _dp(a[4]), _dp(a[5]), _dp(a[6]), _dp(a[7]), _dp(a[8]),
                                                _ip(a[9]), grid.n_meas, _ip(a[10]), _ip(a[11]), _ip(a[12]),
                                                _dp(a[13]), _dp(a[14]), ctypes.byref(gid)))
        self.sizes.append((grid.n_bus, grid.n_meas))
        return gid.value

    def grid_count(self):
        return self.lib.sle_ExBatchGridCount(self.h)

    def set_telemetry(self, gid, z):
        z = np.ascontiguousarray(z, np.float64)
        self._check(self.lib.sle_ExBatchUpdateTelemetry(self.h, int(gid), _dp(z), len(z)))

    def solve(self, grids=None, flat_start=False, max_iterations=20, tolerance=1e-6, robust=False, huber_gamma=1.5):
        """Solve the listed grids (default: all); returns SLE_ExGridResult[n]."""
        ids = np.arange(self.grid_count(), dtype=np.int32) if grids is None else np.ascontiguousarray(grids, np.int32)
        flat = np.full(len(ids), 1 if flat_start is True else 0, np.uint8) if isinstance(flat_start, bool) \
            else np.ascontiguousarray(flat_start, np.uint8)
        res = (N.SLE_ExGridResult * max(len(ids), 1))()
        self._check(self.lib.sle_ExBatchSolve(self.h, len(ids), _ip(ids),
                                              flat.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                              int(max_iterations), float(tolerance), int(bool(robust)),
                                              float(huber_gamma), res))
        return list(res)[:len(ids)]

    def state(self, gid):
        n = self.sizes[gid][0]
        v = np.empty(n, np.float64)
        t = np.empty(n, np.float64)
        self._check(self.lib.sle_ExBatchGetState(self.h, int(gid), _dp(v), _dp(t)))
        return v, t

    def set_branch_status(self, gid, branch, closed):
        self._check(self.lib.sle_ExBatchSetBranchStatus(self.h, int(gid), int(branch), int(bool(closed))))


def _grid_arrays(grid, z=None):
    return [np.ascontiguousarray(x) for x in (
        grid.bus_type.astype(np.int32), grid.v_setpoint.astype(np.float64), grid.br_from.astype(np.int32),
        grid.br_to.astype(np.int32), grid.br_r, grid.br_x, grid.br_b, grid.br_tap, grid.br_shift,
        grid.br_status.astype(np.int32), grid.m_type.astype(np.int32), grid.m_loc.astype(np.int32),
        grid.m_end.astype(np.int32), grid.m_sigma, np.asarray(grid.z if z is None else z, np.float64))]


class Server:
    """Serving runtime (sle_ExServer*; no reference counterpart): a resident
    fleet answering snapshots as they arrive, with continuous batching."""

    def __init__(self, mixed=True, max_iterations=20, tolerance=1e-6, bucket_bus=None, own_unit_bus=None,
                 memory_budget=0, robust=False, huber_gamma=1.5, device_id=0):
        """bucket_bus / own_unit_bus default to the autotuned values shipped in
        tuned.json (see tune.py), else (300, 2000, 20000, 0) / no own units."""
        from .tune import tuned_config

        best = tuned_config().get("serving", {}).get("best", {})
        if bucket_bus is None:
            bucket_bus = tuple(best.get("bucket_bus", (300, 2000, 20000, 0)))
        if own_unit_bus is None:
            own_unit_bus = int(best.get("own_unit_bus", 1 << 30))
        self.lib = N.sle_lib()
        c = N.SLE_ExServerConfig()
        self.lib.sle_ExServerDefaultConfig(ctypes.byref(c))
        c.use_double_precision = 0 if mixed else 1
        c.max_iterations = int(max_iterations)
        c.tolerance = float(tolerance)
        c.robust = int(bool(robust))
        c.huber_gamma = float(huber_gamma)
        for i in range(4):
            c.bucket_bus[i] = int(bucket_bus[i]) if i < len(bucket_bus) else 0
        c.own_unit_bus = int(own_unit_bus)
        c.memory_budget = int(memory_budget)
        c.device_id = int(device_id)
        self.s = ctypes.c_void_p()
        self._check(self.lib.sle_ExServerCreate(ctypes.byref(self.s), ctypes.byref(c)))
        self.sizes = []

    def _check(self, rc):
        if rc != OK:
            err = self.lib.sle_ExServerLastError(self.s) if self.s else None
            raise SLEError(rc, err.decode() if err else "error")
        return rc

    def add_grid(self, grid, z=None):
        a = _grid_arrays(grid, z)
        gid = ctypes.c_int32()
        self._check(self.lib.sle_ExServerAddGrid(self.s, grid.n_bus, _ip(a[0]), _dp(a[1]), grid.n_branch, _ip(a[2]),
                                                 _ip(a[3]), _dp(a[4]), _dp(a[5]), _dp(a[6]), _dp(a[7]), _dp(a[8]),
                                                 _ip(a[9]), grid.n_meas, _ip(a[10]), _ip(a[11]), _ip(a[12]),
                                                 _dp(a[13]), _dp(a[14]), ctypes.byref(gid)))
        self.sizes.append((grid.n_bus, grid.n_meas))
        return gid.value

    def start(self):
        self._check(self.lib.sle_ExServerStart(self.s))

    def submit(self, gid, z, branch=-1, closed=1, out=None):
        """Queue a snapshot; `out` = (v, theta) float64 arrays of the grid's
        bus count receive the state when the request completes (they must stay
        alive until wait() returns the ticket)."""
        z = np.ascontiguousarray(z, np.float64)
        t = ctypes.c_int64()
        if out is None:
            self._check(self.lib.sle_ExServerSubmit(self.s, int(gid), _dp(z), len(z), int(branch), int(closed),
                                                    ctypes.byref(t)))
        else:
            v, th = out
            n = self.sizes[gid][0]
            if v.dtype != np.float64 or th.dtype != np.float64 or len(v) < n or len(th) < n or \
                    not v.flags.c_contiguous or not th.flags.c_contiguous:
                raise ValueError("out buffers must be contiguous float64 arrays of the grid's bus count")
            self._check(self.lib.sle_ExServerSubmitEx(self.s, int(gid), _dp(z), len(z), int(branch), int(closed),
                                                      _dp(v), _dp(th), ctypes.byref(t)))
        return t.value

    def wait(self, ticket, timeout_ms=-1.0):
        r = N.SLE_ExServeResult()
        rc = self.lib.sle_ExServerWait(self.s, int(ticket), float(timeout_ms), ctypes.byref(r))
        if rc < 0:
            self._check(rc)
        return r if rc == 1 else None

    def state(self, gid):
        n = self.sizes[gid][0]
        v = np.empty(n, np.float64)
        t = np.empty(n, np.float64)
        self._check(self.lib.sle_ExServerGetState(self.s, int(gid), _dp(v), _dp(t)))
        return v, t

    def stats(self):
        st = N.SLE_ExServerStats()
        self._check(self.lib.sle_ExServerGetStats(self.s, ctypes.byref(st)))
        return st

    def close(self):
        if self.s:
            self.lib.sle_ExServerDestroy(self.s)
            self.s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
