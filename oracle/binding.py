"""ctypes binding of oracle/_build/liboracle.so (CPU FP64 oracle).

Test infrastructure: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py only.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
I = ctypes.c_int32
D = ctypes.c_double
P = ctypes.POINTER


class OrParams(ctypes.Structure):
    _fields_ = [("max_iterations", I), ("tolerance", D), ("exact_jacobian", I), ("gain_policy", I),
                ("robust", I), ("huber_gamma", D), ("flat_start", I), ("realtime", I), ("vmin", D), ("vmax", D),
                ("huber_stall", D)]


class OrResult(ctypes.Structure):
    _fields_ = [("status", I), ("iterations", I), ("max_mismatch", D), ("objective", D),
                ("largest_residual", D), ("largest_idx", I), ("pad", I)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle not built: %s" % path)
        L = ctypes.CDLL(path)
        L.or_create.restype = ctypes.c_void_p
        L.or_create.argtypes = [I, P(I), P(D), I, P(I), P(I), P(D), P(D), P(D), P(D), P(D), P(I), I, P(I), P(I), P(I),
                                P(D)]
        L.or_destroy.argtypes = [ctypes.c_void_p]
        L.or_ybus.restype = I
        L.or_ybus.argtypes = [ctypes.c_void_p, P(I), P(I), P(D), P(D)]
        L.or_nnz_h.restype = ctypes.c_int64
        L.or_nnz_h.argtypes = [ctypes.c_void_p]
        L.or_evaluate.argtypes = [ctypes.c_void_p, P(D), P(D), P(D), I, I, D, P(D), P(D), P(I), P(I), P(D), P(D),
                                  P(D), P(D)]
        L.or_gain.restype = ctypes.c_int64
        L.or_gain.argtypes = [ctypes.c_void_p, P(I), P(I), P(D)]
        L.or_solve_gain.restype = I
        L.or_solve_gain.argtypes = [ctypes.c_void_p, P(D), P(D)]
        L.or_wls.argtypes = [ctypes.c_void_p, P(D), P(D), P(D), P(OrParams), P(OrResult), P(D)]
        L.or_bad_data.restype = I
        L.or_bad_data.argtypes = [ctypes.c_void_p, P(D), D, P(I), I]
        L.or_ordering.argtypes = [ctypes.c_void_p, P(I)]
        L.or_symbolic.argtypes = [ctypes.c_void_p, P(I), P(I), P(I)]
        L.or_results.argtypes = [ctypes.c_void_p, P(D), P(D), P(D), P(D), P(D), P(D), P(D), P(D)]
        L.or_threads.restype = I
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(P(D))


def _ip(a):
    return a.ctypes.data_as(P(I))


class Oracle:
    """One grid in the CPU oracle, built from the same SoA arrays the GPU gets."""

    def __init__(self, grid):
        L = lib()
        self.L = L
        self.n_bus, self.n_branch, self.n_meas = grid.n_bus, grid.n_branch, grid.n_meas
        self.n_state = 2 * grid.n_bus - 1
        self._keep = [np.ascontiguousarray(a) for a in (
            grid.bus_type.astype(np.int32), grid.v_setpoint.astype(np.float64), grid.br_from.astype(np.int32),
            grid.br_to.astype(np.int32), np.asarray(grid.br_r, np.float64), np.asarray(grid.br_x, np.float64),
            np.asarray(grid.br_b, np.float64), np.asarray(grid.br_tap, np.float64),
            np.asarray(grid.br_shift, np.float64), grid.br_status.astype(np.int32), grid.m_type.astype(np.int32),
            grid.m_loc.astype(np.int32), grid.m_end.astype(np.int32), np.asarray(grid.m_sigma, np.float64))]
        k = self._keep
        self.h = L.or_create(grid.n_bus, _ip(k[0]), _dp(k[1]), grid.n_branch, _ip(k[2]), _ip(k[3]), _dp(k[4]),
                             _dp(k[5]), _dp(k[6]), _dp(k[7]), _dp(k[8]), _ip(k[9]), grid.n_meas, _ip(k[10]),
                             _ip(k[11]), _ip(k[12]), _dp(k[13]))

    def close(self):
        if self.h:
            self.L.or_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ybus(self):
        nnz = self.L.or_ybus(self.h, None, None, None, None)
        ptr = np.empty(self.n_bus + 1, np.int32)
        col = np.empty(nnz, np.int32)
        g = np.empty(nnz)
        b = np.empty(nnz)
        self.L.or_ybus(self.h, _ip(ptr), _ip(col), _dp(g), _dp(b))
        return ptr, col, g, b

    def evaluate(self, v, theta, z, exact=True, robust=False, gamma=1.5):
        nnz = self.L.or_nnz_h(self.h)
        out = dict(hx=np.empty(self.n_meas), r=np.empty(self.n_meas), h_ptr=np.empty(self.n_meas + 1, np.int32),
                   h_col=np.empty(nnz, np.int32), h_val=np.empty(nnz), w_eff=np.empty(self.n_meas),
                   rhs=np.empty(self.n_state))
        J = ctypes.c_double()
        v = np.ascontiguousarray(v, np.float64)
        theta = np.ascontiguousarray(theta, np.float64)
        z = np.ascontiguousarray(z, np.float64)
        self.L.or_evaluate(self.h, _dp(v), _dp(theta), _dp(z), int(exact), int(robust), gamma, _dp(out["hx"]),
                           _dp(out["r"]), _ip(out["h_ptr"]), _ip(out["h_col"]), _dp(out["h_val"]),
                           _dp(out["w_eff"]), _dp(out["rhs"]), ctypes.byref(J))
        out["objective"] = J.value
        return out

    def gain(self):
        n = self.L.or_gain(self.h, None, None, None)
        rows = np.empty(n, np.int32)
        cols = np.empty(n, np.int32)
        vals = np.empty(n)
        self.L.or_gain(self.h, _ip(rows), _ip(cols), _dp(vals))
        return rows, cols, vals

    def solve_gain(self, rhs):
        rhs = np.ascontiguousarray(rhs, np.float64)
        x = np.empty_like(rhs)
        st = self.L.or_solve_gain(self.h, _dp(rhs), _dp(x))
        return st, x

    def wls(self, z, v, theta, max_iterations=20, tolerance=1e-6, exact=True, gain_policy=0, robust=False,
            gamma=1.5, flat_start=True, realtime=False, vmin=0.5, vmax=1.5, huber_stall=0.0):
        v = np.array(v, np.float64)
        theta = np.array(theta, np.float64)
        z = np.ascontiguousarray(z, np.float64)
        p = OrParams(max_iterations, tolerance, int(exact), gain_policy, int(robust), gamma, int(flat_start),
                     int(realtime), vmin, vmax, huber_stall)
        res = OrResult()
        r = np.empty(self.n_meas)
        self.L.or_wls(self.h, _dp(z), _dp(v), _dp(theta), ctypes.byref(p), ctypes.byref(res), _dp(r))
        return v, theta, res, r

    def results(self, v, theta):
        """(p_inj, q_inj, pf, qf, pt, qt) at the state (v, theta)."""
        v = np.ascontiguousarray(v, np.float64)
        theta = np.ascontiguousarray(theta, np.float64)
        out = [np.empty(self.n_bus), np.empty(self.n_bus)] + [np.empty(self.n_branch) for _ in range(4)]
        self.L.or_results(self.h, _dp(v), _dp(theta), *[_dp(a) for a in out])
        return out

    def bad_data(self, r, threshold):
        r = np.ascontiguousarray(r, np.float64)
        idx = np.empty(max(self.n_meas, 1), np.int32)
        c = self.L.or_bad_data(self.h, _dp(r), threshold, _ip(idx), self.n_meas)
        return idx[:c].copy()

    def ordering(self):
        p = np.empty(self.n_bus, np.int32)
        self.L.or_ordering(self.h, _ip(p))
        return p

    def symbolic(self, bus_perm):
        bus_perm = np.ascontiguousarray(bus_perm, np.int32)
        par = np.empty(self.n_bus, np.int32)
        cc = np.empty(self.n_bus, np.int32)
        self.L.or_symbolic(self.h, _ip(bus_perm), _ip(par), _ip(cc))
        return par, cc


def threads():
    return lib().or_threads()


class RefPin:
    """The reference's own Ybus / h(x) / Jacobian kernels (FP32, from the
    cubins in oracle/_ref) run through oracle/refpin.cpp on the GPU."""

    REF_DIR = os.path.join(HERE, "_ref")

    @classmethod
    def available(cls):
        return all(os.path.exists(os.path.join(cls.REF_DIR, u + ".cubin")) for u in ("kernels", "sparse_matrix"))

    def __init__(self):
        L = ctypes.CDLL(os.path.join(HERE, "_build", "librefpin.so"))
        L.rp_error.restype = ctypes.c_char_p
        L.rp_open.restype = I
        L.rp_open.argtypes = [ctypes.c_char_p]
        U8 = P(ctypes.c_uint8)
        F = P(ctypes.c_float)
        L.rp_ybus.restype = I
        L.rp_ybus.argtypes = [I, I, P(I), P(I), F, F, F, F, F, U8, P(I), P(I), F, F, I]
        L.rp_evaluate.restype = I
        L.rp_evaluate.argtypes = [I, I, I, P(I), P(I), F, F, F, F, F, U8, I, U8, P(I), U8, F, F, F, P(I), F]
        self.L = L
        if L.rp_open(self.REF_DIR.encode()) != 0:
            raise RuntimeError(L.rp_error().decode())

    @staticmethod
    def _branch_arrays(grid):
        f32 = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
        return [np.ascontiguousarray(grid.br_from, np.int32), np.ascontiguousarray(grid.br_to, np.int32),
                f32(grid.br_r), f32(grid.br_x), f32(grid.br_b), f32(grid.br_tap), f32(grid.br_shift),
                np.ascontiguousarray(grid.br_status, np.uint8)]

    @staticmethod
    def _args(arrs):
        out = []
        for a in arrs:
            t = {np.int32: I, np.float32: ctypes.c_float, np.uint8: ctypes.c_uint8}[a.dtype.type]
            out.append(a.ctypes.data_as(P(t)))
        return out

    def ybus(self, grid):
        """(row_ptr, col, g, b) in the reference kernels' (arrival) order."""
        br = self._branch_arrays(grid)
        cap = grid.n_bus + 2 * grid.n_branch
        ptr = np.empty(grid.n_bus + 1, np.int32)
        col = np.empty(cap, np.int32)
        g = np.empty(cap, np.float32)
        b = np.empty(cap, np.float32)
        nnz = self.L.rp_ybus(grid.n_bus, grid.n_branch, *self._args(br), *self._args([ptr, col, g, b]), cap)
        if nnz < 0:
            raise RuntimeError(self.L.rp_error().decode())
        return ptr, col[:nnz], g[:nnz], b[:nnz]

    def evaluate(self, grid, v, theta):
        """h(x) [n_meas] and the Jacobian rows as (col, val) arrays of 10 slots
        a row in the kernel's write order (-1 = empty slot)."""
        br = self._branch_arrays(grid)
        m = grid.n_meas
        meas = [np.ascontiguousarray(grid.m_type, np.uint8), np.ascontiguousarray(grid.m_loc, np.int32),
                np.ascontiguousarray(grid.m_end, np.uint8)]
        st = [np.ascontiguousarray(v, np.float32), np.ascontiguousarray(theta, np.float32)]
        h = np.empty(m, np.float32)
        hcol = np.empty(10 * m, np.int32)
        hval = np.empty(10 * m, np.float32)
        rc = self.L.rp_evaluate(grid.n_bus, int(grid.slack), grid.n_branch, *self._args(br), m,
                                *self._args(meas), *self._args(st), *self._args([h, hcol, hval]))
        if rc != 0:
            raise RuntimeError(self.L.rp_error().decode())
        return h, hcol.reshape(m, 10), hval.reshape(m, 10)
