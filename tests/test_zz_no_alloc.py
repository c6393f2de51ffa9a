"""Allocation-free factor/solve (sle_ExFactorSolveNoAlloc) against the
allocating entry point (sle_ExFactorSolve), both through the C ABI.

The file name sorts last so that the suite exercises the static scratch array
after every other GPU test; the tests also pass alone in a fresh process,
where the first call performs the one-time symbol look-up.
Tolerance: max |x_noalloc - x| <= 1e-12 * max |x| (same kernels, same order).
"""
import ctypes

import numpy as np
import pytest

from conftest import gpu_available
from grids import synthetic_state
from state_estimation_with_cuda_gb300 import Estimator, api, workloads
from state_estimation_with_cuda_gb300.workloads import SyntheticGrid

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.fail("GPU tests need a CUDA device; the product has no CPU fallback")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def noalloc_solve(e, rhs):
    x = np.full(rhs.shape, np.nan)
    rc = e.lib.sle_ExFactorSolveNoAlloc(e.h, _dp(np.ascontiguousarray(rhs)), _dp(x))
    return rc, x


@pytest.mark.parametrize("name", ["grid14", "grid2k", "grid10k"])
def test_noalloc_matches_allocating_entry_point_twice(name):
    g = SyntheticGrid(2000, 2800, 0x5E01) if name == "grid2k" else workloads.make(name)
    e = Estimator()
    e.load_network(g)
    e.upload_model()
    v, th = synthetic_state(g)
    e.evaluate_at(v, th, exact=True)
    rng = np.random.default_rng(11)
    n = 2 * g.n_bus - 1
    for call in range(2):  # two calls in a row share (and reuse) the static scratch
        rhs = rng.standard_normal(n)
        x_ref = e.factor_solve(rhs)
        rc, x = noalloc_solve(e, rhs)
        assert rc == api.OK, e.lib.sle_GetLastError(e.h)
        assert np.all(np.isfinite(x))
        assert np.abs(x - x_ref).max() <= TOL * np.abs(x_ref).max(), call
    e.close()


def test_noalloc_rejects_models_beyond_the_static_limit():
    g = SyntheticGrid(40000, 56000, 7)
    e = Estimator()
    e.load_network(g)
    e.upload_model()
    v, th = synthetic_state(g)
    e.evaluate_at(v, th, exact=True)
    rc, x = noalloc_solve(e, np.ones(2 * g.n_bus - 1))
    assert rc == api.ERROR_INVALID_ARGUMENT
    msg = e.lib.sle_GetLastError(e.h).decode()
    assert "bytes of scratch" in msg and str(16 << 20) in msg
    assert np.all(np.isnan(x))  # nothing written
    e.close()


def test_noalloc_on_a_handle_whose_device_is_not_current():
    """A handle binds its own device for the call: with another device made
    current by a second handle, the static scratch is looked up on (and the
    kernels run on) the handle's device.  Needs two GPUs."""
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    other = Estimator()
    other.set_config(device_id=1)
    other.initialize()  # device 1 is now current on this thread
    g = SyntheticGrid(2000, 2800, 0x5E01)
    e = Estimator()
    e.set_config(device_id=0)
    e.load_network(g)
    e.upload_model()
    v, th = synthetic_state(g)
    e.evaluate_at(v, th, exact=True)
    rhs = np.random.default_rng(5).standard_normal(2 * g.n_bus - 1)
    for _ in range(2):
        x_ref = e.factor_solve(rhs)
        rc, x = noalloc_solve(e, rhs)
        assert rc == api.OK, e.lib.sle_GetLastError(e.h)
        assert np.abs(x - x_ref).max() <= TOL * np.abs(x_ref).max()
    e.close()
    other.close()
