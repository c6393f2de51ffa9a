"""GB300-native WLS power-grid state estimator.

A drop-in for the SLE Engine's C ABI (sle_api.h): host C++ (model store,
symbolic analysis, Gauss-Newton driver) over hand-written sm_103a CUDA
kernels, exported from the in-tree library lib/libsle_gb300.so.  This package
holds the ctypes bindings (native.py), a Python mirror of the C interface
(api.py) and the seeded synthetic workloads (workloads.py).
"""
from .api import BatchEstimator, Estimator, Server, SLEError  # noqa: F401
from .native import NativeLibraryMissing, sle_lib, segen_lib  # noqa: F401
from .workloads import SyntheticGrid, make  # noqa: F401

__version__ = "0.20.0"
