import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    from state_estimation_with_cuda_gb300 import _build

    _build.build_all()
    yield


def gpu_available():
    try:
        from state_estimation_with_cuda_gb300 import sle_lib

        return sle_lib().sle_IsGPUAvailable() == 1
    except Exception:
        return False
