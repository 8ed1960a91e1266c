import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


@pytest.fixture(scope="session")
def cuda_lib():
    """libcfdgpu with at least one visible GPU; a GPU test fails (not skips) without one."""
    from mycode_gb300 import api
    n = api.device_count()
    assert n > 0, "no CUDA device visible to libcfdgpu"
    return api
