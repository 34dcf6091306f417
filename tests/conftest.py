import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "kitbase.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def gpu_lib():
    """libkitgpu loaded with a visible CUDA device; GPU tests fail (not skip)
    when the library is missing, so a silent fallback cannot pass them."""
    from kitgpu import _native as N
    if N.cuda_device_count() < 1:
        pytest.fail("no CUDA device visible to a test marked gpu")
    return N.load()
