import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def orc():
    import oracle

    return oracle.lib()


@pytest.fixture(scope="session")
def cuda():
    """The CUDA library and torch CUDA device; fails loudly when missing."""
    import torch

    from ampe_gb300 import _native

    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    assert _native.lib.ampe_device_count() >= 1
    return _native
