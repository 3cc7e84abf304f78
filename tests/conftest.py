import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103)")


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library on a GPU; fails loudly when either is missing."""
    import torch

    from incflo_gb300 import _abi
    from incflo_gb300.build import build

    build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    lib = _abi.load()
    assert lib.gbp_device_check() == 0, lib.gbp_last_error().decode()
    return lib
