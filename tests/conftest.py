import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a) and the built library")


@pytest.fixture(scope="session")
def cuda_lib():
    """Build (if needed) and load libdiffrp_gb300.so; skip when no GPU."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from diffrp_gb300 import build, _ffi
    build.build()
    return _ffi.load()
