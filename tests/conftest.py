import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built voxurf_gb300 library")


@pytest.fixture(scope="session")
def cuda():
    """The CUDA device for GPU tests.  On a machine with a GPU the native
    library must load: a missing library is an error, never a skip."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxurf_gb300 import _native

    _native.load()
    return torch.device("cuda", 0)
