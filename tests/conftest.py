import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and libturbotrace.so")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="session")
def cuda():
    """The GPU tests never skip: on a GPU machine a missing device or library is a failure."""
    import torch

    assert torch.cuda.is_available(), "GPU test needs CUDA"
    from turbulence_tracing_gb300 import _lib

    _lib.lib()
    return torch.device("cuda")
