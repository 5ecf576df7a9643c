import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels")


@pytest.fixture(scope="session")
def fbse():
    """The product library (built in-tree); GPU tests fail loudly if it is missing."""
    import filterbse_gb300 as F
    F.load()
    return F


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test requested but torch.cuda is not available")
    return torch.device("cuda:0")
