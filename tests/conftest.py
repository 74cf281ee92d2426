import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 kernels)")


@pytest.fixture(scope="session")
def built():
    """Compile the oracle and the CUDA library once per session (no-op when up to date)."""
    import oracle
    from capow_gb300 import build as b

    oracle.build()
    b.build()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
