import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the device kernels)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """The in-tree CUDA library; a GPU test fails (not skips) when it is missing."""
    from mpqpcudasolver_gb300 import solver
    if not _has_gpu():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return solver.load()
