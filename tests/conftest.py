import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oakg():
    """The product library, built in-tree; GPU tests only."""
    if not _cuda_available():
        pytest.skip("no CUDA device")
    from oak_gb300 import build
    build.build()
    import oak_gb300
    oak_gb300.lib()
    return oak_gb300
