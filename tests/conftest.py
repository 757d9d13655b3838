import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def gpu():
    """Skip on machines without a GPU; on a GPU machine a missing library is an error."""
    if not HAS_GPU:
        pytest.skip("no CUDA device")
    import codeare_gb300 as cg
    cg.capi.load()  # raises if libcgs.so is absent
    return cg


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
