import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (the GB300 parity tests)")


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def sidlib():
    """libsid.so built in-tree and loaded (no GPU needed to load it)."""
    from sid_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(sidlib):
    if not cuda_available():
        pytest.skip("no CUDA device in this environment")
    import torch
    torch.cuda.init()
    return torch.device("cuda:0")


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
