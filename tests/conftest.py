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


def psf_column(H, X, Y, vox):
    """Sensor response A e_v of a unit voxel v = (px, py, c) (0-based), read
    straight from the PSF: the 'same'-convolution window of H(:, :, px mod N,
    py mod N, c) centred on (px, py) (forwardProjectACC.m:21-25 with the full
    PSF).  Returns ((x0, x1, y0, y1), tile) with tile[x - x0, y - y0] = (A e_v)(x, y)."""
    import numpy as np
    M, _, N, _, _ = H.shape
    px, py, c = (int(t) for t in vox)
    cf = M // 2
    x0, x1 = max(0, px - cf), min(X, px - cf + M)
    y0, y1 = max(0, py - cf), min(Y, py - cf + M)
    tile = np.asarray(H[x0 - px + cf:x1 - px + cf, y0 - py + cf:y1 - py + cf, px % N, py % N, c],
                      dtype=np.float64)
    return (x0, x1, y0, y1), tile


def central_fd(obj_terms, ax, y, vox_cols, h):
    """Central finite differences of a separable sensor objective
    L(x) = sum_j f(Ax_j, y_j) at single voxels: only the pixels of the voxel's
    PSF window change, so [L(x + h e_v) - L(x - h e_v)] / 2h is evaluated over
    that window (FP64).  vox_cols: psf_column outputs; h: per-voxel steps."""
    import numpy as np
    out = np.empty(len(vox_cols))
    for k, ((x0, x1, y0, y1), a) in enumerate(vox_cols):
        u = ax[x0:x1, y0:y1]
        yy = y[x0:x1, y0:y1]
        out[k] = (np.sum(obj_terms(u + h[k] * a, yy)) - np.sum(obj_terms(u - h[k] * a, yy))) / (2 * h[k])
    return out
