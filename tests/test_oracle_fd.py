"""CPU checks of the helpers the finite-difference tests rest on: the PSF
column of a voxel equals the oracle's forward projection of that voxel, and
the windowed central difference equals the full-frame one."""
import numpy as np

from tests.conftest import central_fd, psf_column


def _small():
    from sid_gb300 import synthetic
    N, Z, M, L = 5, 3, 31, 9
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.0, sigma_max=3.0)
    return H, X


def test_psf_column_is_forward_of_unit_voxel(oracle):
    H, X = _small()
    rng = np.random.default_rng(3)
    for _ in range(6):
        v = (rng.integers(0, X), rng.integers(0, X), rng.integers(0, H.shape[4]))
        e = np.zeros((X, X, H.shape[4]))
        e[v] = 1.0
        full = oracle.forward_project(H, e)
        (x0, x1, y0, y1), tile = psf_column(H, X, X, v)
        ref = np.zeros((X, X))
        ref[x0:x1, y0:y1] = tile
        np.testing.assert_array_equal(full, ref)


def test_windowed_fd_matches_full_frame(oracle):
    H, X = _small()
    rng = np.random.default_rng(5)
    x = rng.uniform(0.5, 1.5, (X, X, H.shape[4]))
    y = oracle.forward_project(H, rng.uniform(0.5, 1.5, x.shape))
    ax = oracle.forward_project(H, x)
    terms = lambda u, yy: u - yy * np.log(u)  # noqa: E731  Poisson negative log-likelihood
    vox = [(3, 7, 0), (40, 2, 2), (21, 22, 1)]
    h = np.array([1e-3 * max(abs(x[v]), 1e-3) for v in vox])
    fd = central_fd(terms, ax, y, [psf_column(H, X, X, v) for v in vox], h)
    for k, v in enumerate(vox):
        e = np.zeros_like(x)
        e[v] = h[k]
        full = (np.sum(terms(oracle.forward_project(H, x + e), y)) -
                np.sum(terms(oracle.forward_project(H, x - e), y))) / (2 * h[k])
        assert abs(fd[k] - full) <= 1e-6 * abs(full) + 1e-9
    # and both are the adjoint gradient A'(1 - y ./ Ax) to O(h^2)
    g = oracle.backward_project(H, 1.0 - y / ax)
    np.testing.assert_allclose(fd, [g[v] for v in vox], rtol=1e-6)
