"""Several volumes per pass over the tap spectra (reconstruct_S.m:162-212
reconstructs components side by side): batched projections and batched ISRA
(deconvRL, mode 'basic') against the FP64 oracle and against single calls."""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def geom(gpu, oracle):
    from sid_gb300 import Projector, synthetic
    N, Z, M, L = 5, 3, 31, 9
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.0, sigma_max=3.0)
    P = Projector(H, (X, X), None, methods=("direct", "spectral_f32", "spectral_mixed"))
    return H, P, X, Z


def _volumes(X, Z, n, seed):
    from sid_gb300 import synthetic
    return [synthetic.blob_volume(X, X, Z, 6, sigma=(1.5, 1.5), seed=seed + k) for k in range(n)]


@pytest.mark.parametrize("method,tol", [("spectral_f32", 1e-6), ("spectral_mixed", 1e-6), ("direct", 1e-7)])
def test_batched_projections_equal_single_calls(geom, method, tol):
    import sid_gb300 as s
    H, P, X, Z = geom
    vols = _volumes(X, Z, 6, 50)
    outs = P.forward_batched(vols, method=method)
    for v, o in zip(vols, outs):
        assert rel_l2(s.to_numpy(o), s.to_numpy(P.forward(v, method=method))) < tol
    ims = [s.to_numpy(o) for o in outs]
    backs = P.adjoint_batched(ims, method=method)
    for i, b in zip(ims, backs):
        assert rel_l2(s.to_numpy(b), s.to_numpy(P.adjoint(i, method=method))) < tol


@pytest.mark.parametrize("nb", [1, 7, 30])
@pytest.mark.parametrize("method,tol", [("direct", 1e-5), ("spectral_f32", 1e-5), ("spectral_mixed", 1e-4)])
def test_batched_isra_matches_oracle(geom, oracle, nb, method, tol):
    import sid_gb300 as s
    H, P, X, Z = geom
    vols = _volumes(X, Z, nb, 100)
    fwd = lambda v: oracle.forward_project(H, v)  # noqa: E731
    bwd = lambda i: oracle.backward_project(H, i)  # noqa: E731
    htfs = [bwd(fwd(v)).astype(np.float32) for v in vols]
    outs = P.isra_batched(htfs, htfs, 8, method=method)
    worst = 0.0
    for h, o in zip(htfs, outs):
        ref = oracle.deconvRL(fwd, bwd, h, 8, h)
        worst = max(worst, rel_l2(s.to_numpy(o), ref))
    # the bars of test_deconv_gpu.py's single-volume ISRA test
    assert worst < 10 * tol, worst
