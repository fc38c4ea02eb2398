"""ISRA (deconvRL) and LS_deconv on the GPU against the FP64 oracle."""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small(gpu, oracle):
    from sid_gb300 import Projector, synthetic
    N, Z, M, L = 5, 3, 31, 9
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.0, sigma_max=3.0)
    Vt = synthetic.blob_volume(X, X, Z, 6, sigma=(1.5, 1.5), seed=4)
    y = oracle.forward_project(H, Vt)
    P = Projector(H, (X, X), None, methods=("direct", "spectral_f32", "spectral_mixed"))
    fwd = lambda v: oracle.forward_project(H, v)  # noqa: E731
    bwd = lambda i: oracle.backward_project(H, i)  # noqa: E731
    return H, y, P, fwd, bwd


@pytest.mark.parametrize("method,tol", [("direct", 1e-5), ("spectral_f32", 1e-5), ("spectral_mixed", 1e-4)])
def test_isra_matches_oracle(small, method, tol):
    import sid_gb300 as s
    from oracle import oracle as o
    H, y, P, fwd, bwd = small
    Htf = bwd(y).astype(np.float32)
    ref = o.deconvRL(fwd, bwd, Htf, 8, Htf)
    P.default_method = method
    out = s.to_numpy(s.deconvRL(P.forward, P.adjoint, Htf, 8, Htf, {"lambda": 0, "p": 1, "mode": "basic"}))
    assert rel_l2(out, ref) < 10 * tol, rel_l2(out, ref)


def test_isra_frame225_mixed_vs_fp64(gpu, oracle):
    """8 ISRA iterations on the 225 x 225 x 11 configuration (Nnum 15, PSF 195):
    the mixed-precision spectral forms (16-bit forward; 24-bit float or FP32
    back projection) against the FP64 oracle, bar 1e-4.  (16-bit block-float
    spectra in the back projection are not used for ISRA: their error is
    relative to each frequency row's largest entry, voxels whose PSF leaves the
    sensor have tiny back projections, and the division diverges.)"""
    import sid_gb300 as s
    from sid_gb300 import synthetic
    H, V = synthetic.config_inputs("225x225x11")
    y = oracle.forward_project(H, V)
    fwd = lambda v: oracle.forward_project(H, v)  # noqa: E731
    bwd = lambda i: oracle.backward_project(H, i)  # noqa: E731
    Htf = bwd(y)
    ref = oracle.deconvRL(fwd, bwd, Htf, 8, Htf)
    P = s.Projector(H, V.shape[:2], None, methods=("spectral_mixed", "spectral_f32"))
    for m, tol in (("spectral_mixed", 1e-4), ("spectral_mixed_f32", 1e-4), ("spectral_f32", 1e-5)):
        out = s.to_numpy(P.isra(Htf.astype(np.float32), Htf.astype(np.float32), 8, method=m))
        assert rel_l2(out, ref) < tol, (m, rel_l2(out, ref))


@pytest.mark.parametrize("method,tol", [("direct", 1e-5), ("spectral_f32", 1e-5), ("spectral_mixed", 1e-4)])
def test_rl_poisson_matches_oracle(small, method, tol):
    """Poisson-likelihood RL from the sensor image, 8 iterations, against FP64."""
    from oracle import oracle as o
    import sid_gb300 as s
    H, y, P, fwd, bwd = small
    X0 = np.asfortranarray(bwd(y).astype(np.float32))
    ref = o.rl_poisson(fwd, bwd, y, 8, X0)
    out = s.to_numpy(P.rl_poisson(y.astype(np.float32), X0, 8, method=method))
    assert rel_l2(out, ref) < 10 * tol, rel_l2(out, ref)


def test_rl_poisson_zero_rules(small):
    """Zero image and zero start: every ratio is 0/0 and the result stays 0, finite."""
    import sid_gb300 as s
    H, y, P, fwd, bwd = small
    out = s.to_numpy(P.rl_poisson(np.zeros_like(y, dtype=np.float32), np.zeros((y.shape[0], y.shape[1], H.shape[4]),
                                                                               np.float32, order="F"), 2))
    assert np.all(out == 0)


def _pinned_fortran(a):
    """A Fortran-ordered float32 copy of `a` in page-locked host memory."""
    import torch
    buf = torch.empty(a.size, dtype=torch.float32, pin_memory=True).numpy()
    out = buf.reshape(a.shape, order="F")
    out[...] = a
    return out


@pytest.mark.parametrize("method", ["direct", "spectral_mixed"])
def test_isra_host_matches_device(small, method):
    """The host-array entry point (input and result over the host link, Htf on a
    side stream) gives the device-array call's result bit for bit, from
    pageable and from page-locked host arrays, for several iterations and for
    none."""
    import sid_gb300 as s
    H, y, P, fwd, bwd = small
    Htf = bwd(y).astype(np.float32)
    X0 = np.asfortranarray(0.5 * Htf + 0.01)
    for iters in (0, 3):
        ref = s.to_numpy(P.isra(Htf, X0, iters, method=method))
        np.testing.assert_array_equal(P.isra_host(Htf, X0, iters, method=method), ref)
        xp = _pinned_fortran(X0)
        P.isra_host_inplace(_pinned_fortran(Htf), xp, iters, method=method)
        np.testing.assert_array_equal(xp, ref)


@pytest.mark.parametrize("method,tol", [("direct", 1e-5), ("spectral_f32", 1e-5), ("spectral_mixed", 1e-4)])
def test_ls_deconv_matches_oracle(small, method, tol):
    import sid_gb300 as s
    from oracle import oracle as o
    H, y, P, fwd, bwd = small
    Htf = bwd(y).astype(np.float32)
    opts = {"max_iter": 8, "lamb_L1": 1e-3, "lamb_L2": 1e-2}
    ref = o.LS_deconv(fwd, bwd, Htf, opts)
    P.default_method = method
    out = s.to_numpy(s.LS_deconv(P.forward, P.adjoint, Htf, opts))
    assert rel_l2(out, ref) < 10 * tol, rel_l2(out, ref)


def test_isra_zero_rules(gpu):
    """inf -> 0 and NaN -> 0 (deconvRL.m:85-87): zero voxels stay zero."""
    import sid_gb300 as s
    from sid_gb300 import synthetic
    H = synthetic.gaussian_psf(9, 3, 2, sigma_min=1.0, sigma_max=2.0)
    P = s.Projector(H, (12, 12), None)
    Htf = np.zeros((12, 12, 2), dtype=np.float32)
    Htf[5, 5, 0] = 1.0
    X0 = np.ones((12, 12, 2), dtype=np.float32)
    X0[0, 0, 1] = 0.0
    out = s.to_numpy(P.isra(Htf, X0, 2))
    assert np.all(np.isfinite(out))
    assert out[0, 0, 1] == 0.0


@pytest.mark.parametrize("p,lam", [(1, [0.02, 0.01, 0.005]), (2, [0.05, 0.03, 0.01])])
def test_isra_tv_matches_oracle(small, p, lam):
    """deconvRL mode 'TV' (deconvRL.m:61-83): p = 1 (sign of forward
    differences) and p = 2 (7-point filter), with the iteration history."""
    import sid_gb300 as s
    from oracle import oracle as o
    H, y, P, fwd, bwd = small
    Htf = bwd(y).astype(np.float32)
    opts = {"lambda": lam, "p": p, "mode": "TV"}
    ref = o.deconvRL(fwd, bwd, Htf, 6, Htf, opts)
    P.default_method = "direct"
    out, hist = s.deconvRL(P.forward, P.adjoint, Htf, 6, Htf, opts, nargout=2)
    assert rel_l2(s.to_numpy(out), ref) < 1e-4, rel_l2(s.to_numpy(out), ref)
    h = hist.cpu().numpy()
    assert h.shape == (6,) + Htf.shape
    np.testing.assert_array_equal(h[5], s.to_numpy(out))
    ref3 = o.deconvRL(fwd, bwd, Htf, 3, Htf, opts)
    assert rel_l2(h[2], ref3) < 1e-4


def test_isra_basic_history(small):
    """Xguess_history of mode 'basic' (deconvRL.m:10,90-92): one volume per iteration."""
    import sid_gb300 as s
    from oracle import oracle as o
    H, y, P, fwd, bwd = small
    Htf = bwd(y).astype(np.float32)
    P.default_method = "direct"
    out, hist = s.deconvRL(P.forward, P.adjoint, Htf, 4, Htf, None, nargout=2)
    h = hist.cpu().numpy()
    for k in range(4):
        assert rel_l2(h[k], o.deconvRL(fwd, bwd, Htf, k + 1, Htf)) < 1e-5


@pytest.mark.parametrize("opts", [{"lamb_TV_L2": [0.01, 0.02, 0.005], "max_iter": 6},
                                  {"lamb_TV_L2": [0.01, 0.02, 0.005], "lamb_TV_L1": 0.1, "lamb_L2": 0.05,
                                   "lamb_L1": 1e-3, "max_iter": 6}])
def test_ls_deconv_tv_matches_oracle(small, opts):
    """LS_deconv's lamb_TV_L2 Laplacian term in Q (LS_deconv.m:49-73), and the
    step length from Q itself when lamb_TV_L1 * lamb_TV_L2 * lamb_L2 is nonzero
    in every component (LS_deconv.m:82-83)."""
    import sid_gb300 as s
    from oracle import oracle as o
    H, y, P, fwd, bwd = small
    Htf = bwd(y).astype(np.float32)
    ref = o.LS_deconv(fwd, bwd, Htf, opts)
    P.default_method = "direct"
    out = s.to_numpy(s.LS_deconv(P.forward, P.adjoint, Htf, opts))
    assert rel_l2(out, ref) < 1e-4, rel_l2(out, ref)
