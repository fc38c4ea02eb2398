"""MATLAB quantiles and the per-component reconstruction of reconstruct_S
(reconstruct_S.m:168-205) on the GPU against the FP64 oracle."""
import numpy as np
import pytest

from tests.conftest import rel_l2


def test_oracle_quantile_nan_and_empty(oracle):
    assert np.isnan(oracle.matlab_quantile(np.array([np.nan, np.nan]), 0.5))
    assert oracle.matlab_quantile(np.array([3.0, np.nan, 1.0, 2.0]), 0.5) == 2.0
    assert oracle.matlab_quantile(np.array([5.0]), 0.9) == 5.0


QUANTILE_P = [0.0, 1e-4, 0.25, 0.5, 0.8, 0.9999, 1.0]


def quantile_cases():
    rng = np.random.default_rng(0)
    yield "normal", rng.standard_normal(1_000_003).astype(np.float32), None
    yield "integers", rng.integers(0, 10, 200_001).astype(np.float32), None
    v = rng.standard_normal(50_000).astype(np.float32)
    v[::7] = np.nan
    v[::11] = -0.0
    yield "nan_negzero", v, None
    w = rng.random(300_000).astype(np.float32)
    yield "masked", w, (rng.random(300_000) < 0.3)
    yield "one", np.array([2.5], np.float32), None
    yield "two", np.array([4.0, -1.0], np.float32), None
    yield "clipped", np.maximum(rng.standard_normal(400_000), 0).astype(np.float32), None


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c[0] for c in quantile_cases()])
def test_quantile_gpu_bit_exact(gpu, oracle, case):
    import sid_gb300 as s
    name, v, mask = next(c for c in quantile_cases() if c[0] == case)
    got = s.quantile(v, np.array(QUANTILE_P), exclude=mask)
    keep = v if mask is None else v[~mask]
    want = np.array([oracle.matlab_quantile(keep, p) for p in QUANTILE_P])
    np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
def test_quantile_gpu_empty_is_nan(gpu):
    import sid_gb300 as s
    v = np.ones(100, np.float32)
    assert np.isnan(s.quantile(v, 0.5, exclude=np.ones(100, bool)))
    assert np.isnan(s.quantile(np.full(10, np.nan, np.float32), 0.3))


@pytest.mark.gpu
def test_quantile_gpu_large(gpu, oracle):
    """A volume-sized input (1005 x 1005 x 31 values) at the Htf cap's p."""
    import torch
    import sid_gb300 as s
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand(1005 * 1005 * 31, generator=g, device="cuda") ** 3
    got = s.quantile(x, 1 - 1e-4)
    want = oracle.matlab_quantile(x.cpu().numpy(), 1 - 1e-4)
    assert got == want


@pytest.fixture(scope="module")
def small(gpu, oracle):
    from sid_gb300 import Projector, synthetic
    N, Z, M, L = 5, 3, 31, 9
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.0, sigma_max=3.0)
    Vt = synthetic.blob_volume(X, X, Z, 6, sigma=(1.5, 1.5), seed=4)
    rng = np.random.default_rng(9)
    img = (oracle.forward_project(H, Vt) + 0.02 * rng.random((X, X))).astype(np.float32)
    P = Projector(H, (X, X), None, methods=("direct", "spectral_f32", "spectral_mixed"))
    fwd = lambda v: oracle.forward_project(H, v)  # noqa: E731
    bwd = lambda i: oracle.backward_project(H, i)  # noqa: E731
    return H, np.asfortranarray(img), P, fwd, bwd


def _oracle_solve_from(oracle, Htf, nrm, fwd, bwd, opts):
    """The part of reconstruct_S.m:193-205 after the back projection, in FP64."""
    o = dict(opts)
    o["lamb_L1"] = min(oracle.matlab_quantile(Htf, 1 - 1e-4), o.get("lamb_L1", 0.0))
    if o.get("whichSolver", "fast_nnls") == "ISRA":
        return nrm * oracle.deconvRL(fwd, bwd, Htf, o.get("max_iter", 8), Htf, o)
    return nrm * oracle.LS_deconv(fwd, bwd, Htf, o)


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [{}, {"whichSolver": "ISRA", "max_iter": 6}, {"lamb_L1": 1e-4, "lamb_L2": 1e-2}])
def test_reconstruct_component_direct_matches_oracle(small, oracle, opts):
    """FP32 direct projector: end to end against the FP64 oracle."""
    import sid_gb300 as s
    H, img, P, fwd, bwd = small
    ref = oracle.reconstruct_S_one(img, fwd, bwd, opts)
    out, lam = P.reconstruct_component(img, None, opts, method="direct", return_lambda=True)
    assert rel_l2(s.to_numpy(out), ref) < 1e-4, rel_l2(s.to_numpy(out), ref)
    assert lam <= opts.get("lamb_L1", 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("method,opts,tol", [
    ("spectral_f32", {"lamb_L1": 2e-5, "lamb_L2": 1e-2}, 1e-5),
    # ISRA divides by the back projection: the projector's absolute rounding at
    # near-zero voxels is amplified there, hence the wider bar
    ("spectral_f32", {"whichSolver": "ISRA", "max_iter": 6}, 1e-4),
    ("spectral_mixed", {"q": 0.5}, 1e-4),
])
def test_reconstruct_component_spectral_stages(small, oracle, method, opts, tol):
    """Spectral projectors, stage by stage.  Their rounding error is absolute
    (spread over the field), so near-zero back-projection values change sign;
    LS_deconv's first passive set (x > 0) depends on those signs, which moves
    the reference's own solution by ~1e-3 between two such starting points
    (measured).  So: the back projection is compared with the oracle's, and the
    solve with the oracle's solve from the same back projection."""
    import sid_gb300 as s
    H, img, P, fwd, bwd = small
    im = np.maximum(img.astype(np.float64) - oracle.matlab_quantile(img, opts.get("q", 0.8)), 0.0)
    im = im / im.max()
    nrm = np.sqrt(np.sum(im * im))
    Htf = bwd(im / nrm)
    o0 = dict(opts, max_iter=0)
    if o0.get("whichSolver") == "ISRA":
        o0.pop("whichSolver")
    Hg = s.to_numpy(P.reconstruct_component(img, None, o0, method=method)).astype(np.float64) / nrm
    # FP32 back-projection spectra, or 24-bit floats (16 significant bits) in the mixed form
    htf_tol = 1e-5 if method == "spectral_mixed" else 1e-6
    assert rel_l2(Hg, Htf) < htf_tol, rel_l2(Hg, Htf)
    out = s.to_numpy(P.reconstruct_component(img, None, opts, method=method))
    ref = _oracle_solve_from(oracle, Hg, nrm, fwd, bwd, opts)
    assert rel_l2(out, ref) < tol, rel_l2(out, ref)


@pytest.mark.gpu
def test_reconstruct_component_l1_cap(small, oracle):
    """A large lamb_L1 is capped by the (1 - 1e-4) quantile of Htf
    (reconstruct_S.m:193)."""
    H, img, P, fwd, bwd = small
    im = np.maximum(img.astype(np.float64) - oracle.matlab_quantile(img, 0.8), 0.0)
    im = im / im.max()
    Htf = bwd(im / np.sqrt(np.sum(im * im)))
    want = oracle.matlab_quantile(Htf, 1 - 1e-4)
    _, lam = P.reconstruct_component(img, None, {"lamb_L1": 1e6}, method="direct", return_lambda=True)
    assert abs(lam - want) <= 1e-5 * abs(want)


@pytest.mark.gpu
def test_reconstruct_component_microlens_mask(small, oracle):
    import sid_gb300 as s
    H, img, P, fwd, bwd = small
    ml = np.zeros(img.shape, dtype=np.uint8)
    ml[2::5, 2::5] = 1  # lenslet centres excluded from the background quantile
    ref = oracle.reconstruct_S_one(img, fwd, bwd, {}, microlenses=ml)
    out = P.reconstruct_component(img, ml, {}, method="direct")
    assert rel_l2(s.to_numpy(out), ref) < 1e-4


@pytest.mark.gpu
def test_reconstruct_S_function_api(small, oracle):
    import sid_gb300 as s
    H, img, P, fwd, bwd = small
    S = np.stack([img, np.asfortranarray(img[::-1, :])])
    recon = s.reconstruct_S(S, {"H": H}, {"method": "direct"})
    assert len(recon) == 2
    for k in range(2):
        ref = oracle.reconstruct_S_one(S[k], fwd, bwd, {})
        assert rel_l2(s.to_numpy(recon[k]), ref) < 1e-4


# --------------------------------------------- several components at once --
def _component_images(img, n):
    imgs = [img, np.asfortranarray(img[::-1, :]), np.asfortranarray(img[:, ::-1]),
            np.asfortranarray(img.T), np.asfortranarray(img[::-1, ::-1])]
    return [np.asfortranarray(imgs[k % 5] * (1.0 + 0.1 * k)).astype(np.float32) for k in range(n)]


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [{}, {"whichSolver": "ISRA", "max_iter": 6}, {"lamb_L1": 1e6, "lamb_L2": 1e-2}])
def test_reconstruct_components_equal_single_calls(small, opts):
    """The batched driver (groups of components through the batched back
    projection and solvers) gives what one call per component gives, with the
    same capped lamb_L1 per component; 35 components span two groups."""
    import sid_gb300 as s
    H, img, P, fwd, bwd = small
    imgs = _component_images(img, 35)
    outs, lams = P.reconstruct_components(imgs, None, opts, method="direct", return_lambda=True)
    for k in (0, 1, 17, 31, 32, 34):
        one, lam = P.reconstruct_component(imgs[k], None, opts, method="direct", return_lambda=True)
        assert rel_l2(s.to_numpy(outs[k]), s.to_numpy(one)) < 1e-6, k
        assert lams[k] == pytest.approx(lam, rel=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [{}, {"whichSolver": "ISRA", "max_iter": 6}])
def test_reconstruct_components_tensor_core_plan(gpu, oracle, opts):
    """The tensor-core batched projections (SID_PLAN_SPECTRAL_TC, mixed form)
    inside the component driver, stage by stage as for the single spectral
    calls: the back projections against the oracle's, then each solve against
    the oracle's solve from the same back projection.  LS_deconv holds 1e-4.
    ISRA divides by the back projection, whose absolute rounding is amplified
    at the near-zero voxels of a background-clipped component: there the
    batched solve must stay within twice the single-volume mixed form's error
    from the same start (or 5e-4)."""
    import sid_gb300 as s
    from sid_gb300 import Projector, synthetic
    N, Z, M, L = 5, 3, 31, 9
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.0, sigma_max=3.0)
    Vt = synthetic.blob_volume(X, X, Z, 6, sigma=(1.5, 1.5), seed=4)
    rng = np.random.default_rng(9)
    img = np.asfortranarray((oracle.forward_project(H, Vt) + 0.02 * rng.random((X, X))).astype(np.float32))
    fwd = lambda v: oracle.forward_project(H, v)  # noqa: E731
    bwd = lambda i: oracle.backward_project(H, i)  # noqa: E731
    P = Projector(H, (X, X), None, methods=("spectral_mixed",), batched=True)
    imgs = _component_images(img, 6)
    o0 = dict(opts, max_iter=0)
    o0.pop("whichSolver", None)
    hg = P.reconstruct_components(imgs, None, o0, method="spectral_mixed")
    outs = P.reconstruct_components(imgs, None, opts, method="spectral_mixed")
    isra = opts.get("whichSolver") == "ISRA"
    for k in range(6):
        im = np.maximum(imgs[k].astype(np.float64) - oracle.matlab_quantile(imgs[k], 0.8), 0.0)
        im = im / im.max()
        nrm = np.sqrt(np.sum(im * im))
        Hg = s.to_numpy(hg[k]).astype(np.float64) / nrm
        assert rel_l2(Hg, bwd(im / nrm)) < 2e-5, (k, rel_l2(Hg, bwd(im / nrm)))
        ref = _oracle_solve_from(oracle, Hg, nrm, fwd, bwd, opts)
        err = rel_l2(s.to_numpy(outs[k]), ref)
        if not isra:
            assert err < 1e-4, (k, err)
            continue
        # the single-volume mixed form from the same back projection
        hk = s.to_device(np.asfortranarray((Hg * nrm).astype(np.float32)))
        one = s.to_numpy(P.isra(hk, hk, opts["max_iter"], method="spectral_mixed"))
        err1 = rel_l2(one, ref)
        assert err < max(5e-4, 2.0 * err1), (k, err, err1)
    P.close()
