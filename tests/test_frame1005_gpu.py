"""The 1005 x 1005 x 31 configuration (Nnum 15, PSF 345^2 x 15^2 x 31): the
adjoint checks at full size.

* the dot-product test <Ax, y> = <x, A'y> on 16 random (x, y) pairs;
* central finite differences of the Poisson log-likelihood and of the LS
  objective at 64 random voxels (FP64, step 1e-3 max(|x_i|, 1e-3)) against the
  gradients A'(1 - y ./ Ax) and A'(Ax - y) formed with the GPU back projection;
* forward and back projection against the FP64 oracle at sampled pixels and
  voxels;
* 30 ISRA and Poisson-RL iterations of the mixed-precision and FP32 spectral
  forms against the FP32 direct path.
"""
import numpy as np
import pytest

from tests.conftest import central_fd, psf_column, rel_l2

pytestmark = pytest.mark.gpu

METHODS = ("direct", "spectral_f32", "spectral_mixed")
TOL = {"direct": 1e-5, "spectral_f32": 1e-5, "spectral_mixed": 1e-4, "spectral_mixed_f32": 1e-4}


@pytest.fixture(scope="module")
def frame1005(gpu):
    import torch
    import sid_gb300 as s
    from sid_gb300 import synthetic
    H, V = synthetic.config_inputs("1005x1005x31")
    P = s.Projector(H, V.shape[:2], None, methods=("direct", "spectral_f32", "spectral_mixed"))
    y = synthetic.poisson_image(s.to_numpy(P.forward(V, method="spectral_f32")))
    yield H, V, y, P
    P.close()
    torch.cuda.empty_cache()


def test_frame1005_dot_product_16_pairs(frame1005):
    import torch
    H, V, y, P = frame1005
    X, Y, Z = V.shape
    g = torch.Generator(device="cuda").manual_seed(11)
    x = torch.empty((Z, Y, X), device="cuda").permute(2, 1, 0)
    i = torch.empty((Y, X), device="cuda").permute(1, 0)
    for m in METHODS:
        worst = 0.0
        for _ in range(16):
            x.copy_(torch.rand(x.shape, generator=g, device="cuda"))
            i.copy_(torch.rand(i.shape, generator=g, device="cuda"))
            lhs = torch.sum(P.forward(x, method=m).double() * i.double()).item()
            rhs = torch.sum(x.double() * P.adjoint(i, method=m).double()).item()
            worst = max(worst, abs(lhs - rhs) / abs(lhs))
        assert worst < TOL[m], (m, worst)


@pytest.mark.parametrize("objective", ["poisson", "ls"])
def test_frame1005_finite_differences_64_voxels(frame1005, objective):
    import torch
    import sid_gb300 as s
    H, V, y, P = frame1005
    X, Y, Z = V.shape
    # a point away from the solution, so that the gradients are O(1)
    x = np.asfortranarray((0.5 * V + 0.5 * V.mean()).astype(np.float32))
    rng = np.random.default_rng(21)
    vox = np.stack([rng.integers(0, X, 64), rng.integers(0, Y, 64), rng.integers(0, Z, 64)], axis=1)
    h = 1e-3 * np.maximum(np.abs(x[vox[:, 0], vox[:, 1], vox[:, 2]]).astype(np.float64), 1e-3)
    cols = [psf_column(H, X, Y, v) for v in vox]
    yd = s.to_device(y)
    for m in METHODS:
        ax_t = P.forward(x, method=m)
        ax = s.to_numpy(ax_t).astype(np.float64)
        if objective == "poisson":
            terms = lambda u, yy: u - yy * np.log(u)  # noqa: E731
            r = 1.0 - yd / ax_t
        else:
            terms = lambda u, yy: 0.5 * (u - yy) ** 2  # noqa: E731
            r = ax_t - yd
        grad = s.to_numpy(P.adjoint(r, method=m))
        g = grad[vox[:, 0], vox[:, 1], vox[:, 2]].astype(np.float64)
        fd = central_fd(terms, ax, y.astype(np.float64), cols, h)
        err = np.linalg.norm(g - fd) / np.linalg.norm(fd)
        assert err < TOL[m], (m, objective, err)
    torch.cuda.synchronize()


def test_frame1005_projections_vs_fp64_sampled(frame1005, oracle):
    import sid_gb300 as s
    H, V, y, P = frame1005
    X, Y, Z = V.shape
    rng = np.random.default_rng(7)
    pix = np.stack([rng.integers(0, X, 256), rng.integers(0, Y, 256)], axis=1)
    vox = np.stack([rng.integers(0, X, 64), rng.integers(0, Y, 64), rng.integers(0, Z, 64)], axis=1)
    ref_f = oracle.forward_project_pixels(H, V, pix)
    ref_b = oracle.backward_project_voxels(H, y, vox)
    for m in METHODS:
        f = s.to_numpy(P.forward(V, method=m))[pix[:, 0], pix[:, 1]]
        b = s.to_numpy(P.adjoint(y, method=m))[vox[:, 0], vox[:, 1], vox[:, 2]]
        assert rel_l2(f, ref_f) < TOL[m], (m, rel_l2(f, ref_f))
        assert rel_l2(b, ref_b) < TOL[m], (m, rel_l2(b, ref_b))


def test_frame1005_weak_voxels_exact(frame1005):
    """Voxels whose PSF falls mostly off the sensor (column mass A'1 below 1e-2
    of the largest) get exact back projections from every spectral
    form: per entry within 1e-5 of the direct path, where an FFT-based value
    alone has no correct digits."""
    import torch
    import sid_gb300 as s
    H, V, y, P = frame1005
    nweak = P.info()["weak_voxels"]
    assert nweak > 0
    ones = torch.ones((V.shape[1], V.shape[0]), device="cuda").t()
    mass = s.to_numpy(P.adjoint(ones, method="direct"))
    weak = mass < 1e-2 * mass.max()
    assert abs(int(weak.sum()) - nweak) <= max(4, nweak // 100)  # threshold ties only
    ref = s.to_numpy(P.adjoint(y, method="direct"))[weak].astype(np.float64)
    for m in ("spectral_f32", "spectral_mixed", "spectral_mixed_f32"):
        got = s.to_numpy(P.adjoint(y, method=m))[weak].astype(np.float64)
        err = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30))
        assert err < 1e-5, (m, err)


def test_frame1005_isra_30_iterations(frame1005):
    """30 ISRA iterations from Htf = A'y: the mixed-precision and FP32 spectral
    forms against the FP32 direct path (itself within 1e-5 of FP64 per
    projection)."""
    import sid_gb300 as s
    H, V, y, P = frame1005
    Htf = P.adjoint(y, method="direct")
    ref = s.to_numpy(P.isra(Htf, Htf, 30, method="direct"))
    for m in ("spectral_f32", "spectral_mixed", "spectral_mixed_f32"):
        out = s.to_numpy(P.isra(Htf, Htf, 30, method=m))
        assert rel_l2(out, ref) < TOL[m], (m, rel_l2(out, ref))


def test_frame1005_rl_poisson_30_iterations(frame1005):
    """30 Poisson-RL iterations, spectral forms against the FP32 direct path,
    bar 1e-4: the ratio y ./ AX makes this iteration more sensitive than ISRA,
    and two FP32 forms that agree to ~1e-7 per projection end ~2e-5 apart
    whatever the weak-voxel threshold."""
    import sid_gb300 as s
    H, V, y, P = frame1005
    X0 = P.adjoint(y, method="direct")
    ref = s.to_numpy(P.rl_poisson(y, X0, 30, method="direct"))
    for m in ("spectral_f32", "spectral_mixed"):
        out = s.to_numpy(P.rl_poisson(y, X0, 30, method=m))
        assert rel_l2(out, ref) < 1e-4, (m, rel_l2(out, ref))


# FP32 lenslet taps; tensor-core windows (24-bit window spectra, two-part box spectra)
@pytest.mark.parametrize("fn,bar", [("sid_library", 1e-5), ("sid_library_spectral", 3e-5)])
def test_library_800_neurons_sampled_pixels(frame1005, fn, bar):
    """Library generation at the 800-neuron size (generate_LFM_library_GPU.m:
    63-109: neur_rad 12, axial 2, one component): 20 neurons' rows against an
    FP64 restatement at 500 sampled pixels each inside their sensor footprints,
    summing every voxel of the neuron's box through the PSF
    (forwardProjectACC.m:21-25 with the full PSF)."""
    import ctypes

    import torch
    import sid_gb300 as s
    from sid_gb300 import _lib, synthetic
    H, V, y, P = frame1005
    X, Y, Z = V.shape
    M, N = H.shape[0], H.shape[2]
    cf = M // 2
    K = 800
    vol, centers = synthetic.neuron_volume(X, Y, Z, K)
    dv = s.to_device(vol)
    out = torch.zeros((K, X * Y), dtype=torch.float32, device="cuda")  # column layout: out[n, pixel]
    ptrs = (ctypes.c_void_p * 1)(dv.data_ptr())
    c = np.asfortranarray(centers)
    ids = np.ones((K, 1), dtype=np.uint8, order="F")
    _lib.call(fn, P._plan, ctypes.cast(ptrs, ctypes.c_void_p), 1, c.ctypes.data, ids.ctypes.data, K, 12,
              2.0, out.data_ptr(), 1, s.lfm._stream_ptr())
    torch.cuda.synchronize()
    boxes = s.library_boxes(centers, 12, 2.0, (X, Y, Z))  # 0-based half-open
    rng = np.random.default_rng(17)
    worst = 0.0
    for n in rng.choice(K, 20, replace=False):
        x0, x1, y0, y1, z0, z1 = (int(v) for v in boxes[n])
        p, q, cc = np.meshgrid(np.arange(x0, x1), np.arange(y0, y1), np.arange(z0, z1), indexing="ij")
        p, q, cc = p.ravel(), q.ravel(), cc.ravel()
        val = vol[p, q, cc].astype(np.float64)
        px = rng.integers(max(0, x0 - cf), min(X, x1 + cf), 500)
        py = rng.integers(max(0, y0 - cf), min(Y, y1 + cf), 500)
        i = px[:, None] - p[None, :] + cf
        j = py[:, None] - q[None, :] + cf
        ok = (i >= 0) & (i < M) & (j >= 0) & (j < M)
        hv = H[np.clip(i, 0, M - 1), np.clip(j, 0, M - 1), (p % N)[None, :], (q % N)[None, :], cc[None, :]]
        ref = np.sum(np.where(ok, hv.astype(np.float64), 0.0) * val[None, :], axis=1)
        got = out[int(n)].cpu().numpy()[px + X * py]
        worst = max(worst, rel_l2(got, ref))
    assert worst < bar, worst
