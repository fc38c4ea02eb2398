"""Library generation: bit-exact crop boxes (CPU) and batched projection
against the FP64 oracle (GPU)."""
import numpy as np
import pytest

from tests.conftest import rel_l2


def test_boxes_bit_exact(sidlib, oracle):
    from sid_gb300 import library_boxes
    rng = np.random.default_rng(0)
    X, Y, Z = 60, 45, 9
    # include exact .5 centres (MATLAB rounds half away from zero), edges and corners
    c = np.stack([rng.uniform(-2, X + 2, 200), rng.uniform(-2, Y + 2, 200), rng.uniform(0.5, Z + 0.4, 200)], 1)
    c[:10, 0] = np.arange(10) + 0.5
    c[10:20, 2] = 0.5 + np.arange(10) % Z
    c = c[(np.round(c[:, 0]) + 5 >= 1) & (np.round(c[:, 1]) + 5 >= 1)]
    for r, ax in [(5, 2.0), (3, 1.5), (0, 1.0)]:
        got = library_boxes(c, r, ax, (X, Y, Z))
        ref = oracle.library_boxes(c, (X, Y), Z, r, ax)
        np.testing.assert_array_equal(got, ref)


@pytest.mark.gpu
# neur_rad 4 and 2: the tiled kernel (boxes spanning 2 or 3 lattice points per
# phase); 9: the generic kernel (boxes spanning 4-5)
@pytest.mark.parametrize("rad", [4, 2, 9])
def test_library_matches_oracle(gpu, oracle, rad):
    import sid_gb300 as s
    from sid_gb300 import synthetic
    N, Z, M, L = 5, 7, 41, 12
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.5, sigma_max=6.0)
    rng = np.random.default_rng(3)
    recon = [synthetic.blob_volume(X, X, Z, 30, sigma=(1.5, 3.0), seed=10 + k) for k in range(3)]
    centers = np.stack([rng.uniform(1, X, 12), rng.uniform(1, X, 12), rng.uniform(1, Z, 12)], 1)
    centers[0] = [1.0, 1.0, 1.0]          # corner
    centers[1] = [X - 0.2, X / 2, Z]      # far edge
    neur_id = rng.random((12, 3)) < 0.6
    neur_id[:, 0] = True
    opts = {"neur_rad": rad, "axial": 2.0}
    got = s.to_numpy(s.generate_LFM_library_GPU(recon, centers, neur_id, {"H": H}, opts))
    ref = oracle.generate_library(recon, centers, neur_id, H, rad, 2.0)
    assert got.shape == ref.shape
    assert rel_l2(got, ref) < 1e-5, rel_l2(got, ref)
    for n in range(12):
        assert rel_l2(got[n], ref[n]) < 1e-5, n
    cols = s.to_numpy(s.generate_LFM_library_GPU(recon, centers, neur_id, {"H": H}, opts, layout="columns"))
    np.testing.assert_array_equal(cols, got.T)


def _library_problem(N, Z, M, L, n, rad, seed, sig=(1.5, 6.0), axial=2.0):
    from sid_gb300 import synthetic
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=sig[0], sigma_max=sig[1])
    rng = np.random.default_rng(seed)
    recon = [synthetic.blob_volume(X, X, Z, 30, sigma=(1.5, 3.0), seed=seed + k) for k in range(2)]
    centers = np.stack([rng.uniform(1, X, n), rng.uniform(1, X, n), rng.uniform(1, Z, n)], 1)
    centers[0] = [1.0, 1.0, 1.0]          # corner: most of the footprint outside the frame
    centers[1] = [X - 0.2, X / 2, Z]      # far edge, last depth
    neur_id = rng.random((n, 2)) < 0.6
    neur_id[:, 0] = True
    return H, recon, centers, neur_id, {"neur_rad": rad, "axial": axial}


@pytest.mark.gpu
# boxes of 1, 2 and 4 lattice points per phase (the 3- and 6-point pack kernels)
@pytest.mark.parametrize("rad", [4, 2, 9])
def test_spectral_library_matches_oracle(gpu, oracle, rad):
    """sid_library_spectral (tensor-core windows) against the FP64 oracle: the
    24-bit tap spectra give ~1e-5 per row."""
    import sid_gb300 as s
    H, recon, centers, neur_id, opts = _library_problem(5, 7, 41, 12, 12, rad, 3)
    got = s.to_numpy(s.generate_LFM_library_GPU(recon, centers, neur_id, {"H": H}, opts, method="spectral"))
    ref = oracle.generate_library(recon, centers, neur_id, H, rad, 2.0)
    assert got.shape == ref.shape
    assert rel_l2(got, ref) < 2e-5, rel_l2(got, ref)
    worst = max(rel_l2(got[n], ref[n]) for n in range(12))
    assert worst < 5e-5, worst
    cols = s.to_numpy(s.generate_LFM_library_GPU(recon, centers, neur_id, {"H": H}, opts, layout="columns",
                                                 method="spectral"))
    np.testing.assert_array_equal(cols, got.T)


@pytest.mark.gpu
def test_spectral_library_many_passes(gpu, oracle):
    """150 neurons: three contraction passes (64, 64 and 22 neurons: both tile
    widths), each over its own depth range (5-depth windows of 9), at Nnum 15
    with the 25-pixel boxes of neur_rad 12 (two row tiles of output phases);
    against the FP32 tap kernel, and 6 rows against the oracle."""
    import sid_gb300 as s
    H, recon, centers, neur_id, opts = _library_problem(15, 9, 75, 9, 150, 12, 11, sig=(2.0, 9.0), axial=6.0)
    spec = s.to_numpy(s.generate_LFM_library_GPU(recon, centers, neur_id, {"H": H}, opts, method="spectral"))
    direct = s.to_numpy(s.generate_LFM_library_GPU(recon, centers, neur_id, {"H": H}, opts))
    assert rel_l2(spec, direct) < 2e-5, rel_l2(spec, direct)
    worst = max(rel_l2(spec[n], direct[n]) for n in range(150))
    assert worst < 5e-5, worst
    pick = [0, 1, 40, 77, 128, 149]
    ref = oracle.generate_library(recon, centers[pick], neur_id[pick], H, 12, 6.0)
    for k, n in enumerate(pick):
        assert rel_l2(spec[n], ref[k]) < 5e-5, n


def _kernel_centers(X, Y, Z, n, seed):
    rng = np.random.default_rng(seed)
    c = np.stack([rng.uniform(-3, X + 3, n), rng.uniform(-3, Y + 3, n), rng.uniform(0.2, Z + 0.8, n)], 1)
    c[:6, 0] = np.arange(6) + 0.5          # exact halves: MATLAB rounds away from zero
    c[6:12, 2] = 0.5 + np.arange(6) % Z
    c[12] = [1.0, 1.0, 1.0]                 # corner
    return c


@pytest.mark.parametrize("r,dimz,kernel", [(4, 2.0, None), (3, 1.6, None), (2, 0.5, None),
                                          (0, 1.0, "custom"), (0, 1.0, "even")])
def test_kernel_voxels_bit_exact(sidlib, oracle, r, dimz, kernel):
    """The voxels generate_LFM_library_CPU.m:39-49 paints (ball with integer
    and fractional axial radius, a given kernel with zeros, and one of even
    size whose offsets are half-integers): libsid's host code against the
    oracle, index for index."""
    from sid_gb300 import library_kernel_voxels
    X, Y, Z = 60, 45, 9
    W = None
    if kernel == "custom":
        W = np.random.default_rng(1).random((5, 7, 3)).astype(np.float32)
        W[W < 0.3] = 0
    elif kernel == "even":
        W = np.random.default_rng(2).random((4, 4, 2)).astype(np.float32) + 0.1
    c = _kernel_centers(X, Y, Z, 60, 9)
    got = library_kernel_voxels(c, r, [1, 1, dimz], (X, Y, Z), Z, kernel=W)
    ref = oracle.library_kernel_voxels(c, r, [1, 1, dimz], (X, Y, Z), Z, kernel=W)
    assert len(got) == len(ref)
    for (gx, gv), (rx, rv) in zip(got, ref):
        np.testing.assert_array_equal(gx, rx)
        np.testing.assert_array_equal(gv, rv)


@pytest.mark.gpu
@pytest.mark.parametrize("method,bar", [("direct", 1e-5), ("spectral", 3e-5)])
@pytest.mark.parametrize("case", ["ball", "kernel"])
def test_library_cpu_form_matches_oracle(gpu, oracle, method, bar, case):
    """generate_LFM_library_CPU (generate_LFM_library_CPU.m:18-70): the painted
    kernels through the frame projection, L2-normalised, against the oracle's
    literal patch projection (project_forward_patched.m:8-73: odd lenslet
    patch, conv2 'full', centred paste clipped to the sensor) in FP64."""
    import sid_gb300 as s
    from sid_gb300 import synthetic
    N, Z, M, L = 5, 7, 41, 12
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.5, sigma_max=6.0)
    rng = np.random.default_rng(21)
    c = np.stack([rng.uniform(1, X, 10), rng.uniform(1, X, 10), rng.uniform(1, Z, 10)], 1)
    c[0] = [1.0, 1.0, 1.0]
    c[1] = [X - 0.5, X / 2, Z]
    c[2] = [30.5, 12.5, 3.5]
    W = None
    if case == "kernel":
        W = rng.random((7, 7, 3)).astype(np.float32)
        W[W < 0.2] = 0
    r, dim = 4, [1.0, 1.0, 2.0]
    got = s.to_numpy(s.generate_LFM_library_CPU(c, {"H": H}, r, dim, (X, X, Z), kernel=W, method=method))
    ref = oracle.generate_library_cpu(c, H, r, dim, (X, X), kernel=W)
    assert got.shape == ref.shape
    worst = max(rel_l2(got[n], ref[n]) for n in range(len(c)))
    assert worst < bar, worst
    np.testing.assert_allclose(np.linalg.norm(got.astype(np.float64), axis=1), 1.0, rtol=1e-5)
    cols = s.to_numpy(s.generate_LFM_library_CPU(c, {"H": H}, r, dim, (X, X, Z), kernel=W, method=method,
                                                 layout="columns"))
    np.testing.assert_array_equal(cols, got.T)


@pytest.mark.parametrize("M", [21, 23])
def test_patch_projection_equals_frame_projection(oracle, M):
    """project_forward_patched.m's patch (an odd number of lenslets, conv2
    'full', pasted centred and clipped) equals the frame's conv2 'same'
    projection of the painted volume for odd Nnum and odd PSF width: the
    identity the library's CPU-twin form rests on (FP64, CPU).  With an even
    width the paste's index range runs one past the projection (MATLAB stops
    with an index error; so does the oracle)."""
    from sid_gb300 import synthetic
    N, Z = 5, 4
    X = N * 8
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.0, sigma_max=3.0)
    rng = np.random.default_rng(4)
    c = np.stack([rng.uniform(1, X, 6), rng.uniform(1, X, 6), rng.uniform(1, Z, 6)], 1)
    c[0] = [1.0, 1.0, 1.0]
    c[1] = [X - 0.3, 3.5, Z]
    rows = oracle.generate_library_cpu(c, H, 3, [1, 1, 1.5], (X, X))
    for n, (vox, vals) in enumerate(oracle.library_kernel_voxels(c, 3, [1, 1, 1.5], (X, X), Z)):
        V = np.zeros((X, X, Z), order="F")
        V[vox[:, 0], vox[:, 1], vox[:, 2]] = vals
        ref = oracle.forward_project(H, V).ravel(order="F")
        ref = ref / np.linalg.norm(ref)
        np.testing.assert_allclose(rows[n], ref, rtol=0, atol=1e-12)


def test_patch_projection_even_width_fails_like_the_reference(oracle):
    """An even PSF width makes the 'full' projection even, and the centred
    paste's range for a neuron away from the sensor's far edges one pixel
    longer than it (project_forward_patched.m:63-72): an index error."""
    from sid_gb300 import synthetic
    N, Z, X = 5, 2, 80
    H = synthetic.gaussian_psf(22, N, Z, sigma_min=1.0, sigma_max=2.0)
    with pytest.raises(ValueError):
        oracle.generate_library_cpu(np.array([[40.0, 40.0, 1.0]]), H, 3, [1, 1, 1.0], (X, X))
