"""Neuron-kernel composition of the projector (reconstruct_S.m:110-114,
126-127, 188-189) and generate_kernel.m: kernels against their definitions on
the CPU; the composed GPU operator and solvers against the FP64 oracle."""
import numpy as np
import pytest

from tests.conftest import rel_l2


def test_convn_same_oracle_matches_definition(oracle):
    rng = np.random.default_rng(0)
    V = rng.uniform(0, 1, (9, 8, 5))
    for shape in [(3, 3, 3), (4, 3, 2), (2, 5, 1)]:
        k = rng.uniform(0, 1, shape)
        o = [s // 2 for s in shape]
        ref = np.zeros_like(V)
        for x in range(9):
            for y in range(8):
                for z in range(5):
                    acc = 0.0
                    for i in range(shape[0]):
                        for j in range(shape[1]):
                            for l in range(shape[2]):
                                xx, yy, zz = x + o[0] - i, y + o[1] - j, z + o[2] - l
                                if 0 <= xx < 9 and 0 <= yy < 8 and 0 <= zz < 5:
                                    acc += V[xx, yy, zz] * k[i, j, l]
                    ref[x, y, z] = acc
        np.testing.assert_allclose(oracle.convn_same(V, k), ref, rtol=1e-12, atol=1e-14)


def test_generate_kernel_shapes():
    from sid_gb300 import generate_kernel
    b = generate_kernel("ball", [2, 1])
    assert b.shape == (5, 5, 3)
    # ball: x^2/4 + y^2/4 + z^2 <= 1 on the integer grid, unit L2 norm
    g = np.mgrid[-2:3, -2:3, -1:2]
    inside = (g[0] ** 2 / 4 + g[1] ** 2 / 4 + g[2] ** 2) <= 1
    np.testing.assert_allclose(b, inside / np.sqrt(inside.sum()), rtol=1e-12)
    gk = generate_kernel("gaussian", [1.0, 1.0])
    assert gk.shape == (11, 11, 7)
    assert abs(np.linalg.norm(gk) - 1) < 1e-12 and np.allclose(gk, gk[::-1, ::-1, ::-1])
    # separable: the lateral slices are scalar multiples of one another
    c = gk[:, :, 3]
    np.testing.assert_allclose(gk[:, :, 2], c * (gk[5, 5, 2] / gk[5, 5, 3]), rtol=1e-10)
    lz = generate_kernel("lorentz", [0.5, 0.4])
    assert lz.shape == (7, 7, 5) and abs(np.linalg.norm(lz) - 1) < 1e-12
    u = generate_kernel("user", np.ones((2, 3, 1)))
    np.testing.assert_allclose(u, np.ones((2, 3, 1)) / np.sqrt(6))


@pytest.fixture(scope="module")
def small(gpu, oracle):
    from sid_gb300 import Projector, synthetic
    N, Z, M, L = 5, 3, 31, 9
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.0, sigma_max=3.0)
    Vt = synthetic.blob_volume(X, X, Z, 6, sigma=(1.5, 1.5), seed=4)
    P = Projector(H, (X, X), None, methods=("direct", "spectral_f32", "spectral_mixed"))
    return H, Vt, P


KERNELS = {"ball": ("ball", [2, 1]), "even_user": ("user", np.arange(1, 25, dtype=float).reshape(4, 3, 2)),
           "gaussian": ("gaussian", [1.6, 0.8]),
           # wider than 32 along x: the generic kernel
           "wide_user": ("user", np.random.default_rng(5).uniform(0, 1, (33, 3, 2)))}


@pytest.mark.gpu
@pytest.mark.parametrize("kname", list(KERNELS))
@pytest.mark.parametrize("method,tol", [("direct", 1e-5), ("spectral_f32", 1e-5), ("spectral_mixed", 1e-4)])
def test_composed_projections_match_oracle(small, oracle, kname, method, tol):
    import sid_gb300 as s
    H, Vt, P = small
    k = s.generate_kernel(*KERNELS[kname])
    P.set_kernel(k)
    try:
        f = s.to_numpy(P.forward(Vt, method=method))
        ref_f = oracle.forward_project(H, oracle.convn_same(Vt, k))
        assert rel_l2(f, ref_f) < tol
        b = s.to_numpy(P.adjoint(ref_f.astype(np.float32), method=method))
        ref_b = oracle.convn_same(oracle.backward_project(H, ref_f), k)
        assert rel_l2(b, ref_b) < tol
    finally:
        P.set_kernel(None)
    # removed again: the raw projector
    assert rel_l2(s.to_numpy(P.forward(Vt, method=method)), oracle.forward_project(H, Vt)) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("method,tol", [("direct", 1e-5), ("spectral_mixed", 1e-4)])
def test_composed_isra_matches_oracle(small, oracle, method, tol):
    import sid_gb300 as s
    H, Vt, P = small
    k = s.generate_kernel("ball", [2, 1])
    fwd = lambda v: oracle.forward_project(H, oracle.convn_same(v, k))  # noqa: E731
    bwd = lambda i: oracle.convn_same(oracle.backward_project(H, i), k)  # noqa: E731
    y = oracle.forward_project(H, Vt)
    Htf = bwd(y)
    ref = oracle.deconvRL(fwd, bwd, Htf, 8, Htf)
    P.set_kernel(k)
    try:
        out = s.to_numpy(P.isra(Htf.astype(np.float32), Htf.astype(np.float32), 8, method=method))
    finally:
        P.set_kernel(None)
    assert rel_l2(out, ref) < 10 * tol, rel_l2(out, ref)
