"""The FP64 oracle against the golden fixtures and against properties of the
maths it restates (CPU only)."""
import numpy as np
import pytest

from tests.conftest import rel_l2

GOLDEN = "tests/golden/projector_cases.npz"
CASES = ["small_full", "ragged", "cropped", "nnum5"]


@pytest.fixture(scope="module")
def golden():
    import os
    from tests.conftest import ROOT
    return np.load(os.path.join(ROOT, GOLDEN))


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_golden(oracle, golden, case):
    g = {k.split("/")[1]: golden[k] for k in golden.files if k.startswith(case + "/")}
    f = oracle.forward_project(g["H"], g["V"], g["CAindex"])
    b = oracle.backward_project(g["H"], g["I"], g["CAindex"])
    assert rel_l2(f, g["fwd"]) < 1e-13
    assert rel_l2(b, g["adj"]) < 1e-13


@pytest.mark.parametrize("M", [7, 9, 10])
def test_oracle_adjoint_identity(oracle, M):
    """<Ax, y> == <x, A'y> exactly for odd widths; even widths follow the
    reference's imrotate centring, which is one pixel off the true adjoint."""
    rng = np.random.default_rng(M)
    N, Z, X, Y = 3, 2, 14, 11
    H = rng.random((M, M, N, N, Z)).astype(np.float32)
    V = rng.random((X, Y, Z))
    I = rng.random((X, Y))
    lhs = np.sum(oracle.forward_project(H, V) * I)
    rhs = np.sum(V * oracle.backward_project(H, I))
    if M % 2:
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    else:
        assert abs(lhs - rhs) > 1e-9 * abs(lhs)


def test_sampled_pixels_match_full(oracle):
    rng = np.random.default_rng(3)
    M, N, Z, X, Y = 11, 3, 3, 16, 13
    H = rng.random((M, M, N, N, Z)).astype(np.float32)
    V = rng.random((X, Y, Z))
    I = rng.random((X, Y))
    full_f = oracle.forward_project(H, V)
    full_b = oracle.backward_project(H, I)
    pix = np.stack([rng.integers(0, X, 20), rng.integers(0, Y, 20)], 1)
    vox = np.stack([rng.integers(0, X, 20), rng.integers(0, Y, 20), rng.integers(0, Z, 20)], 1)
    np.testing.assert_allclose(oracle.forward_project_pixels(H, V, pix), full_f[pix[:, 0], pix[:, 1]], rtol=1e-14)
    np.testing.assert_allclose(oracle.backward_project_voxels(H, I, vox), full_b[vox[:, 0], vox[:, 1], vox[:, 2]],
                               rtol=1e-14)


@pytest.mark.parametrize("M,N", [(11, 3), (10, 5)])
def test_cpu_baseline_computes_the_forward_projection(oracle, M, N):
    """The timed CPU baseline (FP32 lenslet-sparse loop) is the forward
    projection: equal to the FP64 oracle to FP32 rounding over all columns, and
    a column range [y0, y1) gives exactly those columns of the whole result."""
    rng = np.random.default_rng(M + N)
    Z, X, Y = 3, 4 * N + 2, 3 * N + 1
    H = rng.random((M, M, N, N, Z)).astype(np.float32)
    V = (rng.random((X, Y, Z)) * (rng.random((X, Y, Z)) < 0.3)).astype(np.float32)
    full = oracle.baseline_forward_f32(H, V, nthreads=2)
    assert rel_l2(full, oracle.forward_project(H, V)) < 1e-6
    y0, y1 = 2, Y - 3
    part = oracle.baseline_forward_f32(H, V, y0, y1, nthreads=1)
    np.testing.assert_array_equal(part[:, y0:y1], full[:, y0:y1])
    assert not part[:, :y0].any() and not part[:, y1:].any()


def test_matlab_quantile(oracle):
    rng = np.random.default_rng(0)
    v = rng.random(1001)
    for p in [0.0, 1e-4, 0.3, 0.8, 1 - 1e-4, 1.0]:
        assert abs(oracle.matlab_quantile(v, p) - np.quantile(v, p, method="hazen")) < 1e-14


def test_isra_monotone_objective(oracle):
    """ISRA does not increase ||y - Ax||^2 (its fixed points are LS solutions)."""
    rng = np.random.default_rng(5)
    M, N, Z, X = 9, 3, 2, 12
    H = rng.random((M, M, N, N, Z)).astype(np.float32)
    xt = rng.random((X, X, Z))
    y = oracle.forward_project(H, xt)
    fwd = lambda v: oracle.forward_project(H, v)  # noqa: E731
    bwd = lambda i: oracle.backward_project(H, i)  # noqa: E731
    Htf = bwd(y)
    prev = None
    x = Htf.copy()
    for _ in range(5):
        x = oracle.deconvRL(fwd, bwd, Htf, 1, x)
        obj = np.sum((y - fwd(x)) ** 2)
        if prev is not None:
            assert obj <= prev * (1 + 1e-12)
        prev = obj


def test_ls_deconv_decreases_objective(oracle):
    rng = np.random.default_rng(6)
    M, N, Z, X = 9, 3, 2, 12
    H = rng.random((M, M, N, N, Z)).astype(np.float32)
    y = oracle.forward_project(H, rng.random((X, X, Z)))
    fwd = lambda v: oracle.forward_project(H, v)  # noqa: E731
    bwd = lambda i: oracle.backward_project(H, i)  # noqa: E731
    Htf = bwd(y)
    objs = []
    for it in [0, 2, 8]:
        x = oracle.LS_deconv(fwd, bwd, Htf, {"max_iter": it})
        objs.append(np.sum((y - fwd(x)) ** 2))
    assert objs[2] < objs[1] < objs[0]


def _sparse_nnls_problem(seed, P=600, K=40, F=8, dens=0.05):
    rng = np.random.default_rng(seed)
    A = rng.random((P, K)) * (rng.random((P, K)) < dens)
    A[rng.integers(0, P, K), np.arange(K)] += 1.0  # no empty column
    T = rng.random((K, F)) * (rng.random((K, F)) < 0.5)
    Y = A @ T + 0.01 * rng.standard_normal((P, F))
    return A, Y


def _kkt(A, Y, X, lam=0.0):
    g = A.T @ (A @ X - Y) + lam
    scale = np.abs(A.T @ Y).max()
    return float(np.abs(np.where(X > 0, g, np.minimum(g, 0))).max() / scale)


@pytest.mark.parametrize("solver", ["fast_nnls", "LS_nnls"])
def test_oracle_nnls_reaches_scipy_optimum(oracle, solver):
    """fast_nnls.m / LS_nnls.m restated: on a well-conditioned problem the
    retired columns sit at the NNLS optimum of an independent solver."""
    from scipy.optimize import nnls
    A, Y = _sparse_nnls_problem(1)
    if solver == "fast_nnls":
        X = oracle.fast_nnls(A, Y, {})[0]
    else:
        X = oracle.LS_nnls(A, Y, {})[0]
    Xs = np.stack([nnls(A, Y[:, j])[0] for j in range(Y.shape[1])], axis=1)
    assert np.linalg.norm(X - Xs) / np.linalg.norm(Xs) < 1e-4
    assert X.min() >= 0 and _kkt(A, Y, X) < 1e-4


@pytest.mark.parametrize("solver", ["fast_nnls", "LS_nnls"])
def test_oracle_nnls_lambda_is_l1_weight(oracle, solver):
    """opts.lambda enters as h = A'Y - lambda (LS_nnls.m:76) or
    df = diag(h)(-A'Y + lambda) (fast_nnls.m:57): both minimise
    0.5 ||A x - y||^2 + lambda * sum(x) over x >= 0."""
    A, Y = _sparse_nnls_problem(2)
    lam = 0.05
    if solver == "fast_nnls":
        X = oracle.fast_nnls(A, Y, {"lambda": lam})[0]
    else:
        X = oracle.LS_nnls(A, Y, {"lambda": lam})[0]
    assert X.min() >= 0 and _kkt(A, Y, X, lam) < 1e-4


def test_rl_poisson_is_em(oracle):
    """Richardson-Lucy is the EM algorithm of the Poisson likelihood: every
    iteration keeps sum(A x) = sum(y) (x_new = x A'(y/Ax) / A'1) and does not
    lower sum(y log(Ax) - Ax)."""
    rng = np.random.default_rng(8)
    M, N, Z, X = 9, 3, 2, 12
    H = rng.random((M, M, N, N, Z)).astype(np.float32)
    fwd = lambda v: oracle.forward_project(H, v)  # noqa: E731
    bwd = lambda i: oracle.backward_project(H, i)  # noqa: E731
    y = rng.poisson(50.0 * fwd(rng.random((X, X, Z)))).astype(np.float64)
    x = np.full((X, X, Z), 0.5)
    prev = None
    for _ in range(6):
        x = oracle.rl_poisson(fwd, bwd, y, 1, x)
        ax = fwd(x)
        assert abs(ax.sum() - y.sum()) <= 1e-9 * y.sum()
        ll = float(np.sum(y * np.log(ax) - ax))
        if prev is not None:
            assert ll >= prev - 1e-9 * abs(prev)
        prev = ll
