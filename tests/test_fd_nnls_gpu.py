"""Central finite differences of the NNLS and demixing objectives against the
gradients formed with the GPU contractions (the adjoint checks of the temporal
NNLS and of the alternating S/T demixing):

* NNLS, min ||Y - A T||^2 / 2 with A = S' (P x K): grad_T = A'A T - A'Y from
  sid_gram and sid_cross, at 32 random entries of T;
* demixing, ||Y - S T||^2 / 2 (Y: P x F, S: P x R, T: R x F): grad_S =
  S (T T') - Y T' and grad_T = (S'S) T - S'Y, the back projection of the
  residual through the contractions, at 32 random entries each.

Differences are taken in FP64 on the host; the objectives are quadratic, so a
central difference is exact up to rounding.  Bars over the sampled entries:
1e-5 rel-L2 with FP32 contractions; 5e-5 with split-precision (BF16 hi/lo)
contractions, each within 1e-5 of FP64, whose difference the gradient is."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fd_col(Y, A, t, k, h):
    """[f(t + h e_k) - f(t - h e_k)] / 2h of f(t) = ||y - A t||^2 / 2 for one column."""
    r = Y - A @ t
    a = A[:, k]
    fp = 0.5 * np.sum((r - h * a) ** 2)
    fm = 0.5 * np.sum((r + h * a) ** 2)
    return (fp - fm) / (2 * h)


@pytest.mark.parametrize("prec,tol", [("fp32", 1e-5), ("split", 5e-5)])
def test_nnls_objective_central_differences(gpu, prec, tol):
    import sid_gb300 as s
    rng = np.random.default_rng(31)
    P, K, F = 30000, 48, 300
    A = np.asfortranarray(rng.uniform(0, 1, (P, K)).astype(np.float32) ** 4)
    T = np.asfortranarray(rng.uniform(0, 1, (K, F)).astype(np.float32))
    Y = np.asfortranarray((A.astype(np.float64) @ (2.0 * T) + 0.01 * rng.standard_normal((P, F))).astype(np.float32))
    ctx = s.Context()
    G = s.to_numpy(ctx.gram(A, prec=prec)).astype(np.float64)
    C = s.to_numpy(ctx.cross(A, Y, prec=prec)).astype(np.float64)
    grad = G @ T.astype(np.float64) - C
    ent = np.stack([rng.integers(0, K, 32), rng.integers(0, F, 32)], axis=1)
    A64, Y64, T64 = A.astype(np.float64), Y.astype(np.float64), T.astype(np.float64)
    fd = np.array([_fd_col(Y64[:, f], A64, T64[:, f], k, 1e-3 * max(abs(T64[k, f]), 1e-3)) for k, f in ent])
    g = grad[ent[:, 0], ent[:, 1]]
    assert np.linalg.norm(g - fd) / np.linalg.norm(fd) < tol, np.linalg.norm(g - fd) / np.linalg.norm(fd)


@pytest.mark.parametrize("prec,tol", [("fp32", 1e-5), ("split", 5e-5)])
def test_demixing_residual_adjoint_central_differences(gpu, prec, tol):
    import torch
    import sid_gb300 as s
    rng = np.random.default_rng(37)
    P, R, F = 20000, 40, 240
    S = np.asfortranarray(rng.uniform(0, 1, (P, R)).astype(np.float32) ** 3)
    T = np.asfortranarray(rng.uniform(0, 1, (R, F)).astype(np.float32))
    Y = np.asfortranarray((S.astype(np.float64) @ (0.8 * T) + 0.05).astype(np.float32))
    ctx = s.Context()
    S64, T64, Y64 = (x.astype(np.float64) for x in (S, T, Y))
    # grad_T = (S'S) T - S'Y
    QS = s.to_numpy(ctx.gram(S, prec=prec)).astype(np.float64)
    qT = s.to_numpy(ctx.cross(S, Y, prec=prec)).astype(np.float64)
    gT = QS @ T64 - qT
    # grad_S = S (T T') - Y T'; T T' = gram(T'), Y T' = cross(T', Y')'
    Tt = np.asfortranarray(T.T)
    QT = s.to_numpy(ctx.gram(Tt, prec=prec)).astype(np.float64)
    qS = s.to_numpy(ctx.cross(Tt, np.asfortranarray(Y.T), prec=prec)).astype(np.float64).T
    gS = S64 @ QT - qS
    torch.cuda.synchronize()
    eT = np.stack([rng.integers(0, R, 32), rng.integers(0, F, 32)], axis=1)
    fdT = np.array([_fd_col(Y64[:, f], S64, T64[:, f], k, 1e-3 * max(T64[k, f], 1e-3)) for k, f in eT])
    # entries of S: the objective restricted to row p is ||Y(p,:) - S(p,:) T||^2 / 2
    eS = np.stack([rng.integers(0, P, 32), rng.integers(0, R, 32)], axis=1)
    fdS = np.array([_fd_col(Y64[p, :], T64.T, S64[p, :], r, 1e-3 * max(S64[p, r], 1e-3)) for p, r in eS])
    for g, fd in ((gT[eT[:, 0], eT[:, 1]], fdT), (gS[eS[:, 0], eS[:, 1]], fdS)):
        assert np.linalg.norm(g - fd) / np.linalg.norm(fd) < tol, np.linalg.norm(g - fd) / np.linalg.norm(fd)
