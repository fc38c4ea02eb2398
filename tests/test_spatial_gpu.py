"""Spatial update (update_spatial_component -> reg_nnls -> NQP) on the GPU
against the FP64 oracle, and the oracle's NQP against the exact NNLS optimum."""
import numpy as np
import pytest

from tests.conftest import rel_l2


def demix_problem(seed, R=7, F=60, side=24):
    rng = np.random.default_rng(seed)
    P = side * side
    tmpl = np.zeros((R, P), dtype=bool)
    yy, xx = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    S = np.zeros((R + 1, P))
    for r in range(R):
        cx, cy, rad = rng.uniform(4, side - 4), rng.uniform(4, side - 4), rng.uniform(3, 7)
        m = ((xx - cx) ** 2 + (yy - cy) ** 2 < rad ** 2).ravel()
        tmpl[r] = m
        S[r, m] = rng.random(m.sum())
    S[R] = 0.05
    T = np.abs(rng.standard_normal((R + 1, F)))
    T[R] = 1.0
    Y = S.T @ T + 0.01 * rng.standard_normal((P, F))
    return np.asfortranarray(T.astype(np.float32)), np.asfortranarray(Y.astype(np.float32)), tmpl


def test_oracle_nqp_is_nnls_optimum(oracle):
    from scipy.optimize import nnls
    rng = np.random.default_rng(0)
    for n in [1, 3, 8, 15]:
        A = rng.random((40, n))
        d = rng.standard_normal(40)
        x, _, _ = oracle.NQP(A.T @ A, -(A.T @ d))
        xs, _ = nnls(A, d)
        np.testing.assert_allclose(x, xs, atol=1e-10)


def test_oracle_reg_nnls_options_pinned(oracle):
    """reg_nnls.m:40-66 against independent forms of the same problem: lamb_L2
    is NNLS on [A; sqrt(l2) I] x ~ [d; 0]; use_std is NNLS on A and d with their
    means over the rows removed; with lamb_L1 and lamb_orth_L1 the solution
    meets the KKT conditions of 0.5 x'Qx + q'x over x >= 0."""
    from scipy.optimize import nnls
    rng = np.random.default_rng(4)
    A = rng.random((60, 7))
    d = A @ (rng.random(7) * (rng.random(7) < 0.6)) + 0.05 * rng.standard_normal(60)
    l2 = 0.3
    x = oracle.reg_nnls(A, d, {"lamb_L2": l2})
    xs, _ = nnls(np.vstack([A, np.sqrt(l2) * np.eye(7)]), np.concatenate([d, np.zeros(7)]))
    np.testing.assert_allclose(x, xs, atol=1e-10)
    x = oracle.reg_nnls(A, d, {"use_std": True})
    xs, _ = nnls(A - A.mean(axis=0), d - d.mean())
    np.testing.assert_allclose(x, xs, atol=1e-10)
    opts = {"lamb_L1": 0.2, "lamb_orth_L1": 0.05, "bg_sub": 1}
    x = oracle.reg_nnls(A, d, opts)
    hilf = np.ones((7, 7)) - np.eye(7)
    hilf[:, -1] = 0
    hilf[-1, :] = 0
    g = (A.T @ A + 0.05 * hilf) @ x - A.T @ d + 0.2
    assert x.min() >= 0
    assert np.abs(g[x > 0]).max(initial=0.0) < 1e-9
    assert g[x == 0].min(initial=0.0) > -1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [{"bg_sub": 1}, {"bg_sub": 1, "lamb_L1": 0.01, "lamb_L2": 0.05,
                                                   "lamb_orth_L1": 1e-3}, {"bg_sub": 0}, {"bg_sub": 1, "use_std": True}])
def test_spatial_update_matches_oracle(gpu, oracle, opts):
    import sid_gb300 as s
    T, Y, tmpl = demix_problem(4)
    if not opts.get("bg_sub", 1):
        T = np.asfortranarray(T[:-1])
    ref = oracle.update_spatial_component(T, Y, tmpl, opts)
    got = s.to_numpy(s.update_spatial_component(T, Y, tmpl, opts))
    assert got.shape == ref.shape
    # FP32 products into an FP64 active-set solve: the support (which entries
    # are zero) must agree and the values within the FP32 path's bar
    assert rel_l2(got, ref) < 1e-4, rel_l2(got, ref)


def _nqp_problems(rng, n, B):
    Qs = np.empty((n, n, B))
    bs = np.empty((n, B))
    for k in range(B):
        M = rng.standard_normal((n + 3, n))
        Qs[:, :, k] = M.T @ M + 1e-3 * np.eye(n)
        bs[:, k] = rng.standard_normal(n)
    return np.asfortranarray(Qs), np.asfortranarray(bs)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 5, 17, 32, 33, 64, 128])
def test_nqp_batched_matches_oracle(gpu, oracle, n):
    """[x, w, info] = NQP(Q, b) (NQP.m:42-178) for a stack of independent
    problems against the oracle's Lawson-Hanson restatement, both FP64."""
    import sid_gb300 as s
    rng = np.random.default_rng(11 + n)
    Qs, bs = _nqp_problems(rng, n, 40)
    x, w, info = s.NQP(Qs, bs)
    x, w, its = x.cpu().numpy(), w.cpu().numpy(), info["iter"].cpu().numpy()
    same_iters = 0
    for k in range(bs.shape[1]):
        xo, wo, ito = oracle.NQP(Qs[:, :, k], bs[:, k])
        scale = np.abs(bs[:, k]).max()
        np.testing.assert_allclose(x[:, k], xo, rtol=1e-9, atol=1e-12 * scale)
        np.testing.assert_allclose(w[:, k], wo, rtol=1e-8, atol=1e-9 * scale)
        same_iters += int(its[k] == ito)
    # FMA contraction differs between the host and device compilers: an
    # active-set tie could take another order, never a different optimum
    assert same_iters >= 0.95 * bs.shape[1]
    x1, w1, info1 = s.NQP(Qs[:, :, 0], bs[:, 0])
    assert tuple(x1.shape) == (n,) and isinstance(info1["iter"], int)
    np.testing.assert_array_equal(x1.cpu().numpy(), x[:, 0])


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [{}, {"lamb_L1": 0.1, "lamb_L2": 0.05},
                                  {"use_std": True, "lamb_orth_L1": 0.02, "bg_sub": 1}])
def test_reg_nnls_matches_oracle(gpu, oracle, opts):
    """x = reg_nnls(A, d, opts) (reg_nnls.m:40-69)."""
    import sid_gb300 as s
    rng = np.random.default_rng(12)
    A = rng.random((200, 12))
    d = A @ (rng.random(12) * (rng.random(12) < 0.6)) + 0.01 * rng.standard_normal(200)
    x = s.reg_nnls(A, d, opts).cpu().numpy()
    xo = oracle.reg_nnls(A, d, opts)
    np.testing.assert_allclose(x, xo, rtol=1e-8, atol=1e-10 * np.abs(xo).max())


@pytest.mark.gpu
def test_nqp_rejects_oversized_problem(gpu):
    import sid_gb300 as s
    with pytest.raises(s.SidError):
        s.NQP(np.eye(4097), np.ones(4097))


def crowded_problem(seed, R=60, F=400, side=16):
    """R templates that all cover the centre of a small field: the centre
    pixels have up to R + 1 covering components (with the background), far
    more than the 32 a thread keeps in registers."""
    rng = np.random.default_rng(seed)
    P = side * side
    yy, xx = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    tmpl = np.zeros((R, P), dtype=bool)
    S = np.zeros((R + 1, P))
    for r in range(R):
        cx, cy = side / 2 + rng.uniform(-2, 2), side / 2 + rng.uniform(-2, 2)
        rad = rng.uniform(4, 8)
        m = ((xx - cx) ** 2 + (yy - cy) ** 2 < rad ** 2).ravel()
        tmpl[r] = m
        S[r, m] = rng.random(m.sum())
    S[R] = 0.05
    # sparse transients keep the 61 x 61 pixel Grams well conditioned (about 75),
    # so FP32 products into the FP64 solve stay within the 1e-4 bar
    T = rng.random((R + 1, F)) * (rng.random((R + 1, F)) < 0.2)
    T[R] = 1.0
    Y = S.T @ T + 0.01 * rng.standard_normal((P, F))
    return np.asfortranarray(T.astype(np.float32)), np.asfortranarray(Y.astype(np.float32)), tmpl


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [{"bg_sub": 1}, {"bg_sub": 1, "lamb_L2": 0.05, "lamb_orth_L1": 1e-3}])
def test_spatial_update_crowded_pixels(gpu, oracle, opts):
    """update_spatial_component.m:86-97 solves every pixel whatever the number
    of neurons covering it: pixels with 33 to 61 components against the oracle."""
    import sid_gb300 as s
    T, Y, tmpl = crowded_problem(8)
    counts = tmpl.sum(axis=0) + 1
    assert counts.max() > 40 and (counts > 32).sum() >= 20
    ref = oracle.update_spatial_component(T, Y, tmpl, opts)
    got = s.to_numpy(s.update_spatial_component(T, Y, tmpl, opts))
    big = counts > 32
    assert rel_l2(got[:, big], ref[:, big]) < 1e-4, rel_l2(got[:, big], ref[:, big])
    assert rel_l2(got, ref) < 1e-4, rel_l2(got, ref)
