"""Pseudo-inverse timeseries extraction (incremental_temporal_update_gpu.m,
LS branch) on the GPU against the FP64 oracle."""
import numpy as np
import pytest

from tests.conftest import rel_l2


def extraction_problem(seed, K=24, P=5000, N=350, density=0.04):
    rng = np.random.default_rng(seed)
    F = rng.random((K, P)) * (rng.random((K, P)) < density)
    F[np.arange(K), rng.choice(P, K, replace=False)] += 1.0  # every footprint non-empty
    T = np.abs(rng.standard_normal((K, N)))
    Y = F.T @ T + 0.01 * rng.standard_normal((P, N))
    return np.asfortranarray(F.astype(np.float32)), np.asfortranarray(Y.astype(np.float32)), T


def test_oracle_pinv_is_least_squares(oracle):
    F, Y, _ = extraction_problem(0, K=6, P=300, N=20)
    out = oracle.pinv_extract(F, [Y[:, :7], Y[:, 7:]])
    ls = np.linalg.lstsq(F.T.astype(np.float64), Y.astype(np.float64), rcond=None)[0]
    np.testing.assert_allclose(np.hstack(out), ls, rtol=1e-9, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "split"])
def test_extract_gpu_matches_oracle(gpu, oracle, prec):
    import sid_gb300 as s
    F, Y, _ = extraction_problem(1)
    base = np.linspace(0.8, 1.2, Y.shape[1]).astype(np.float32)
    ref = np.hstack(oracle.pinv_extract(F, [Y[:, c:c + 100] / base[c:c + 100] for c in range(0, Y.shape[1], 100)]))
    ex = s.Extractor(F, prec=prec)
    out = None
    for c in range(0, Y.shape[1], 100):
        n = min(100, Y.shape[1] - c)
        if out is None:
            import torch
            out = torch.empty((Y.shape[1], F.shape[0]), device="cuda").T
        ex.apply(Y[:, c:c + n], base[c:c + n], out=out, col0=c)
    cond = np.linalg.cond(F.astype(np.float64) @ F.T.astype(np.float64))
    assert cond < 1e3
    assert rel_l2(s.to_numpy(out), ref) < 1e-5


@pytest.mark.gpu
def test_extract_gpu_function_api(gpu, oracle):
    import sid_gb300 as s
    F, Y, _ = extraction_problem(2, N=230)
    ref = np.hstack(oracle.pinv_extract(F, [Y]))
    T = s.incremental_temporal_update_gpu(F, Y, None, 64, {})
    assert T.shape == (F.shape[0], Y.shape[1])
    assert rel_l2(s.to_numpy(T), ref) < 1e-5
    # pixel-major forward model and FP16 frames
    ex = s.Extractor(np.asfortranarray(F.T), pixel_major=True)
    Th = ex.apply(Y.astype(np.float16))
    refh = np.hstack(oracle.pinv_extract(F, [Y.astype(np.float16).astype(np.float32)]))
    assert rel_l2(s.to_numpy(Th), refh) < 1e-5


@pytest.mark.gpu
def test_extract_gpu_pixel_subset(gpu, oracle):
    import sid_gb300 as s
    F, Y, _ = extraction_problem(3, N=90)
    keep = np.arange(Y.shape[0]) % 2 == 0
    Fk = np.asfortranarray(F[:, keep])
    ref = np.hstack(oracle.pinv_extract(Fk, [Y[keep]]))
    T = s.incremental_temporal_update_gpu(Fk, Y, None, 50, {"idx": keep})
    assert rel_l2(s.to_numpy(T), ref) < 1e-5


@pytest.mark.gpu
def test_extract_gpu_rejects_singular_gram(gpu):
    import sid_gb300 as s
    F, _, _ = extraction_problem(4, K=8, P=400)
    F[5] = F[2]  # two identical footprints: F*F' is singular
    with pytest.raises(s.SidError):
        s.Extractor(np.asfortranarray(F))


@pytest.mark.gpu
def test_extract_gpu_nonneg_branch(gpu):
    import sid_gb300 as s
    F, Y, T_true = extraction_problem(5, K=10, P=2000, N=120)
    T = s.to_numpy(s.incremental_temporal_update_gpu(F, Y, None, 40, {"non_neg_on": True}))
    assert T.min() >= 0.0
    assert rel_l2(T, T_true) < 0.05
