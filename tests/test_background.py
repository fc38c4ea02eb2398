"""Rank-1 background factorisation and standard-deviation image
(rank_1_factorization.m, compute_std_image.m): the oracle against NumPy's own
definitions on the CPU, the GPU scans against the oracle."""
import numpy as np
import pytest

from tests.conftest import rel_l2


def test_oracle_std_image_is_population_std(oracle):
    rng = np.random.default_rng(1)
    Y = rng.uniform(0, 1, (300, 70))
    np.testing.assert_allclose(oracle.compute_std_image(Y), Y.std(axis=1), rtol=1e-12)


def test_oracle_rank1_recovers_factors(oracle):
    rng = np.random.default_rng(2)
    s0, t0 = rng.uniform(0.5, 1, 400), rng.uniform(0.5, 1, 90)
    s, t = oracle.rank_1_factorization(np.outer(s0, t0), 2)
    np.testing.assert_allclose(t, t0 / np.linalg.norm(t0), rtol=1e-12)
    np.testing.assert_allclose(np.outer(s, t), np.outer(s0, t0), rtol=1e-12)


def _movie(P, F, seed):
    rng = np.random.default_rng(seed)
    base = rng.uniform(0.2, 1.0, P)[:, None] * rng.uniform(0.5, 1.5, F)[None, :]
    return np.asfortranarray(base + 0.3 * rng.uniform(0, 1, (P, F)))


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float32, np.float16])
@pytest.mark.parametrize("iters", [1, 2, 3])
def test_rank1_and_fused_std_match_oracle(gpu, oracle, dtype, iters):
    import sid_gb300 as s
    Y = _movie(40001, 2500, 3).astype(dtype)  # F above the 2048-frame staging chunk, P odd
    ref_s, ref_t = oracle.rank_1_factorization(Y.astype(np.float64), iters)
    ref_std = oracle.compute_std_image(Y.astype(np.float64), ref_s, ref_t)
    ctx = s.Context()
    bs, bt, sd = ctx.rank_1_factorization(Y, iters, std_image=True)
    assert rel_l2(bs.cpu().numpy(), ref_s) < 1e-5
    assert rel_l2(bt.cpu().numpy(), ref_t) < 1e-5
    assert rel_l2(sd.cpu().numpy(), ref_std) < 1e-5
    bs2, bt2 = s.rank_1_factorization(Y, iters)
    np.testing.assert_array_equal(bs2.cpu().numpy(), bs.cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("with_factors", [False, True])
def test_std_image_matches_oracle(gpu, oracle, with_factors):
    import sid_gb300 as s
    Y = _movie(9999, 777, 4).astype(np.float16)
    rng = np.random.default_rng(5)
    y1 = rng.uniform(0, 0.01, Y.shape[0]).astype(np.float32) if with_factors else None
    y2 = rng.uniform(0, 1, Y.shape[1]).astype(np.float32) if with_factors else None
    ref = oracle.compute_std_image(Y.astype(np.float64), y1, y2)
    got = s.compute_std_image(Y, y1, y2).cpu().numpy()
    assert rel_l2(got, ref) < 1e-5


@pytest.mark.gpu
def test_rank1_full_size_exact_rank1_movie(gpu):
    """1,010,025 pixels x 3000 frames (the FP16 movie size of the NNLS
    workload): a movie that is exactly s0 t0' in FP32 is factored back, t to
    1e-6 of t0/||t0||, and its std image about the factors is ~0."""
    import torch
    import sid_gb300 as s
    P, F = 1010025, 3000
    g = torch.Generator(device="cuda").manual_seed(9)
    s0 = torch.rand(P, generator=g, device="cuda") + 0.5
    t0 = torch.rand(F, generator=g, device="cuda") + 0.5
    Y = torch.outer(t0, s0).t()  # column-major P x F view
    bs, bt, sd = s.Context().rank_1_factorization(Y, 2, std_image=True)
    tn = (t0 / torch.linalg.vector_norm(t0.double())).double()
    assert float(torch.linalg.vector_norm(bt.double() - tn) / torch.linalg.vector_norm(tn)) < 1e-6
    rec = torch.linalg.vector_norm(bs.double()) * float(torch.linalg.vector_norm(bt.double()))
    assert abs(rec / float(torch.linalg.vector_norm(s0.double()) * torch.linalg.vector_norm(t0.double())) - 1) < 1e-5
    del Y
    assert bool(torch.isfinite(sd).all())
