"""merge_filters.m and SNR_order.m: the oracle on hand-checked cases (CPU), the
GPU implementation against the oracle."""
import numpy as np
import pytest


def test_matlab_smooth_known_values(oracle):
    y = np.array([1, 4, 9, 16, 25, 36, 49], dtype=float)
    np.testing.assert_allclose(oracle.matlab_smooth(y, 5), [1, 14 / 3, 11, 18, 27, 110 / 3, 49])
    # span 8 acts as 7
    np.testing.assert_allclose(oracle.matlab_smooth(y, 8), oracle.matlab_smooth(y, 7))


def test_highpass_as_mode_subtraction(oracle):
    """Zeroing DFT bins 1..6 and their mirrors of [x flip(x)] equals subtracting
    the six modes, the form the GPU kernel evaluates."""
    rng = np.random.default_rng(0)
    x = rng.standard_normal(301)
    n2 = 2 * len(x)
    ext = np.concatenate([x, x[::-1]])
    hh = np.fft.fft(ext)
    hh[1:7] = 0
    hh[-6:] = 0
    ref = np.real(np.fft.ifft(hh))[:len(x)]
    n = np.arange(len(x))
    got = x.copy()
    for m in range(1, 7):
        X = np.sum(ext * np.exp(-2j * np.pi * m * np.arange(n2) / n2))
        got -= 2 * np.real(X * np.exp(2j * np.pi * m * n / n2)) / n2
    np.testing.assert_allclose(got, ref, atol=1e-12)


def test_merge_filters_oracle_hand_case(oracle):
    # 4 components + background; 0 and 1 share their template and trace -> merged into 0
    P, F = 30, 50
    rng = np.random.default_rng(1)
    base = rng.standard_normal(F)
    ts = np.stack([base, base + 1e-3 * rng.standard_normal(F), rng.standard_normal(F), rng.standard_normal(F),
                   np.ones(F) + 0.1 * rng.standard_normal(F)])
    tp = np.zeros((4, P), dtype=np.float32)
    tp[0, 0:10] = 1
    tp[1, 2:10] = 1
    tp[2, 12:20] = 1
    tp[3, 22:28] = 1
    fm, t2, tp2, idx = oracle.merge_filters(np.arange(5)[:, None] * np.ones((5, 3)), ts, tp, np.arange(5))
    np.testing.assert_array_equal(idx, [0, 2, 3, 4])
    np.testing.assert_array_equal(tp2[0], (np.arange(P) < 10).astype(np.float32))


def _merge_case(seed, K=41, F=600, P=6000):
    rng = np.random.default_rng(seed)
    ts = rng.standard_normal((K, F)).astype(np.float32)
    tp = np.zeros((K - 1, P), dtype=np.float32)
    for k in range(K - 1):
        c = rng.integers(0, P - 200)
        tp[k, c:c + rng.integers(40, 200)] = 1
    for i in range(8):  # pairs (2i, 2i+1): shared footprint, correlated traces
        a, b = 2 * i, 2 * i + 1
        tp[b] = 0
        nz = np.flatnonzero(tp[a])
        tp[b, nz[: 2 * len(nz) // 3]] = 1
        ts[b] = ts[a] + 0.05 * rng.standard_normal(F).astype(np.float32)
    fm = rng.uniform(0, 1, (K, 97)).astype(np.float32)
    return np.asfortranarray(fm), np.asfortranarray(ts), np.asfortranarray(tp), np.arange(K) + 100


@pytest.mark.gpu
def test_merge_filters_matches_oracle(gpu, oracle):
    import sid_gb300 as s
    fm, ts, tp, idx = _merge_case(3)
    r_fm, r_ts, r_tp, r_idx = oracle.merge_filters(fm, ts, tp, idx, 0.9, True)
    assert len(r_idx) < len(idx)  # something merged
    g_fm, g_ts, g_tp, g_idx = s.merge_filters(fm, ts, tp, idx, {"limit": 0.9, "bg_sub": True})
    np.testing.assert_array_equal(g_idx, r_idx)
    np.testing.assert_array_equal(s.to_numpy(g_tp), r_tp)
    np.testing.assert_array_equal(s.to_numpy(g_ts), np.asarray(r_ts, dtype=np.float32))
    np.testing.assert_array_equal(s.to_numpy(g_fm), r_fm)


@pytest.mark.gpu
def test_snr_order_matches_oracle(gpu, oracle):
    import sid_gb300 as s
    rng = np.random.default_rng(4)
    K, F = 51, 1200
    tr = rng.standard_normal((K, F)) * rng.uniform(0.2, 2.0, (K, 1))
    for k in range(K):  # sparse transients of varying size
        for t0 in rng.integers(0, F - 60, 4):
            tr[k, t0:t0 + 40] += rng.uniform(0, 6) * np.exp(-np.arange(40) / 8.0)
    tr = np.asfortranarray(tr.astype(np.float32))
    ref, pp = oracle.snr_order(tr)
    got = s.SNR_order(tr)
    assert sorted(np.diff(np.sort(pp)))[0] > 1e-6  # no near-ties in the fixture
    np.testing.assert_array_equal(got, ref)
