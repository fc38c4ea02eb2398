"""NMF steps (T_update.m, S_update.m): the oracle's descent properties and
MATLAB semantics on the CPU; the GPU steps against the FP64 oracle."""
import numpy as np
import pytest

from tests.conftest import rel_l2


def nmf_problem(seed, P=2000, R=10, F=150, f16=False):
    rng = np.random.default_rng(seed)
    S_true = rng.random((P, R)) * (rng.random((P, R)) < 0.3)
    T_true = np.abs(rng.standard_normal((R, F)))
    Y = S_true @ T_true + 0.05 * rng.standard_normal((P, F))
    S0 = rng.random((P, R)) * (rng.random((P, R)) < 0.4)
    T0 = np.abs(rng.standard_normal((R, F))) * (rng.random((R, F)) < 0.8)
    Y = Y.astype(np.float16 if f16 else np.float32)
    return (np.asfortranarray(Y), np.asfortranarray(S0.astype(np.float32)), np.asfortranarray(T0.astype(np.float32)))


def hilf_matrix(R):
    return np.asfortranarray((np.ones((R, R)) - np.eye(R)).astype(np.float32))


def objective(Y, S, T):
    return float(np.sum((np.asarray(Y, np.float64) - S @ T) ** 2))


# ---------------------------------------------------------------- CPU ------
def test_oracle_zscore_is_matlab(oracle):
    T = np.array([[1.0, 2.0, 4.0], [3.0, 2.0, 0.0], [5.0, 2.0, 1.0]])
    z = oracle._matlab_zscore(T)
    # columns standardised (MATLAB zscore on a matrix works along dimension 1)
    np.testing.assert_allclose(z.mean(axis=0), 0.0, atol=1e-15)
    np.testing.assert_allclose(z[:, 0], (T[:, 0] - 3.0) / 2.0)
    # a constant column has zero deviation: MATLAB divides by 1
    np.testing.assert_allclose(z[:, 1], 0.0)
    # a single row is standardised along its frames
    r = oracle._matlab_zscore(np.array([[1.0, 2.0, 3.0]]))
    np.testing.assert_allclose(r, [[-1.0, 0.0, 1.0]])


def test_oracle_t_update_descends(oracle):
    Y, S, T = nmf_problem(0, P=400, R=6, F=50)
    f0 = objective(Y, S.astype(np.float64), T.astype(np.float64))
    S1, T1 = oracle.T_update(Y, T, S, {})
    assert objective(Y, S1, T1) < f0
    assert T1.min() >= 0.0
    # exact line search: a second step from the new point still descends
    S2, T2 = oracle.T_update(Y, T1, S1, {})
    assert objective(Y, S2, T2) <= objective(Y, S1, T1)


def test_oracle_s_update_descends(oracle):
    Y, S, T = nmf_problem(1, P=400, R=6, F=50)
    f0 = objective(Y, S.astype(np.float64), T.astype(np.float64))
    S1, T1 = oracle.S_update(Y, S, T, {})
    assert objective(Y, S1, T1) < f0
    assert S1.min() >= 0.0
    S2, _ = oracle.S_update(Y, S, T, {"pointwise": True})
    assert objective(Y, S2, T) < f0


def test_oracle_s_update_orth_normalises(oracle):
    Y, S, T = nmf_problem(2, P=300, R=5, F=40)
    S1, T1 = oracle.S_update(Y, S, T, {"lamb_orth_L1": 0.01, "hilf": hilf_matrix(5)})
    np.testing.assert_allclose(np.linalg.norm(S1, axis=0), 1.0, rtol=1e-12)
    # T's rows carry the norms: T1 = platz' .* T
    ratio = T1 / np.where(T == 0, np.nan, T.astype(np.float64))
    np.testing.assert_allclose(np.nanmax(ratio, axis=1), np.nanmin(ratio, axis=1), rtol=1e-12)


def test_oracle_s_update_rejects_spatial_tv(oracle):
    Y, S, T = nmf_problem(3, P=100, R=3, F=10)
    with pytest.raises(ValueError):
        oracle.S_update(Y, S, T, {"lamb_spat_TV": 0.1})


# ---------------------------------------------------------------- GPU ------
T_CASES = [
    {},
    {"lamb_temp": 0.02, "pointwise": True},
    {"active": "half", "use_std": True},
    {"lamb_corr": 0.05, "lamb_temp": 0.01},
    {"lamb_temp_TV": 0.05},
    {"lamb_corr": 0.02, "lamb_temp_TV": 0.01, "pointwise": True, "use_std": True},
]


def _t_opts(opts, Y, P):
    o = dict(opts)
    if o.get("active") == "half":
        o["active"] = (np.arange(P) % 3) != 0
    if o.get("use_std"):
        o["Y"] = np.asarray(Y, np.float64).sum(axis=1).astype(np.float32)
    return o


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(T_CASES)))
@pytest.mark.parametrize("prec", ["fp32", "split"])
def test_t_update_gpu_matches_oracle(gpu, oracle, case, prec):
    import sid_gb300 as s
    Y, S, T = nmf_problem(10 + case)
    P = Y.shape[0]
    o = _t_opts(T_CASES[case], Y, P)
    S_ref, T_ref = oracle.T_update(Y, T, S, o)
    S_g, T_g = s.Context().t_update(Y, T, S, o, prec=prec)
    tol = 1e-5
    assert rel_l2(s.to_numpy(T_g), T_ref) < tol
    assert rel_l2(s.to_numpy(S_g), S_ref) < 1e-6


@pytest.mark.gpu
def test_t_update_gpu_half_movie(gpu, oracle):
    import sid_gb300 as s
    Y, S, T = nmf_problem(20, f16=True)
    S_ref, T_ref = oracle.T_update(Y.astype(np.float32), T, S, {"lamb_temp": 0.01})
    _, T_g = s.T_update(Y, T, S, {"lamb_temp": 0.01})
    assert rel_l2(s.to_numpy(T_g), T_ref) < 1e-5


S_CASES = [
    {},
    {"lamb_spat": 0.01, "pointwise": True},
    {"use_std": True},
    {"lamb_orth_L1": 0.02},
    {"lamb_orth_L2": 0.02},
    {"lamb_orth_L1": 0.01, "lamb_orth_L2": 0.01, "pointwise": True},
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(S_CASES)))
def test_s_update_gpu_matches_oracle(gpu, oracle, case):
    import sid_gb300 as s
    Y, S, T = nmf_problem(30 + case, P=1500, R=8, F=120)
    P, R = S.shape
    o = dict(S_CASES[case])
    if o.get("use_std"):
        o["Y"] = np.asarray(Y, np.float64).sum(axis=1).astype(np.float32)
    if o.get("lamb_orth_L1") or o.get("lamb_orth_L2"):
        o["hilf"] = hilf_matrix(R)
    S_ref, T_ref = oracle.S_update(Y, S, T, o)
    S_g, T_g = s.S_update(Y, S, T, o)
    # use_std (S_update.m:11-15) centres both products by the frame means: the
    # centred gradient is small against q_S = Y T' and S Q_T, whose tensor-core
    # accumulation (FP32 adds that truncate) leaves ~1e-5 of it
    tol = 2e-5 if o.get("use_std") else 1e-5
    assert rel_l2(s.to_numpy(S_g), S_ref) < tol
    assert rel_l2(s.to_numpy(T_g), T_ref) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "split", "bf16"])
@pytest.mark.parametrize("f16", [False, True])
def test_s_update_gpu_precisions(gpu, oracle, prec, f16):
    """The pixel-by-rank products (Y T', S Q_T, v Q_T) run on the tensor cores
    for the split and BF16 precisions (FP16 movies unsplit, FP32 factors as
    BF16 hi/lo) and on the FP32 SIMT GEMM for fp32; P and R off the tile
    sizes."""
    import sid_gb300 as s
    Y, S, T = nmf_problem(60 + int(f16), P=2345, R=70, F=133, f16=f16)
    o = {"lamb_spat": 0.01, "lamb_orth_L2": 0.01, "hilf": hilf_matrix(70)}
    S_ref, T_ref = oracle.S_update(Y.astype(np.float32), S, T, o)
    S_g, T_g = s.Context().s_update(Y, S, T, o, prec=prec)
    tol = 3e-3 if prec == "bf16" else 1e-5
    assert rel_l2(s.to_numpy(S_g), S_ref) < tol
    assert rel_l2(s.to_numpy(T_g), T_ref) < tol


@pytest.mark.gpu
def test_nmf_gpu_alternating_descends(gpu):
    """Alternating S and T steps (fast_NMF.m:185-186) lower the residual."""
    import sid_gb300 as s
    Y, S, T = nmf_problem(40, P=3000, R=12, F=200)
    ctx = s.Context()
    f = [objective(Y, S.astype(np.float64), T.astype(np.float64))]
    Sg, Tg = s.to_device(S), s.to_device(T)
    for _ in range(5):
        Sg, Tg = ctx.s_update(Y, Sg, Tg, {})
        Sg, Tg = ctx.t_update(Y, Tg, Sg, {})
        f.append(objective(Y, s.to_numpy(Sg).astype(np.float64), s.to_numpy(Tg).astype(np.float64)))
    assert all(b <= a * (1 + 1e-6) for a, b in zip(f, f[1:]))
    assert f[-1] < 0.5 * f[0]


@pytest.mark.gpu
def test_s_update_gpu_rejects_spatial_tv(gpu):
    import sid_gb300 as s
    Y, S, T = nmf_problem(50, P=100, R=3, F=10)
    with pytest.raises(s.SidError):
        s.S_update(Y, S, T, {"lamb_spat_TV": 0.1})
