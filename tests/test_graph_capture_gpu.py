"""T_update / S_update (T_update.m, S_update.m) keep their operand scales and
step sizes on the device, so an alternation of the two steps -- the inner loop
of the factorisation (fast_NMF.m:185-186) -- can be captured once in a CUDA
graph and replayed; so can batched ISRA iterations on the tensor-core
projections.  The replays must give what the same calls give eagerly."""
import ctypes

import numpy as np
import pytest

from tests.conftest import rel_l2
from tests.test_nmf import hilf_matrix, nmf_problem

pytestmark = pytest.mark.gpu


def _raw_steps(ctx, Yd, half, S, T, opts_t, opts_s, hilf, prec):
    """The libsid calls of one T_update + S_update alternation on fixed buffers
    (what the Python mirrors do after their argument checks and copies)."""
    import torch
    from sid_gb300 import _lib
    from sid_gb300.nmf import _nmf_opts
    P, R = S.shape
    F = T.shape[1]
    ot, os_ = _nmf_opts(opts_t), _nmf_opts(opts_s)
    dt = _lib.DTYPE_F16 if half else _lib.DTYPE_F32

    def run():
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.call("sid_t_update", ctx._ctx, Yd.data_ptr(), dt, T.data_ptr(), S.data_ptr(), P, R, F, None, None,
                  ctypes.byref(ot), _lib.PREC[prec], st)
        _lib.call("sid_s_update", ctx._ctx, Yd.data_ptr(), dt, S.data_ptr(), T.data_ptr(), P, R, F, None,
                  hilf.data_ptr() if hilf is not None else None, ctypes.byref(os_), _lib.PREC[prec], st)
    return run


def _capture(step):
    import torch
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            step()
    torch.cuda.synchronize()
    return g


@pytest.mark.parametrize("f16", [False, True])
@pytest.mark.parametrize("orth", [False, True])
def test_alternation_replays_in_a_cuda_graph(gpu, f16, orth):
    import torch
    import sid_gb300 as s
    from sid_gb300.nnls import _movie
    Y, S0, T0 = nmf_problem(31, P=6000, R=12, F=200, f16=f16)
    opts_t = {"lamb_temp": 0.01}
    opts_s = {"lamb_spat": 0.01}
    hilf = None
    if orth:
        opts_s.update(lamb_orth_L1=0.05, lamb_orth_L2=0.02)
        hilf = s.to_device(hilf_matrix(12))
    ctx = s.Context()
    Yd, half = _movie(Y)
    # eager: three alternations on their own buffers
    Se, Te = s.to_device(S0).clone(), s.to_device(T0).clone()
    eager = _raw_steps(ctx, Yd, half, Se, Te, opts_t, opts_s, hilf, "split")
    snaps = []
    for _ in range(3):
        eager()
        torch.cuda.synchronize()
        snaps.append((Se.clone(), Te.clone()))
    # the same alternation captured once (workspaces already sized by the eager calls)
    Sg, Tg = s.to_device(S0).clone(), s.to_device(T0).clone()
    g = _capture(_raw_steps(ctx, Yd, half, Sg, Tg, opts_t, opts_s, hilf, "split"))
    # capture records without running: the buffers still hold the start point
    assert torch.equal(Sg, s.to_device(S0)) and torch.equal(Tg, s.to_device(T0))
    for k in range(3):
        g.replay()
        torch.cuda.synchronize()
        Sref, Tref = snaps[k]
        assert rel_l2(s.to_numpy(Sg), s.to_numpy(Sref)) < 1e-6, k
        assert rel_l2(s.to_numpy(Tg), s.to_numpy(Tref)) < 1e-6, k
    assert np.all(np.isfinite(s.to_numpy(Sg)))
    ctx.sync()


def test_replayed_steps_follow_the_oracle(gpu, oracle):
    """One eager and two replayed alternations against three oracle alternations."""
    import torch
    import sid_gb300 as s
    from sid_gb300.nnls import _movie
    Y, S0, T0 = nmf_problem(32, P=3000, R=8, F=120)
    opts_t, opts_s = {"lamb_temp": 0.02}, {"lamb_spat": 0.02}
    ctx = s.Context()
    Yd, half = _movie(Y)
    Sg, Tg = s.to_device(S0).clone(), s.to_device(T0).clone()
    step = _raw_steps(ctx, Yd, half, Sg, Tg, opts_t, opts_s, None, "split")
    step()  # sizes the workspaces (and takes the first alternation eagerly)
    torch.cuda.synchronize()
    g = _capture(step)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    S, T = np.asarray(S0, np.float64), np.asarray(T0, np.float64)
    Y64 = np.asarray(Y, np.float64)
    for _ in range(3):
        S, T = oracle.T_update(Y64, T, S, dict(opts_t))
        S, T = oracle.S_update(Y64, S, T, dict(opts_s))
    assert rel_l2(s.to_numpy(Sg), S) < 1e-4
    assert rel_l2(s.to_numpy(Tg), T) < 1e-4


def test_batched_isra_replays_in_a_cuda_graph(gpu):
    """ISRA over several components on the tensor-core batched projections
    (deconvRL, reconstruct_S.m:162-212) makes no host round trip either: two
    iterations for 6 volumes captured once and replayed equal the eager calls."""
    import torch
    import sid_gb300 as s
    from sid_gb300 import Projector, _lib, synthetic
    N, Z, M, L = 5, 3, 31, 9
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=1.0, sigma_max=3.0)
    P = Projector(H, (X, X), None, methods=("spectral_mixed",), batched=True)
    vols = [synthetic.blob_volume(X, X, Z, 6, sigma=(1.5, 1.5), seed=70 + k) for k in range(6)]
    htfs = [P.adjoint(P.forward(v)).clone() for v in vols]
    method = _lib.METHODS["spectral_mixed"]

    def run(xs):
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.call("sid_deconv_isra_batched", P._plan, method, len(xs),
                  ctypes.cast(P._ptr_array(htfs), ctypes.c_void_p), ctypes.cast(P._ptr_array(xs), ctypes.c_void_p),
                  2, 0.0, st)

    xe = [h.clone() for h in htfs]
    run(xe)
    torch.cuda.synchronize()
    run(xe)  # four iterations eagerly
    torch.cuda.synchronize()
    xg = [h.clone() for h in htfs]
    g = _capture(lambda: run(xg))
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip(xg, xe):
        assert rel_l2(s.to_numpy(a), s.to_numpy(b)) < 1e-6
    P.close()
