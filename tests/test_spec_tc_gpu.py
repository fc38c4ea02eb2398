"""Batched projections on the tensor cores (plan flag SID_PLAN_SPECTRAL_TC;
reconstruct_S.m:162-212 reconstructs components side by side): forward and
back projections of many volumes per pass over the 24-bit tap spectra, and
ISRA (deconvRL, mode 'basic') over several components, against the FP64
oracle.  The geometries put more than one 128-row tile on both the forward
(225 output phases) and the back projection, and more than one 1024-element
accumulation chunk on the forward reduction."""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _geom(N, Z, M, L, sig=(1.0, 3.0)):
    from sid_gb300 import Projector, synthetic
    X = N * L
    H = synthetic.gaussian_psf(M, N, Z, sigma_min=sig[0], sigma_max=sig[1])
    P = Projector(H, (X, X), None, methods=("spectral_mixed",), batched=True)
    return H, P, X, Z


@pytest.fixture(scope="module")
def small(gpu):
    return _geom(5, 3, 31, 9)


@pytest.fixture(scope="module")
def wide(gpu):
    # 225 output phases (two row tiles forward), 675 channels (six row tiles back,
    # a 1360-element forward reduction: two accumulation chunks)
    return _geom(15, 3, 45, 7, sig=(1.5, 4.0))


def _volumes(X, Z, n, seed):
    from sid_gb300 import synthetic
    return [synthetic.blob_volume(X, X, Z, 6, sigma=(1.5, 1.5), seed=seed + k) for k in range(n)]


@pytest.mark.parametrize("which", ["small", "wide"])
@pytest.mark.parametrize("nb", [2, 7, 33])
def test_tc_projections_match_oracle(request, oracle, which, nb):
    import sid_gb300 as s
    H, P, X, Z = request.getfixturevalue(which)
    vols = _volumes(X, Z, nb, 300)
    outs = P.forward_batched(vols, method="spectral_mixed")
    worst = 0.0
    for v, o in zip(vols, outs):
        worst = max(worst, rel_l2(s.to_numpy(o), oracle.forward_project(H, v)))
    assert worst < 2e-5, worst
    ims = [oracle.forward_project(H, v).astype(np.float32) for v in vols]
    backs = P.adjoint_batched(ims, method="spectral_mixed")
    worst = 0.0
    for i, b in zip(ims, backs):
        worst = max(worst, rel_l2(s.to_numpy(b), oracle.backward_project(H, i)))
    assert worst < 2e-5, worst
    P.sync()


def test_tc_volumes_are_independent(small):
    """Each volume's result does not depend on the others in its pass (a zero
    volume among non-zero ones projects to zero; order does not matter)."""
    import sid_gb300 as s
    H, P, X, Z = small
    vols = _volumes(X, Z, 5, 400)
    vols[2] = np.zeros_like(vols[2])
    a = P.forward_batched(vols, method="spectral_mixed")
    b = P.forward_batched(vols[::-1], method="spectral_mixed")
    assert float(np.abs(s.to_numpy(a[2])).max()) == 0.0
    for k in range(5):
        assert rel_l2(s.to_numpy(a[k]), s.to_numpy(b[4 - k])) < 1e-6 or k == 2


@pytest.mark.parametrize("which,nb", [("small", 7), ("small", 30), ("wide", 9)])
def test_tc_isra_matches_oracle(request, oracle, which, nb):
    import sid_gb300 as s
    H, P, X, Z = request.getfixturevalue(which)
    vols = _volumes(X, Z, nb, 500)
    fwd = lambda v: oracle.forward_project(H, v)  # noqa: E731
    bwd = lambda i: oracle.backward_project(H, i)  # noqa: E731
    htfs = [bwd(fwd(v)).astype(np.float32) for v in vols]
    outs = P.isra_batched(htfs, htfs, 8, method="spectral_mixed")
    worst = 0.0
    for h, o in zip(htfs, outs):
        ref = oracle.deconvRL(fwd, bwd, h, 8, h)
        worst = max(worst, rel_l2(s.to_numpy(o), ref))
    # the mixed form's bar for 8 ISRA iterations (test_deconv_gpu.py)
    assert worst < 1e-4, worst


def test_tc_plan_needs_f24(gpu):
    import ctypes
    from sid_gb300 import _lib, synthetic
    H = synthetic.gaussian_psf(31, 5, 3)
    plan = ctypes.c_void_p()
    rc = _lib.load().sid_plan_create(H.ctypes.data, 31, 5, 3, None, 45, 45,
                                     _lib.PLAN_SPECTRAL_I16 | _lib.PLAN_SPECTRAL_TC, ctypes.byref(plan))
    assert rc == _lib.SID_EINVAL
