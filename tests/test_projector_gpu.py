"""Parity of the CUDA projector (direct FP32, spectral FP32 / FP16) with the
FP64 oracle and the golden fixtures, plus the adjoint dot-product test."""
import os

import numpy as np
import pytest

from tests.conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu

# rel-L2 bars against FP64: plain FP32 path 1e-5, mixed (FP16 spectra) 1e-4
TOL = {"direct": 1e-5, "spectral_f32": 1e-5, "spectral_i16": 1e-4, "spectral_mixed": 1e-4, "spectral_mixed_f32": 1e-4}
ALL = ("direct", "spectral_f32", "spectral_i16", "spectral_mixed", "spectral_mixed_f32")


def _golden(case):
    d = np.load(os.path.join(ROOT, "tests/golden/projector_cases.npz"))
    return {k.split("/")[1]: d[k] for k in d.files if k.startswith(case + "/")}


@pytest.mark.parametrize("case", ["small_full", "ragged", "nnum5"])
def test_golden_all_methods(gpu, case):
    from sid_gb300 import Projector, to_numpy
    g = _golden(case)
    X, Y = g["I"].shape
    P = Projector(g["H"], (X, Y), None, methods=ALL)
    for m in ALL:
        f = to_numpy(P.forward(g["V"], method=m))
        b = to_numpy(P.adjoint(g["I"], method=m))
        assert rel_l2(f, g["fwd"]) < TOL[m], (m, rel_l2(f, g["fwd"]))
        assert rel_l2(b, g["adj"]) < TOL[m], (m, rel_l2(b, g["adj"]))
    P.sync()


def test_golden_cropped_direct(gpu):
    from sid_gb300 import Projector, to_numpy
    g = _golden("cropped")
    X, Y = g["I"].shape
    P = Projector(g["H"], (X, Y), g["CAindex"], methods=("direct",))
    assert rel_l2(to_numpy(P.forward(g["V"])), g["fwd"]) < 1e-5
    assert rel_l2(to_numpy(P.adjoint(g["I"])), g["adj"]) < 1e-5


def test_even_width_follows_reference_centring(gpu, oracle):
    """Even PSF widths: forward uses floor(M/2), back projection the imrotate
    centre; the GPU must match the oracle (not the true adjoint)."""
    from sid_gb300 import Projector, to_numpy
    rng = np.random.default_rng(7)
    M, N, Z, X, Y = 10, 3, 2, 15, 12
    H = rng.random((M, M, N, N, Z)).astype(np.float32)
    V = rng.random((X, Y, Z)).astype(np.float32)
    I = rng.random((X, Y)).astype(np.float32)
    P = Projector(H, (X, Y), None, methods=("direct",))
    assert P.info()["adj_separate"] == 1
    assert rel_l2(to_numpy(P.forward(V)), oracle.forward_project(H, V)) < 1e-5
    assert rel_l2(to_numpy(P.adjoint(I)), oracle.backward_project(H, I)) < 1e-5
    with pytest.raises(Exception):
        Projector(H, (X, Y), None, methods=("spectral_f32",))


@pytest.fixture(scope="module")
def frame225(gpu):
    from sid_gb300 import Projector, synthetic
    H, V = synthetic.config_inputs("225x225x11")
    P = Projector(H, V.shape[:2], None, methods=ALL)
    return H, V, P


@pytest.mark.parametrize("method", ALL)
def test_frame225_forward_adjoint_vs_oracle(frame225, oracle, method):
    """Full 225 x 225 x 11 geometry (Nnum 15, 225 x 225 x 11, PSF 195): specialised D=15 kernels."""
    from sid_gb300 import to_numpy
    H, V, P = frame225
    ref_f = oracle.forward_project(H, V)
    f = to_numpy(P.forward(V, method=method))
    assert rel_l2(f, ref_f) < TOL[method], rel_l2(f, ref_f)
    I = (ref_f / ref_f.max()).astype(np.float32)
    ref_b = oracle.backward_project(H, I)
    b = to_numpy(P.adjoint(I, method=method))
    assert rel_l2(b, ref_b) < TOL[method], rel_l2(b, ref_b)


@pytest.mark.parametrize("method", ALL)
def test_dot_product_adjoint(frame225, method):
    """<A x, y> == <x, A^T y> on random pairs, in FP32 on the GPU."""
    import torch
    from sid_gb300.lfm import _fortran_tensor
    H, V, P = frame225
    g = torch.Generator(device="cuda").manual_seed(11)
    for _ in range(4):
        x = _fortran_tensor((P.X, P.Y, P.Z), "cuda")
        x.copy_(torch.rand(x.shape, generator=g, device="cuda"))
        y = _fortran_tensor((P.X, P.Y), "cuda")
        y.copy_(torch.rand(y.shape, generator=g, device="cuda"))
        lhs = torch.sum(P.forward(x, method=method).double() * y.double()).item()
        rhs = torch.sum(x.double() * P.adjoint(y, method=method).double()).item()
        # the mixed form pairs a 16-bit forward with an FP32 back projection, so
        # it is an adjoint pair only to the 16-bit precision
        assert abs(lhs - rhs) / abs(lhs) < (1e-5 if method in ("direct", "spectral_f32") else 1e-4)


def test_host_entry_points_match_device(frame225):
    from sid_gb300 import to_numpy
    H, V, P = frame225
    f_dev = to_numpy(P.forward(V))
    f_host = P.forward_host(V)
    np.testing.assert_array_equal(f_dev, f_host)
    b_host = P.adjoint_host(f_host)
    np.testing.assert_array_equal(to_numpy(P.adjoint(f_dev)), b_host)
    # page-locked host arrays take the same path through their device addresses
    import torch
    vp = torch.empty(V.size, dtype=torch.float32, pin_memory=True).numpy().reshape(V.shape, order="F")
    vp[...] = V
    np.testing.assert_array_equal(P.forward_host(vp), f_dev)


def test_function_api(gpu, oracle):
    import sid_gb300 as s
    g = _golden("small_full")
    f = s.to_numpy(s.forwardProjectGPU(g["H"], g["V"]))
    b = s.to_numpy(s.backwardProjectGPU_new(g["H"], g["I"]))
    assert rel_l2(f, g["fwd"]) < 1e-5 and rel_l2(b, g["adj"]) < 1e-5
    f2 = s.to_numpy(s.forwardProjectACC(g["H"], g["V"], g["CAindex"]))
    assert rel_l2(f2, g["fwd"]) < 1e-5
