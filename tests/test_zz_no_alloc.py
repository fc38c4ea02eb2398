"""The allocation-free Gram entry point (sid_gram_noalloc).

Callers whose device memory is owned by another allocator (MATLAB's gpuArray
memory manager behind a MEX function, or a program that reserves the GPU's
memory up front) cannot let the library call cudaMalloc.  This file is named
to be collected last: the entry point shares one fixed device array between
calls, and its test must pass both alone and after every other test.
"""
import ctypes

import numpy as np
import pytest

from tests.conftest import rel_l2


def test_noalloc_rejects_oversize_before_gpu_work(sidlib):
    """K beyond the fixed scratch limit is refused with SID_EINVAL (host check)."""
    from sid_gb300 import _lib
    dummy = ctypes.c_void_p(16)
    rc = sidlib.sid_gram_noalloc(dummy, 10, 4096, dummy, None)
    assert rc == _lib.SID_EINVAL
    assert b"2048" in sidlib.sid_last_error()


@pytest.mark.gpu
def test_noalloc_gram_matches_context_gram_twice(gpu):
    import torch

    from sid_gb300 import Context, _lib, to_device
    from sid_gb300.lfm import _fortran_tensor, _stream_ptr
    lib = _lib.load()
    ctx = Context()
    rng = np.random.default_rng(21)
    for call, (P, K) in enumerate([(20000, 300), (9001, 777)]):
        A = to_device(np.asfortranarray(rng.random((P, K), dtype=np.float32)))
        ref = ctx.gram(A, prec="fp32")
        G = _fortran_tensor((K, K), A.device)
        G.fill_(float("nan"))
        rc = lib.sid_gram_noalloc(ctypes.c_void_p(A.data_ptr()), P, K, ctypes.c_void_p(G.data_ptr()), _stream_ptr())
        assert rc == 0, lib.sid_last_error()
        torch.cuda.synchronize()
        # FP32 tolerance of the contraction tests (1e-5), against the context path
        # and against FP64
        assert rel_l2(G.cpu().numpy(), ref.cpu().numpy()) < 1e-5, call
        A64 = A.double().cpu().numpy()
        assert rel_l2(G.cpu().numpy(), A64.T @ A64) < 1e-5, call
