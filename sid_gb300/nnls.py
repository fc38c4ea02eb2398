"""NNLS contractions and solvers, mirroring the reference's MATLAB API.

Reference functions mirrored here:

* ``[X, G] = LS_nnls(A, Y, opts, G, x)``             LS_nnls.m:1
* ``[xx, Q, df, h] = fast_nnls(A, Y, opts, Q, df, h)`` fast_nnls.m:1
* the Gram ``A'*A`` and cross ``A'*Y`` products they start from
  (LS_nnls.m:76,82; fast_nnls.m:54-57).

Matrices are MATLAB column-major: NumPy Fortran-order arrays or CUDA tensors
with column-major strides (see ``sid_gb300.lfm``).  All arithmetic runs in
libsid (tcgen05 tensor-core or FP32 SIMT contractions, CUDA solver kernels).
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np
import torch

from . import _lib
from .lfm import _fortran_tensor, _stream_ptr, to_device


def _to_device_half(a):
    if isinstance(a, torch.Tensor):
        t = a.to(device="cuda", dtype=torch.float16)
        return t.permute(*reversed(range(t.dim()))).contiguous().permute(*reversed(range(t.dim())))
    arr = np.asfortranarray(np.asarray(a, dtype=np.float16))
    t = torch.from_numpy(np.ascontiguousarray(arr.T)).to("cuda")
    return t.permute(*reversed(range(t.dim())))


class Context:
    """Workspace owner for the contractions and NNLS solvers (a ``sid_ctx``)."""

    def __init__(self):
        if not torch.cuda.is_available():
            raise RuntimeError("sid_gb300 needs a CUDA GPU: the NNLS path has no CPU implementation")
        torch.cuda.current_device()
        h = ctypes.c_void_p()
        _lib.call("sid_ctx_create", ctypes.byref(h))
        self._ctx = h
        self._fin = weakref.finalize(self, _lib.load().sid_ctx_destroy, h)

    def sync(self):
        _lib.call("sid_ctx_sync", self._ctx, _stream_ptr())

    def gram(self, A, prec="split") -> torch.Tensor:
        """G = A'*A for A (P x K)."""
        A = to_device(A)
        P, K = A.shape
        G = _fortran_tensor((K, K), A.device)
        _lib.call("sid_gram", self._ctx, A.data_ptr(), P, K, G.data_ptr(), _lib.PREC[prec], _stream_ptr())
        return G

    def cross(self, A, Y, prec="split") -> torch.Tensor:
        """h = A'*Y for A (P x K) and Y (P x F), Y single or half."""
        A = to_device(A)
        half = (isinstance(Y, torch.Tensor) and Y.dtype == torch.float16) or \
               (isinstance(Y, np.ndarray) and Y.dtype == np.float16)
        Yd = _to_device_half(Y) if half else to_device(Y)
        P, K = A.shape
        F = Yd.shape[1]
        h = _fortran_tensor((K, F), A.device)
        _lib.call("sid_cross", self._ctx, A.data_ptr(), Yd.data_ptr(), _lib.DTYPE_F16 if half else _lib.DTYPE_F32,
                  P, K, F, h.data_ptr(), _lib.PREC[prec], _stream_ptr())
        return h
