"""Whole-movie scans of SID's preprocessing, mirroring the reference's MATLAB
functions:

* ``[bg_spatial, bg_temporal] = rank_1_factorization(Y, maxIter)``
  rank_1_factorization.m:1 (called as sid_main.m:95 with maxIter = bg_iter)
* ``std_image = compute_std_image(Y, y_1, y_2)``   compute_std_image.m:1
  (sid_main.m:101)

Y is the P x F movie (single or half, column-major: a frame per column).
Results are CUDA tensors: bg_spatial (P,), bg_temporal (F,), std_image (P,).
All arithmetic runs in libsid (``sid_rank1_background`` / ``sid_std_image``).
"""
from __future__ import annotations

import torch

from . import _lib
from .lfm import _stream_ptr, to_device
from .nnls import Context, _ctx, _movie


def _rank1(self, Y, maxIter=1, std_image=False):
    """rank_1_factorization on the GPU; with std_image=True also the
    standard-deviation image of Y - bg_spatial*bg_temporal, computed in the same
    pass over Y as the last spatial update."""
    Yd, half = _movie(Y)
    P, F = Yd.shape
    s = torch.empty(P, device=Yd.device, dtype=torch.float32)
    t = torch.empty(F, device=Yd.device, dtype=torch.float32)
    sd = torch.empty(P, device=Yd.device, dtype=torch.float32) if std_image else None
    _lib.call("sid_rank1_background", self._ctx, Yd.data_ptr(), _lib.DTYPE_F16 if half else _lib.DTYPE_F32, P, F,
              int(maxIter), s.data_ptr(), t.data_ptr(), sd.data_ptr() if sd is not None else None, _stream_ptr())
    return (s, t, sd) if std_image else (s, t)


def _std(self, Y, y_1=None, y_2=None):
    """compute_std_image on the GPU (y_1, y_2 default to zeros)."""
    Yd, half = _movie(Y)
    P, F = Yd.shape
    y1 = to_device(y_1).reshape(-1).contiguous() if y_1 is not None else None
    y2 = to_device(y_2).reshape(-1).contiguous() if y_2 is not None else None
    out = torch.empty(P, device=Yd.device, dtype=torch.float32)
    _lib.call("sid_std_image", self._ctx, Yd.data_ptr(), _lib.DTYPE_F16 if half else _lib.DTYPE_F32, P, F,
              y1.data_ptr() if y1 is not None else None, y2.data_ptr() if y2 is not None else None,
              out.data_ptr(), _stream_ptr())
    return out


Context.rank_1_factorization = _rank1
Context.std_image = _std


def rank_1_factorization(Y, maxIter=1):
    """[bg_spatial, bg_temporal] = rank_1_factorization(Y, maxIter) (rank_1_factorization.m:1)."""
    return _ctx().rank_1_factorization(Y, maxIter)


def compute_std_image(Y, y_1=None, y_2=None):
    """std_image = compute_std_image(Y, y_1, y_2) (compute_std_image.m:1)."""
    return _ctx().std_image(Y, y_1, y_2)
