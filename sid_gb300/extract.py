"""Timeseries extraction with the forward model's pseudo-inverse, mirroring
``incremental_temporal_update_gpu`` (incremental_temporal_update_gpu.m:1).

The reference reads TIFF frames from a directory, rectifies them
(ImageRect.m) and processes them in chunks of ``Junk_size``: with
``opts.non_neg_on`` each chunk is solved by LS_nnls, otherwise
``Q = inv(F*F')*F`` is formed once (:83-84) and every chunk is ``Q * Y``
(:89, 99), with frames divided by their baseline (:66-68).  Here the frames
are given as a P x N array (already rectified); the chunk loop, the baseline
division and both branches run in libsid (``sid_pinv_*``, ``sid_ls_nnls``).
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np
import torch

from . import _lib
from .lfm import _fortran_tensor, _stream_ptr, to_device
from .nnls import _ctx, _movie


class Extractor:
    """Q = inv(F*F')*F for a forward model F (K x P, or P x K with
    ``pixel_major=True``), applied chunk by chunk."""

    def __init__(self, forward_model, pixel_major=False, prec="split", ctx=None):
        self._ctx = ctx or _ctx()
        F = to_device(forward_model)
        if pixel_major:
            P, K = F.shape
        else:
            K, P = F.shape
        self.K, self.P = K, P
        h = ctypes.c_void_p()
        _lib.call("sid_pinv_create", self._ctx._ctx, F.data_ptr(), K, P, 1 if pixel_major else 0, _lib.PREC[prec],
                  ctypes.byref(h), _stream_ptr())
        self._h = h
        self._fin = weakref.finalize(self, _lib.load().sid_pinv_destroy, h)

    def apply(self, Y, baseline=None, out=None, col0=0):
        """T = Q * (Y ./ baseline) for Y (P x n, single or half); written into
        columns col0.. of ``out`` (K x N) when given."""
        Yd, half = _movie(Y)
        if Yd.shape[0] != self.P:
            raise ValueError(f"frames must have {self.P} pixels, got {Yd.shape[0]}")
        n = Yd.shape[1]
        b = None
        if baseline is not None:
            b = torch.as_tensor(np.asarray(baseline, dtype=np.float32).reshape(-1), device="cuda")
            if b.numel() != n:
                raise ValueError(f"baseline must have {n} entries")
        if out is None:
            out = _fortran_tensor((self.K, n), Yd.device)
            col0 = 0
        dst = out.data_ptr() + 4 * self.K * col0
        _lib.call("sid_pinv_apply", self._h, Yd.data_ptr(), _lib.DTYPE_F16 if half else _lib.DTYPE_F32, n,
                  b.data_ptr() if b is not None else None, dst, out.stride(1), _stream_ptr())
        return out

    def close(self):
        self._fin()


def incremental_temporal_update_gpu(forward_model, frames, bg_spatial=None, Junk_size=200, opts=None):
    """timeseries = incremental_temporal_update_gpu(forward_model, frames, [], Junk_size, opts)

    forward_model: K x P; frames: P x N (rectified, cropped); opts fields read:
    ``non_neg_on`` (LS_nnls per chunk instead of the pseudo-inverse),
    ``baseline`` (N per-frame divisors), ``idx`` (pixel subset of the frames,
    MATLAB 1-based indices or a logical mask) and the LS_nnls options.
    Returns the K x N timeseries (CUDA tensor)."""
    opts = dict(opts or {})
    if bg_spatial is not None and np.size(bg_spatial):
        # the reference allocates K+1 rows for a background but assigns K rows
        # per chunk (incremental_temporal_update_gpu.m:47,89), which MATLAB rejects
        raise ValueError("incremental_temporal_update_gpu: bg_spatial must be empty")
    Yall = frames
    idx = opts.get("idx")
    if idx is not None:
        sel = np.asarray(idx)
        sel = np.flatnonzero(sel) if sel.dtype == bool else sel.astype(np.int64) - 1
        Yall = Yall[sel, :] if isinstance(Yall, np.ndarray) else Yall[torch.as_tensor(sel, device=Yall.device), :]
    N = Yall.shape[1]
    base = np.asarray(opts.get("baseline"), dtype=np.float32).reshape(-1) if opts.get("baseline") is not None \
        else None
    if base is not None and base.size != N:
        raise ValueError(f"opts.baseline must have {N} entries")
    step = max(1, int(Junk_size))
    ctx = _ctx()
    K = forward_model.shape[0]
    out = _fortran_tensor((K, N), "cuda")
    if opts.get("non_neg_on"):
        # LS_nnls on every chunk, the Gram of the first chunk reused by the
        # others (the reference's intent at :78,94, whose output list does not
        # match LS_nnls's)
        A = _fortran_tensor((forward_model.shape[1], K), "cuda")
        A.copy_(to_device(forward_model).T)
        nn_opts = {k: v for k, v in opts.items() if k in ("lambda", "sample", "tol", "tol_", "max_iter", "use_std")}
        G = None
        for c0 in range(0, N, step):
            c1 = min(N, c0 + step)
            Yc = Yall[:, c0:c1]
            if base is not None:
                Yc = to_device(Yc) / torch.as_tensor(base[c0:c1], device="cuda")[None, :]
            X, G = ctx.ls_nnls(A, Yc, nn_opts, G=G)
            out[:, c0:c1] = X
        return out
    ex = Extractor(forward_model, ctx=ctx)
    try:
        for c0 in range(0, N, step):
            c1 = min(N, c0 + step)
            ex.apply(Yall[:, c0:c1], base[c0:c1] if base is not None else None, out=out, col0=c0)
    finally:
        ex.close()
    return out
