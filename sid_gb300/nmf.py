"""Projected-gradient steps of the SID factorisation Y ~ S*T, mirroring the
reference's MATLAB functions:

* ``[S, T] = T_update(Y, T, S, opts)``   T_update.m:1
* ``[S, T] = S_update(Y, S, T, opts)``   S_update.m:1

Y is the P x F movie (single or half), S the P x R spatial components and T
the R x F timeseries, MATLAB column-major (Fortran-order arrays or CUDA tensors
with column-major strides).  The inputs are not modified: like the MATLAB
functions, each call returns new S and T (CUDA tensors).  All arithmetic runs
in libsid (``sid_t_update`` / ``sid_s_update``).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .lfm import _stream_ptr, to_device
from .nnls import Context, _ctx, _movie


class NmfOpts(ctypes.Structure):
    """sid_nmf_opts: the reference's opts fields read by T_update / S_update."""
    _fields_ = [("lamb_temp", ctypes.c_double), ("lamb_corr", ctypes.c_double), ("lamb_temp_TV", ctypes.c_double),
                ("lamb_spat", ctypes.c_double), ("lamb_spat_TV", ctypes.c_double),
                ("lamb_orth_L1", ctypes.c_double), ("lamb_orth_L2", ctypes.c_double), ("use_std", ctypes.c_int),
                ("pointwise", ctypes.c_int)]


_FLOAT_FIELDS = ("lamb_temp", "lamb_corr", "lamb_temp_TV", "lamb_spat", "lamb_spat_TV", "lamb_orth_L1",
                 "lamb_orth_L2")
# fields the reference's opts carries for other functions or for its diagnostic plots
_IGNORED = ("active", "Y", "hilf", "diagnostic", "rank", "size", "T", "gpu", "gpu_id", "display")


def _nmf_opts(opts: dict) -> NmfOpts:
    o = NmfOpts()
    _lib.load().sid_nmf_defaults(ctypes.byref(o))
    for k, v in opts.items():
        if k in _FLOAT_FIELDS:
            setattr(o, k, float(v))
        elif k in ("use_std", "pointwise"):
            setattr(o, k, int(bool(v)))
        elif k not in _IGNORED:
            raise ValueError(f"unknown NMF option {k!r}")
    return o


def _vector(v, n, what):
    t = to_device(np.asarray(v, dtype=np.float32).reshape(-1) if not isinstance(v, torch.Tensor) else v.reshape(-1))
    if t.numel() != n:
        raise ValueError(f"{what} must have {n} elements, got {t.numel()}")
    return t.contiguous()


def _active_mask(active, P):
    a = active.detach().cpu().numpy() if isinstance(active, torch.Tensor) else np.asarray(active)
    a = a.reshape(-1)
    if a.dtype == bool or (a.size == P and set(np.unique(a)).issubset({0, 1})):
        mask = a.astype(bool)
        if mask.size != P:
            raise ValueError(f"opts.active must have {P} entries")
    else:  # MATLAB linear indices (1-based)
        mask = np.zeros(P, dtype=bool)
        mask[a.astype(np.int64) - 1] = True
    return torch.from_numpy(mask.astype(np.uint8)).to("cuda")


def _t_update(self, Y, T, S, opts=None, prec="split"):
    """[S, T] = T_update(Y, T, S, opts) (T_update.m:1) on the GPU."""
    opts = dict(opts or {})
    Yd, half = _movie(Y)
    T = to_device(T).clone()
    S = to_device(S).clone()
    P, R = S.shape
    F = T.shape[1]
    if T.shape[0] != R or Yd.shape != (P, F):
        raise ValueError(f"shapes: Y {tuple(Yd.shape)}, T {tuple(T.shape)}, S {tuple(S.shape)}")
    act = _active_mask(opts["active"], P) if opts.get("active") is not None else None
    ym = _vector(opts["Y"], P, "opts.Y") if opts.get("use_std") else None
    o = _nmf_opts(opts)
    _lib.call("sid_t_update", self._ctx, Yd.data_ptr(), _lib.DTYPE_F16 if half else _lib.DTYPE_F32, T.data_ptr(),
              S.data_ptr(), P, R, F, act.data_ptr() if act is not None else None,
              ym.data_ptr() if ym is not None else None, ctypes.byref(o), _lib.PREC[prec], _stream_ptr())
    return S, T


def _s_update(self, Y, S, T, opts=None, prec="split"):
    """[S, T] = S_update(Y, S, T, opts) (S_update.m:1) on the GPU."""
    opts = dict(opts or {})
    Yd, half = _movie(Y)
    T = to_device(T).clone()
    S = to_device(S).clone()
    P, R = S.shape
    F = T.shape[1]
    if T.shape[0] != R or Yd.shape != (P, F):
        raise ValueError(f"shapes: Y {tuple(Yd.shape)}, T {tuple(T.shape)}, S {tuple(S.shape)}")
    ym = _vector(opts["Y"], P, "opts.Y") if opts.get("use_std") else None
    hilf = None
    if opts.get("lamb_orth_L1", 0) or opts.get("lamb_orth_L2", 0):
        hilf = to_device(opts["hilf"])
        if tuple(hilf.shape) != (R, R):
            raise ValueError(f"opts.hilf must be {R} x {R}")
    o = _nmf_opts(opts)
    _lib.call("sid_s_update", self._ctx, Yd.data_ptr(), _lib.DTYPE_F16 if half else _lib.DTYPE_F32, S.data_ptr(),
              T.data_ptr(), P, R, F, ym.data_ptr() if ym is not None else None,
              hilf.data_ptr() if hilf is not None else None, ctypes.byref(o), _lib.PREC[prec], _stream_ptr())
    return S, T


Context.t_update = _t_update
Context.s_update = _s_update


def T_update(Y, T, S, opts=None):
    """[S, T] = T_update(Y, T, S, opts) (T_update.m:1)."""
    return _ctx().t_update(Y, T, S, opts)


def S_update(Y, S, T, opts=None):
    """[S, T] = S_update(Y, S, T, opts) (S_update.m:1)."""
    return _ctx().s_update(Y, S, T, opts)
