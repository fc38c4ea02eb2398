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

    def timing(self, on: bool):
        """Time the tensor-core GEMM launches of gram / cross (sid_ctx_timing_enable)."""
        _lib.call("sid_ctx_timing_enable", self._ctx, 1 if on else 0)

    def timing_read(self):
        """(total_ms, timed calls) of the GEMM launches since the last read."""
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        _lib.call("sid_ctx_timing_read", self._ctx, ctypes.byref(ms), ctypes.byref(n))
        return ms.value, n.value

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


class NnlsOpts(ctypes.Structure):
    """sid_nnls_opts: the reference's opts fields for LS_nnls / fast_nnls."""
    _fields_ = [("lambda_", ctypes.c_double), ("sample", ctypes.c_int64), ("tol", ctypes.c_double),
                ("tol_", ctypes.c_double), ("max_iter", ctypes.c_int64), ("use_std", ctypes.c_int),
                ("tol_p", ctypes.c_int)]


def _opts(kind: str, opts: dict | None) -> NnlsOpts:
    o = NnlsOpts()
    getattr(_lib.load(), f"sid_{kind}_defaults")(ctypes.byref(o))
    for k, v in (opts or {}).items():
        if k == "lambda":
            o.lambda_ = float(v)
        elif k in ("sample", "max_iter"):
            setattr(o, k, int(v))
        elif k in ("tol", "tol_"):
            setattr(o, k, float(v))
        elif k in ("use_std", "tol_p"):
            setattr(o, k, int(bool(v)) if k == "use_std" else int(v))
        elif k in ("warm_start", "gpu", "gpu_id", "gpu_ids", "display", "total"):
            pass
        else:
            raise ValueError(f"unknown NNLS option {k!r}")
    return o


def _movie(Y):
    half = (isinstance(Y, torch.Tensor) and Y.dtype == torch.float16) or \
           (isinstance(Y, np.ndarray) and Y.dtype == np.float16)
    return (_to_device_half(Y) if half else to_device(Y)), half


def _need(who, what, t, n):
    """t holds n elements (libsid reads exactly that many from a device pointer)."""
    if t is not None and t.numel() != n:
        raise ValueError(f"{who}: {what} must hold {n} elements, got {t.numel()}")


def _ls_nnls(self, A, Y, opts=None, G=None, x=None, prec="split", return_iters=False):
    """[X, G] = LS_nnls(A, Y, opts, G, x) (LS_nnls.m:1) on the GPU."""
    A = to_device(A)
    Yd, half = _movie(Y)
    P, K = A.shape
    F = Yd.shape[1]
    o = _opts("ls_nnls", opts)
    _need("LS_nnls", "Y's rows x frames", Yd, P * F)
    Gd = to_device(G) if G is not None else _fortran_tensor((K, K), A.device)
    X = to_device(x).clone() if x is not None else _fortran_tensor((K, F), A.device)
    _need("LS_nnls", "G", Gd, K * K)
    _need("LS_nnls", "x", X, K * F)
    it = torch.zeros(F, dtype=torch.int32, device=A.device)
    _lib.call("sid_ls_nnls", self._ctx, A.data_ptr(), Yd.data_ptr(), _lib.DTYPE_F16 if half else _lib.DTYPE_F32,
              P, K, F, ctypes.byref(o), Gd.data_ptr(), 1 if G is not None else 0, X.data_ptr(),
              1 if x is not None else 0, _lib.PREC[prec], it.data_ptr(), _stream_ptr())
    return (X, Gd, it) if return_iters else (X, Gd)


def _fast_nnls(self, A, Y, opts=None, Q=None, df=None, h=None, prec="split", return_iters=False, full=False):
    """[xx, Q] = fast_nnls(A, Y, opts, Q, df, h) (fast_nnls.m:1) on the GPU.

    opts may carry warm_start (a K x F matrix, or the scalar 1 for the
    inverse-Gram start of fast_nnls.m:66-69) and total (one step length for
    all columns, fast_nnls.m:101-117).  Q and h (the normalised Gram and the
    scaling of a previous call) are passed together; df is optional
    (fast_nnls.m:58-62).  ``opts=None`` is the reference's two-argument call,
    whose tolerance is 1e-12 (fast_nnls.m:12-15).  full=True returns
    (xx, Q, df, h) like the reference's four outputs (df has no columns unless
    total mode, as the reference removes every retired column from it)."""
    two_args = opts is None
    opts = dict(opts or {})
    if two_args:
        opts["tol"] = 1e-12
    warm = opts.get("warm_start", None)
    total = 1 if opts.get("total", 0) else 0
    warm_mode, W = 0, None
    if warm is not None and np.ndim(warm) == 0:
        if float(warm) != 1:
            raise ValueError("fast_nnls: a scalar warm_start must be 1 (the inverse-Gram start)")
        warm_mode = 1
    elif warm is not None and np.size(warm):
        warm_mode, W = 2, to_device(warm)
    o = _opts("fast_nnls", opts)
    if (Q is None) != (h is None):
        raise ValueError("fast_nnls: Q and h are passed together (fast_nnls.m:58-62)")
    Qd = to_device(Q) if Q is not None else None
    hd = to_device(np.reshape(h, -1) if not isinstance(h, torch.Tensor) else h.reshape(-1)) if h is not None else None
    dfd = to_device(df) if df is not None and np.size(df) else None
    Ad = to_device(A) if A is not None else None
    K = Ad.shape[1] if Ad is not None else Qd.shape[0]
    if Y is not None:
        Yd, half = _movie(Y)
        F = Yd.shape[1]
    else:
        Yd, half = None, False
        F = dfd.shape[1]
    P = Ad.shape[0] if Ad is not None else 0
    if Ad is not None and Yd is not None:
        _need("fast_nnls", "Y (the rows of A x frames)", Yd, P * F)
    _need("fast_nnls", "warm_start", W, K * F)
    _need("fast_nnls", "Q", Qd, K * K)
    _need("fast_nnls", "h", hd, K)
    _need("fast_nnls", "df", dfd, K * F)
    X = _fortran_tensor((K, F), "cuda")
    Qo = _fortran_tensor((K, K), "cuda")
    ho = torch.empty(K, dtype=torch.float32, device="cuda")
    dfo = _fortran_tensor((K, F), "cuda") if total else None
    it = torch.zeros(F, dtype=torch.int32, device="cuda")
    _lib.call("sid_fast_nnls_ex", self._ctx, Ad.data_ptr() if Ad is not None else None,
              Yd.data_ptr() if Yd is not None else None, _lib.DTYPE_F16 if half else _lib.DTYPE_F32, P, K, F,
              ctypes.byref(o), total, warm_mode, W.data_ptr() if W is not None else None,
              Qd.data_ptr() if Qd is not None else None, dfd.data_ptr() if dfd is not None else None,
              hd.data_ptr() if hd is not None else None, X.data_ptr(), Qo.data_ptr(),
              dfo.data_ptr() if dfo is not None else None, ho.data_ptr(), _lib.PREC[prec], it.data_ptr(),
              _stream_ptr())
    if full:
        dfr = dfo if dfo is not None else _fortran_tensor((K, 0), "cuda")
        out = (X, Qo, dfr, ho)
        return out + (it,) if return_iters else out
    return (X, Qo, it) if return_iters else (X, Qo)


def _flat_f(a, dtype):
    """1-D contiguous CUDA tensor of a's elements in column-major order."""
    if isinstance(a, torch.Tensor):
        t = a.to(device="cuda", dtype=dtype)
        return t.permute(*reversed(range(t.dim()))).contiguous().reshape(-1)
    arr = np.asarray(a)
    arr = arr.astype(np.float32 if dtype == torch.float32 else np.uint8)
    return torch.from_numpy(np.ascontiguousarray(arr.ravel(order="F"))).to("cuda")


def _quantile(self, x, p, exclude=None):
    """MATLAB quantile(x(exclude == 0), p) of a vector (NaN ignored), computed
    by libsid's radix select; returns a float or a NumPy array like p."""
    xd = _flat_f(x, torch.float32)
    ex = None
    if exclude is not None:
        ex = _flat_f(exclude, torch.uint8)
        if ex.numel() != xd.numel():
            raise ValueError("exclude must have one entry per value")
    ps = np.atleast_1d(np.asarray(p, dtype=np.float64))
    out = np.zeros(ps.size)
    _lib.call("sid_quantile", self._ctx, xd.data_ptr(), xd.numel(), ex.data_ptr() if ex is not None else None,
              ps.ctypes.data, ps.size, out.ctypes.data, _stream_ptr())
    return float(out[0]) if np.ndim(p) == 0 else out.reshape(np.shape(p))


Context.quantile = _quantile
Context.ls_nnls = _ls_nnls
Context.fast_nnls = _fast_nnls

_DEFAULT_CTX = None


def _ctx():
    global _DEFAULT_CTX
    if _DEFAULT_CTX is None:
        _DEFAULT_CTX = Context()
    return _DEFAULT_CTX


def quantile(x, p, exclude=None):
    """MATLAB quantile of a vector on the GPU (see Context.quantile)."""
    return _ctx().quantile(x, p, exclude)


def LS_nnls(A, Y, opts=None, G=None, x=None):
    """[X, G] = LS_nnls(A, Y, opts, G, x) (LS_nnls.m:1)."""
    return _ctx().ls_nnls(A, Y, opts, G, x)


def fast_nnls(A, Y, opts=None, Q=None, df=None, h=None):
    """[xx, Q, df, h] = fast_nnls(A, Y, opts, Q, df, h) (fast_nnls.m:1)."""
    return _ctx().fast_nnls(A, Y, opts, Q, df, h, full=True)


def _spatial_update(self, timeseries, sensor_movie, template, opts=None):
    """forward_model = update_spatial_component(timeseries, sensor_movie,
    template, opts) (update_spatial_component.m:1), dense (R x P)."""
    opts = dict(opts or {})
    T = to_device(timeseries)
    Yd, half = _movie(sensor_movie)
    R, F = T.shape
    P = Yd.shape[0]
    tm = template
    if isinstance(tm, torch.Tensor):
        tm = tm.to(device="cuda", dtype=torch.uint8)
        tm = tm.permute(1, 0).contiguous().permute(1, 0)
    else:
        arr = np.asfortranarray(np.asarray(tm).astype(np.uint8))
        tm = torch.from_numpy(np.ascontiguousarray(arr.T)).to("cuda").permute(1, 0)
    bg = 1 if opts.get("bg_sub", 1) else 0
    if tm.shape != (R - bg, P):
        raise ValueError(f"template must be {(R - bg, P)}, got {tuple(tm.shape)}")
    out = _fortran_tensor((R, P), T.device)
    status = torch.zeros(P, dtype=torch.int32, device=T.device)
    _lib.call("sid_spatial_update", self._ctx, T.data_ptr(), Yd.data_ptr(),
              _lib.DTYPE_F16 if half else _lib.DTYPE_F32, tm.data_ptr(), R, F, P,
              float(opts.get("lamb_L1", 0.0)), float(opts.get("lamb_L2", 0.0)),
              float(opts.get("lamb_orth_L1", 0.0)), 1 if opts.get("use_std", False) else 0, bg,
              out.data_ptr(), status.data_ptr(), _stream_ptr())
    return out


Context.spatial_update = _spatial_update


def update_spatial_component(timeseries, sensor_movie, template, opts=None):
    """forward_model = update_spatial_component(timeseries, sensor_movie, template, opts)."""
    return _ctx().spatial_update(timeseries, sensor_movie, template, opts)


def _f64_fortran(a):
    """1-D contiguous CUDA float64 tensor of a's elements in column-major order."""
    if isinstance(a, torch.Tensor):
        t = a.to(device="cuda", dtype=torch.float64)
        return t.permute(*reversed(range(t.dim()))).contiguous().reshape(-1)
    arr = np.asarray(a, dtype=np.float64)
    return torch.from_numpy(np.ascontiguousarray(arr.ravel(order="F"))).to("cuda")


def _nqp(self, Q, b, opts=None):
    """[x, w, info] = NQP(Q, b, opts) (NQP.m:1, default options) on the GPU:
    argmin_{x >= 0} 0.5 x'Qx + b'x in FP64 by the Lawson-Hanson active set.
    Q is n x n, or n x n x B for B independent problems solved at once (b then
    n x B); n <= 4096 (problems above 32 components keep their working
    arrays in device scratch).  x and w are CUDA float64 tensors shaped like b; info
    carries ``iter`` (an int, or a B-vector).  A problem that reaches the
    iteration cap raises SidError, as NQP.m:116-119 raises its error."""
    opts = dict(opts or {})
    # NQP.m reads Tol, Iter and Order (NQP.m:63-80); other fields are ignored
    if "Order" in opts or opts.get("Tol", 0) != 0 or "Iter" in opts:
        raise NotImplementedError("NQP: only the default options (no Order, Tol 0, default Iter) are supported")
    Qs = tuple(Q.shape) if isinstance(Q, torch.Tensor) else np.shape(Q)
    bs = tuple(b.shape) if isinstance(b, torch.Tensor) else np.shape(b)
    if len(Qs) not in (2, 3) or Qs[0] != Qs[1]:
        raise ValueError(f"NQP: Q must be n x n or n x n x B, got {Qs}")
    n = int(Qs[0])
    B = int(Qs[2]) if len(Qs) == 3 else 1
    if int(np.prod(bs)) != n * B:
        raise ValueError(f"NQP: b must hold {n} x {B} values, got {bs}")
    Qd, bd = _f64_fortran(Q), _f64_fortran(b)
    x = torch.empty(B, n, dtype=torch.float64, device="cuda")
    w = torch.empty(B, n, dtype=torch.float64, device="cuda")
    it = torch.zeros(B, dtype=torch.int32, device="cuda")
    _lib.call("sid_nqp_batched", self._ctx, Qd.data_ptr(), bd.data_ptr(), n, B, x.data_ptr(), w.data_ptr(),
              it.data_ptr(), None, _stream_ptr())
    if len(Qs) == 2:
        return x[0], w[0], {"iter": int(it[0])}
    return x.T, w.T, {"iter": it}


Context.nqp = _nqp


def NQP(Q, b, opts=None):
    """[x, w, info] = NQP(Q, b, opts) (NQP.m:1)."""
    return _ctx().nqp(Q, b, opts)


def reg_nnls(A, d, opts=None):
    """x = reg_nnls(A, d, opts) (reg_nnls.m:1): the regularised NNLS
    min_{x >= 0} ||A x - d||^2 (+ L1, L2, orthogonality terms) as one NQP.  The
    n x n system is formed in FP64 by libsid (reg_nnls.m:40-66) and solved by
    its Lawson-Hanson kernel (sid_reg_nnls)."""
    return _ctx().reg_nnls(A, d, opts)


def _reg_nnls(self, A, d, opts=None):
    opts = dict(opts or {})
    At = _f64_fortran(A)
    m, n = (tuple(A.shape) if isinstance(A, torch.Tensor) else np.shape(A))[:2]
    dt = _f64_fortran(d)
    if dt.numel() != m:
        raise ValueError(f"reg_nnls: d must hold {m} values, got {dt.numel()}")
    hilf = opts.get("hilf")
    hd = _f64_fortran(hilf) if hilf is not None else None
    if hd is not None and hd.numel() != n * n:
        raise ValueError(f"reg_nnls: hilf must be {n} x {n}")
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.call("sid_reg_nnls", self._ctx, At.data_ptr(), m, n, dt.data_ptr(), float(opts.get("lamb_L1", 0.0)),
              float(opts.get("lamb_L2", 0.0)), float(opts.get("lamb_orth_L1", 0.0)),
              1 if opts.get("use_std", False) else 0, 1 if opts.get("bg_sub", 0) else 0,
              hd.data_ptr() if hd is not None else None, x.data_ptr(), _stream_ptr())
    return x


Context.reg_nnls = _reg_nnls
