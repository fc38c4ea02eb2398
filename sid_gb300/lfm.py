"""Light-field projector and deconvolution, mirroring the reference's MATLAB API.

Reference functions mirrored here (names, argument meaning, error behaviour):

* ``forwardProjectGPU(H, realspace)``            forwardProjectGPU.m:1
* ``backwardProjectGPU_new(H, projection)``       backwardProjectGPU_new.m:1
* ``forwardProjectACC(H, realspace, CAindex)``    forwardProjectACC.m:1
* ``backwardProjectACC_new(H, projection, CAindex)`` backwardProjectACC_new.m:1
* ``deconvRL(forwardFUN, backwardFUN, Htf, maxIter, Xguess, opts)`` deconvRL.m:1
* ``LS_deconv(forwardFUN, backwardFUN, df, opts)`` LS_deconv.m:1

Arrays use MATLAB's shapes and column-major layout: a NumPy array in Fortran
order, or a CUDA ``torch.Tensor`` whose reversed-dimension view is contiguous
(e.g. ``torch.empty(Z, Y, X).permute(2, 1, 0)``).  All arithmetic runs in
libsid on the GPU; this module only moves buffers and checks arguments.

The reference passes projectors as function handles.  Here a ``Projector``
owns the resident PSF plan; its ``forward`` / ``adjoint`` methods are the
handles, and the solvers recognise them and run the whole iteration natively.
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np
import torch

from . import _lib

_DEFAULT_METHOD = "direct"


def set_default_method(method: str):
    """Projection form used by the function-style API: 'direct' (FP32 lenslet
    convolution), 'spectral_f32' (FP32 lenslet-grid spectra), 'spectral_i16'
    (16-bit block-floating-point spectra), 'spectral_mixed' (16-bit forward,
    24-bit float back projection) or 'spectral_mixed_f32' (16-bit forward, FP32
    back projection)."""
    global _DEFAULT_METHOD
    if method not in _lib.METHODS:
        raise ValueError(f"unknown method {method!r}")
    _DEFAULT_METHOD = method


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("sid_gb300 needs a CUDA GPU: the projector has no CPU implementation")


def _fortran_tensor(shape, device):
    """Uninitialised float32 CUDA tensor with MATLAB column-major strides."""
    return torch.empty(tuple(reversed(shape)), dtype=torch.float32, device=device).permute(
        *reversed(range(len(shape))))


def _is_fortran(t: torch.Tensor) -> bool:
    return t.permute(*reversed(range(t.dim()))).is_contiguous()


def to_device(a, device=None) -> torch.Tensor:
    """MATLAB-layout float32 CUDA tensor from a NumPy array or tensor."""
    _require_cuda()
    if isinstance(a, torch.Tensor):
        t = a.to(device=device or "cuda", dtype=torch.float32)
        if not _is_fortran(t):
            t = t.permute(*reversed(range(t.dim()))).contiguous().permute(*reversed(range(t.dim())))
        return t
    arr = np.asfortranarray(np.asarray(a, dtype=np.float32))
    t = torch.from_numpy(np.ascontiguousarray(arr.T)).to(device or "cuda")
    return t.permute(*reversed(range(t.dim())))


def to_numpy(t: torch.Tensor) -> np.ndarray:
    """Fortran-ordered NumPy copy of a MATLAB-layout tensor."""
    return np.asfortranarray(t.permute(*reversed(range(t.dim()))).contiguous().cpu().numpy().T)


def _stream_ptr():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class ReconOpts(ctypes.Structure):
    """sid_recon_opts: the reconstruct_S options the component driver reads."""
    _fields_ = [("q", ctypes.c_double), ("lamb_L1", ctypes.c_double), ("lamb_L2", ctypes.c_double),
                ("solver", ctypes.c_int), ("max_iter", ctypes.c_int)]


class Projector:
    """Resident light-field projector for one PSF (a ``sid_plan``).

    Parameters
    ----------
    H : (M, M, Nnum, Nnum, Z) array, the PSF ``psf_ballistic.H``.
    image_size : (X, Y) sensor / volume lateral size.
    CAindex : optional (Z, 2) 1-based per-depth crop (``psf_ballistic.CAindex``);
        None reproduces forwardProjectGPU / backwardProjectGPU_new.
    methods : operator forms to build ('direct', 'spectral_f32', 'spectral_i16').
    batched : also build the transposed 24-bit spectra (SID_PLAN_SPECTRAL_TC) so
        that the batched calls of 'spectral_mixed' contract up to 64 volumes per
        pass on the tensor cores.
    """

    def __init__(self, H, image_size, CAindex=None, methods=("direct",), batched=False):
        _require_cuda()
        Hn = np.asfortranarray(np.asarray(H, dtype=np.float32))
        if Hn.ndim == 4:
            Hn = Hn[..., None]
        if Hn.ndim != 5 or Hn.shape[0] != Hn.shape[1] or Hn.shape[2] != Hn.shape[3]:
            raise ValueError(f"H must be M x M x Nnum x Nnum x Z, got {Hn.shape}")
        self.M, _, self.Nnum, _, self.Z = Hn.shape
        self.X, self.Y = int(image_size[0]), int(image_size[1])
        ca = None
        if CAindex is not None:
            ca = np.asfortranarray(np.asarray(CAindex, dtype=np.int32).reshape(self.Z, 2))
        flags = 0
        for m in methods:
            flags |= _lib.PLAN_FLAG_FOR_METHOD[m]
        if batched:
            flags |= _lib.PLAN_SPECTRAL_F24 | _lib.PLAN_SPECTRAL_TC
        self.methods = tuple(methods)
        self.default_method = self.methods[0]
        plan = ctypes.c_void_p()
        torch.cuda.current_device()  # make sure the CUDA context exists
        _lib.call("sid_plan_create", Hn.ctypes.data, self.M, self.Nnum, self.Z,
                  ca.ctypes.data if ca is not None else None, self.X, self.Y, flags, ctypes.byref(plan))
        self._plan = plan
        self._finalizer = weakref.finalize(self, _lib.load().sid_plan_destroy, plan)

    # -- info ---------------------------------------------------------------
    def info(self) -> dict:
        buf = (ctypes.c_int64 * 14)()
        _lib.call("sid_plan_info", self._plan, ctypes.cast(buf, ctypes.c_void_p))
        keys = ["M", "Nnum", "Z", "X", "Y", "Lx", "Ly", "D", "L", "device_bytes", "flags", "adj_separate",
                "weak_voxels", "weak_launches"]
        return dict(zip(keys, list(buf)))

    def set_kernel(self, kernel):
        """Compose every projection of this plan with convn(., kernel, 'same')
        (reconstruct_S.m:126-127): forward P(convn(X, k)), back projection
        convn(P'(y), k).  kernel: 3-D array (kx, ky, kz <= 64); None removes it."""
        if kernel is None:
            _lib.call("sid_plan_set_kernel", self._plan, None, 0, 0, 0)
            return
        k = np.asfortranarray(np.asarray(kernel, dtype=np.float32))
        k = k.reshape(k.shape + (1,) * (3 - k.ndim), order="F")
        _lib.call("sid_plan_set_kernel", self._plan, k.ctypes.data, *k.shape)

    def set_weak_fraction(self, frac: float):
        """Voxels with column mass A'1 below `frac` of the largest get exact back
        projections in the spectral forms (default 1e-2; 0 turns it off)."""
        _lib.call("sid_plan_set_weak_fraction", self._plan, float(frac))

    def close(self):
        self._finalizer()

    def release_workspaces(self):
        """Free the plan's solver and projection workspaces (sid_plan_release_workspaces)."""
        _lib.call("sid_plan_release_workspaces", self._plan)

    def _need(self, who, kind, *arrays):
        """Every array holds the plan's volume (kind 'v': X*Y*Z elements) or
        sensor image ('i': X*Y): libsid reads exactly that many."""
        n = self.X * self.Y * (self.Z if kind == "v" else 1)
        for a in arrays:
            m = a.numel() if isinstance(a, torch.Tensor) else int(np.size(a))
            if m != n:
                raise ValueError(f"{who}: expected the plan's {'volume' if kind == 'v' else 'image'} "
                                 f"({n} elements), got {m}")

    def _method(self, method):
        m = method or self.default_method
        if m not in _lib.METHODS:
            raise ValueError(f"unknown method {m!r}")
        return _lib.METHODS[m]

    # -- operators ------------------------------------------------------------
    def forward(self, V, method=None, out=None) -> torch.Tensor:
        """Sensor image A V (X, Y) of a volume V (X, Y, Z)."""
        V = to_device(V)
        if tuple(V.shape) != (self.X, self.Y, self.Z):
            raise ValueError(f"volume must be {(self.X, self.Y, self.Z)}, got {tuple(V.shape)}")
        I = out if out is not None else _fortran_tensor((self.X, self.Y), V.device)
        _lib.call("sid_forward", self._plan, self._method(method), V.data_ptr(), I.data_ptr(), _stream_ptr())
        return I

    def adjoint(self, I, method=None, out=None) -> torch.Tensor:
        """Back projection A^T I (X, Y, Z) of a sensor image I (X, Y)."""
        I = to_device(I)
        if tuple(I.shape) != (self.X, self.Y):
            raise ValueError(f"image must be {(self.X, self.Y)}, got {tuple(I.shape)}")
        V = out if out is not None else _fortran_tensor((self.X, self.Y, self.Z), I.device)
        _lib.call("sid_adjoint", self._plan, self._method(method), I.data_ptr(), V.data_ptr(), _stream_ptr())
        return V

    def forward_host(self, V, method=None) -> np.ndarray:
        """Host-array form (inputs and result on the host, copies inside)."""
        Vn = np.asfortranarray(np.asarray(V, dtype=np.float32))
        self._need("forward_host", "v", Vn)
        I = np.zeros((self.X, self.Y), dtype=np.float32, order="F")
        _lib.call("sid_forward_host", self._plan, self._method(method), Vn.ctypes.data, I.ctypes.data)
        return I

    def adjoint_host(self, I, method=None) -> np.ndarray:
        In = np.asfortranarray(np.asarray(I, dtype=np.float32))
        self._need("adjoint_host", "i", In)
        V = np.zeros((self.X, self.Y, self.Z), dtype=np.float32, order="F")
        _lib.call("sid_adjoint_host", self._plan, self._method(method), In.ctypes.data, V.ctypes.data)
        return V

    def sync(self):
        """Wait for the current stream; raise if a device-side wait expired."""
        _lib.call("sid_plan_sync", self._plan, _stream_ptr())

    # -- solvers ----------------------------------------------------------------
    def isra(self, Htf, Xguess, maxIter, lam=0.0, method=None) -> torch.Tensor:
        Htf = to_device(Htf)
        X = to_device(Xguess).clone()
        self._need("isra", "v", Htf, X)
        _lib.call("sid_deconv_isra", self._plan, self._method(method), Htf.data_ptr(), X.data_ptr(),
                  int(maxIter), float(lam), _stream_ptr())
        return X

    def isra_ex(self, Htf, Xguess, maxIter, mode="basic", p=1, lam=0.0, history=False, method=None):
        """deconvRL in every mode (deconvRL.m:1): mode 'basic' (lam a scalar)
        or 'TV' (lam one weight per axis, p = 1 or 2).  history=True also
        returns Xguess_history (maxIter x X x Y x Z, deconvRL.m:10,90-92)."""
        Htf = to_device(Htf)
        X = to_device(Xguess).clone()
        self._need("isra_ex", "v", Htf, X)
        lam3 = np.zeros(3, dtype=np.float32)
        lv = np.asarray(lam, dtype=np.float64).ravel()
        if mode == "TV":
            lam3[:] = np.broadcast_to(lv, (3,)) if lv.size in (1, 3) else lv[:3]
        else:
            lam3[0] = lv[0] if lv.size else 0.0
        H = None
        if history:
            H = torch.zeros((Htf.shape[2], Htf.shape[1], Htf.shape[0], int(maxIter)), dtype=torch.float32,
                            device=Htf.device).permute(3, 2, 1, 0)
        _lib.call("sid_deconv_isra_ex", self._plan, self._method(method), Htf.data_ptr(), X.data_ptr(),
                  int(maxIter), 1 if mode == "TV" else 0, int(p), lam3.ctypes.data,
                  H.data_ptr() if H is not None else None, _stream_ptr())
        return (X, H) if history else X

    def _ptr_array(self, ts):
        return (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])

    def forward_batched(self, volumes, method=None):
        """[forwardProjectGPU(H, V) for V in volumes], up to four volumes per
        pass over the tap spectra."""
        vs = [to_device(v) for v in volumes]
        self._need("forward_batched", "v", *vs)
        outs = [_fortran_tensor((self.X, self.Y), vs[0].device) for _ in vs]
        _lib.call("sid_forward_batched", self._plan, self._method(method), len(vs),
                  ctypes.cast(self._ptr_array(vs), ctypes.c_void_p), ctypes.cast(self._ptr_array(outs), ctypes.c_void_p),
                  _stream_ptr())
        return outs

    def adjoint_batched(self, images, method=None):
        """[backwardProjectGPU_new(H, I) for I in images]."""
        ims = [to_device(i) for i in images]
        self._need("adjoint_batched", "i", *ims)
        outs = [_fortran_tensor((self.X, self.Y, self.Z), ims[0].device) for _ in ims]
        _lib.call("sid_adjoint_batched", self._plan, self._method(method), len(ims),
                  ctypes.cast(self._ptr_array(ims), ctypes.c_void_p), ctypes.cast(self._ptr_array(outs), ctypes.c_void_p),
                  _stream_ptr())
        return outs

    def isra_batched(self, Htfs, Xguesses, maxIter, lam=0.0, method=None):
        """deconvRL (mode 'basic') for several components at once: one list of
        volumes in, one out (the inputs are not modified)."""
        hs = [to_device(h) for h in Htfs]
        xs = [to_device(x).clone() for x in Xguesses]
        if len(hs) != len(xs):
            raise ValueError("isra_batched: Htf and Xguess lists differ in length")
        self._need("isra_batched", "v", *hs, *xs)
        _lib.call("sid_deconv_isra_batched", self._plan, self._method(method), len(hs),
                  ctypes.cast(self._ptr_array(hs), ctypes.c_void_p), ctypes.cast(self._ptr_array(xs), ctypes.c_void_p),
                  int(maxIter), float(lam), _stream_ptr())
        return xs

    def rl_poisson(self, y, Xguess, maxIter, method=None) -> torch.Tensor:
        """Poisson-likelihood Richardson-Lucy from the sensor image y:
        X <- X .* A'(y ./ AX) ./ A'1 (the reference's deconvRL is the ISRA form)."""
        y = to_device(y)
        X = to_device(Xguess).clone()
        self._need("rl_poisson", "i", y)
        self._need("rl_poisson", "v", X)
        _lib.call("sid_deconv_rl_poisson", self._plan, self._method(method), y.data_ptr(), X.data_ptr(),
                  int(maxIter), _stream_ptr())
        return X

    def isra_host(self, Htf, Xguess, maxIter, lam=0.0, method=None) -> np.ndarray:
        """Host-array ISRA (the MEX path for non-gpuArray inputs): the input
        volume and the result cross the host link inside their layout
        conversions, Htf on a copy engine during the first projections."""
        Hn = np.asfortranarray(np.asarray(Htf, dtype=np.float32))
        X = np.array(Xguess, dtype=np.float32, order="F", copy=True)
        self._need("isra_host", "v", Hn, X)
        _lib.call("sid_deconv_isra_host", self._plan, self._method(method), Hn.ctypes.data, X.ctypes.data,
                  int(maxIter), float(lam))
        return X

    def isra_host_inplace(self, Htf, X, maxIter, lam=0.0, method=None):
        """Like isra_host, updating the Fortran-ordered float32 host array X."""
        if not (isinstance(X, np.ndarray) and X.dtype == np.float32 and X.flags.f_contiguous):
            raise TypeError("X must be a Fortran-ordered float32 array")
        Hn = np.asfortranarray(np.asarray(Htf, dtype=np.float32))
        self._need("isra_host_inplace", "v", Hn, X)
        _lib.call("sid_deconv_isra_host", self._plan, self._method(method), Hn.ctypes.data, X.ctypes.data,
                  int(maxIter), float(lam))
        return X

    def timing(self, on: bool):
        """Enable/disable CUDA-event timing of the dominant kernel launches."""
        _lib.call("sid_plan_timing_enable", self._plan, 1 if on else 0)

    def timing_read(self):
        """(total_ms, launches) of the dominant kernel since the last read."""
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        _lib.call("sid_plan_timing_read", self._plan, ctypes.byref(ms), ctypes.byref(n))
        return ms.value, n.value

    def _recon_opts(self, opts):
        opts = dict(opts or {})
        o = ReconOpts()
        _lib.load().sid_recon_defaults(ctypes.byref(o))
        o.q = float(opts.get("q", o.q))
        o.lamb_L1 = float(opts.get("lamb_L1", o.lamb_L1))
        o.lamb_L2 = float(opts.get("lamb_L2", o.lamb_L2))
        o.max_iter = int(opts.get("max_iter", o.max_iter))
        solver = opts.get("whichSolver", "fast_nnls")
        if solver not in ("fast_nnls", "ISRA"):
            raise NotImplementedError(f"reconstruct_S: solver {solver!r} does not run natively")
        o.solver = 0 if solver == "fast_nnls" else 1
        return o

    def _microlens_mask(self, microlenses):
        if microlenses is None:
            return None
        if isinstance(microlenses, torch.Tensor):  # X x Y mask, flattened column-major
            ml = microlenses.to(device="cuda", dtype=torch.uint8).permute(1, 0).contiguous().reshape(-1)
        else:
            m = np.asarray(microlenses) != 0
            ml = torch.from_numpy(np.ascontiguousarray(m.astype(np.uint8).ravel(order="F"))).to("cuda")
        if ml.numel() != self.X * self.Y:
            raise ValueError("microlenses must be X x Y")
        return ml

    def reconstruct_component(self, img, microlenses=None, opts=None, method=None, return_lambda=False):
        """nrm * solve(A'(img / nrm)) for one component image after the
        background clip of reconstruct_S (reconstruct_S.m:168-205); opts:
        q, lamb_L1, lamb_L2, whichSolver ('fast_nnls' or 'ISRA'), max_iter."""
        o = self._recon_opts(opts)
        im = to_device(img)
        if tuple(im.shape) != (self.X, self.Y):
            raise ValueError(f"component image must be {(self.X, self.Y)}, got {tuple(im.shape)}")
        ml = self._microlens_mask(microlenses)
        X = _fortran_tensor((self.X, self.Y, self.Z), im.device)
        lam = ctypes.c_double()
        _lib.call("sid_reconstruct_component", self._plan, self._method(method), im.data_ptr(),
                  ml.data_ptr() if ml is not None else None, ctypes.byref(o), X.data_ptr(), ctypes.byref(lam),
                  _stream_ptr())
        return (X, lam.value) if return_lambda else X

    def reconstruct_components(self, imgs, microlenses=None, opts=None, method=None, return_lambda=False):
        """reconstruct_component for several component images at once
        (reconstruct_S.m:162-212): back projections and solver iterations run
        on groups of up to 64 components (sid_reconstruct_components)."""
        o = self._recon_opts(opts)
        ims = [to_device(i) for i in imgs]
        for im in ims:
            if tuple(im.shape) != (self.X, self.Y):
                raise ValueError(f"component image must be {(self.X, self.Y)}, got {tuple(im.shape)}")
        ml = self._microlens_mask(microlenses)
        outs = [_fortran_tensor((self.X, self.Y, self.Z), ims[0].device) for _ in ims]
        lam = (ctypes.c_double * len(ims))()
        _lib.call("sid_reconstruct_components", self._plan, self._method(method), len(ims),
                  ctypes.cast(self._ptr_array(ims), ctypes.c_void_p), ml.data_ptr() if ml is not None else None,
                  ctypes.byref(o), ctypes.cast(self._ptr_array(outs), ctypes.c_void_p),
                  ctypes.cast(lam, ctypes.c_void_p), _stream_ptr())
        return (outs, list(lam)) if return_lambda else outs

    def ls_deconv_batched(self, dfs, max_iter=8, lamb_L1=0.0, lamb_L2=0.0, method=None):
        """LS_deconv (plain mode) for several volumes; lamb_L1: one value or one per volume."""
        xs = [to_device(d).clone() for d in dfs]
        self._need("ls_deconv_batched", "v", *xs)
        l1 = np.broadcast_to(np.asarray(lamb_L1, dtype=np.float32), (len(xs),)).copy()
        _lib.call("sid_deconv_ls_batched", self._plan, self._method(method), len(xs),
                  ctypes.cast(self._ptr_array(xs), ctypes.c_void_p), int(max_iter), l1.ctypes.data,
                  float(lamb_L2), _stream_ptr())
        return xs

    def ls_deconv(self, df, max_iter=8, lamb_L1=0.0, lamb_L2=0.0, method=None, lamb_TV_L2=(0.0, 0.0, 0.0),
                  lamb_TV_L1=0.0) -> torch.Tensor:
        X = to_device(df).clone()
        self._need("ls_deconv", "v", X)
        tv = np.zeros(3, dtype=np.float32)
        tv[:] = np.asarray(lamb_TV_L2, dtype=np.float32).ravel()[:3]
        _lib.call("sid_deconv_ls_ex", self._plan, self._method(method), X.data_ptr(), int(max_iter),
                  float(lamb_L1), float(lamb_L2), tv.ctypes.data, float(lamb_TV_L1), _stream_ptr())
        return X


# ---------------------------------------------------------------------------
# Function-style API with the reference's names.  A plan is cached per PSF
# array object (the MEX layer keeps one per psf_ballistic.H in the same way).
# ---------------------------------------------------------------------------
_PLANS: dict = {}


def _plan_for(H, image_size, CAindex, method, batched=False):
    key = (id(H), tuple(np.shape(H)), tuple(image_size), None if CAindex is None else
           tuple(np.asarray(CAindex).ravel().tolist()), method, batched)
    pr = _PLANS.get(key)
    if pr is None or pr[0]() is not H:
        try:
            ref = weakref.ref(H)
        except TypeError:
            ref = (lambda h=H: h)
        _PLANS[key] = (ref, Projector(H, image_size, CAindex, methods=(method,), batched=batched))
        pr = _PLANS[key]
    return pr[1]


def forwardProjectGPU(H, realspace):
    """TOTALprojection = forwardProjectGPU(H, realspace) (forwardProjectGPU.m:1)."""
    shp = tuple(np.shape(realspace))
    return _plan_for(H, shp[:2], None, _DEFAULT_METHOD).forward(realspace)


def backwardProjectGPU_new(H, projection):
    """Backprojection = backwardProjectGPU_new(H, projection) (backwardProjectGPU_new.m:1)."""
    shp = tuple(np.shape(projection))
    return _plan_for(H, shp[:2], None, _DEFAULT_METHOD).adjoint(projection)


def forwardProjectACC(H, realspace, CAindex):
    """TOTALprojection = forwardProjectACC(H, realspace, CAindex) (forwardProjectACC.m:1)."""
    shp = tuple(np.shape(realspace))
    return _plan_for(H, shp[:2], CAindex, "direct").forward(realspace)


def backwardProjectACC_new(H, projection, CAindex):
    """Backprojection = backwardProjectACC_new(H, projection, CAindex) (backwardProjectACC_new.m:1)."""
    shp = tuple(np.shape(projection))
    return _plan_for(H, shp[:2], CAindex, "direct").adjoint(projection)


def _native_pair(forwardFUN, backwardFUN):
    f = getattr(forwardFUN, "__self__", None)
    b = getattr(backwardFUN, "__self__", None)
    if isinstance(f, Projector) and f is b and forwardFUN.__func__ is Projector.forward \
            and backwardFUN.__func__ is Projector.adjoint:
        return f
    return None


def deconvRL(forwardFUN, backwardFUN, Htf, maxIter, Xguess, opts=None, nargout=1):
    """[Xguess, Xguess_history] = deconvRL(forwardFUN, backwardFUN, Htf, maxIter,
    Xguess, opts) (deconvRL.m:1): ISRA in mode 'basic' (opts.lambda a scalar,
    p = 1) or 'TV' (opts.lambda one weight per axis, p = 1 or 2).  The
    projector handles must be a Projector's ``forward`` / ``adjoint``.
    nargout=2 also returns Xguess_history (maxIter x size(Xguess))."""
    opts = dict(opts if opts is not None else {"lambda": 0, "p": 1, "mode": "basic"})
    mode = opts.get("mode", "basic")
    if mode not in ("basic", "TV"):
        raise ValueError(f"deconvRL: unknown mode {mode!r}")
    lam = np.asarray(opts.get("lambda", 0.0), dtype=np.float64).ravel()
    p = int(opts.get("p", 1))
    if mode == "basic" and np.any(lam != 0) and p != 1:
        raise ValueError("deconvRL: mode 'basic' with p != 1 is undefined in the reference")
    if mode == "TV" and np.any(lam != 0) and lam.size != 3:
        raise ValueError("deconvRL: mode 'TV' needs opts.lambda with one weight per axis (1 x 3)")
    proj = _native_pair(forwardFUN, backwardFUN)
    if proj is None:
        raise TypeError("deconvRL: forwardFUN/backwardFUN must be a Projector's forward/adjoint")
    if mode == "basic" and nargout < 2:
        return proj.isra(Htf, Xguess, maxIter, float(lam[0]) if lam.size else 0.0)
    return proj.isra_ex(Htf, Xguess, maxIter, mode=mode, p=p, lam=lam if lam.size else 0.0, history=nargout > 1)


def LS_deconv(forwardFUN, backwardFUN, df, opts=None):
    """Xguess = LS_deconv(forwardFUN, backwardFUN, df, opts) (LS_deconv.m:1),
    with the TV Laplacian term lamb_TV_L2 (1 x 3) and lamb_TV_L1's role in the
    step-length test."""
    opts = dict(opts or {})
    tv = np.asarray(opts.get("lamb_TV_L2", [0.0, 0.0, 0.0]), dtype=np.float64).ravel()
    if tv.size != 3:
        if np.any(tv != 0):
            # LS_deconv.m:50-55 broadcasts a scalar into opts.p, then reads lamb_TV_L2(3)
            raise ValueError("LS_deconv: lamb_TV_L2 must have 3 entries")
        tv = np.zeros(3)
    proj = _native_pair(forwardFUN, backwardFUN)
    if proj is None:
        raise TypeError("LS_deconv: forwardFUN/backwardFUN must be a Projector's forward/adjoint")
    return proj.ls_deconv(df, int(opts.get("max_iter", 8)), float(opts.get("lamb_L1", 0.0)),
                          float(opts.get("lamb_L2", 0.0)), lamb_TV_L2=tv, lamb_TV_L1=float(opts.get("lamb_TV_L1", 0.0)))


def _colon(a, b, step=1.0):
    """MATLAB a:step:b."""
    n = int(np.floor((b - a) / step + 1e-9)) + 1
    return a + step * np.arange(max(n, 0))


def _meshgrid3(x, y, z):
    """MATLAB [X, Y, Z] = meshgrid(x, y, z): arrays of size (numel(y), numel(x), numel(z))."""
    Yg, Xg, Zg = np.meshgrid(y, x, z, indexing="ij")
    return Xg, Yg, Zg


def _fspecial_gaussian(hsize, sigma):
    """The rotationally symmetric Gaussian of fspecial('gaussian', hsize, sigma):
    exp(-(x^2 + y^2) / 2 sigma^2) on an hsize x hsize grid centred at 0, values
    below eps * max set to 0, normalised to sum 1."""
    r = _colon(-(hsize - 1) / 2, (hsize - 1) / 2)
    Xg, Yg = np.meshgrid(r, r)
    h = np.exp(-(Xg ** 2 + Yg ** 2) / (2 * sigma ** 2))
    h[h < np.finfo(np.float64).eps * h.max()] = 0
    return h / h.sum()


def generate_kernel(ker_shape, ker_param):
    """kernel = generate_kernel(ker_shape, ker_param) (generate_kernel.m:1):
    'ball' (radii ker_param(1) laterally, ker_param(2) axially), 'gaussian',
    'lorentz' or 'user' (ker_param is the kernel), normalised to unit L2 norm.
    Returns a Fortran-ordered float64 array."""
    if ker_shape == "ball":
        r1, r2 = float(ker_param[0]), float(ker_param[1])
        Xg, Yg, Zg = _meshgrid3(_colon(-r1, r1), _colon(-r1, r1), _colon(-r2, r2))
        k = ((Xg ** 2 / r1 ** 2 + Yg ** 2 / r1 ** 2 + Zg ** 2 / r2 ** 2) <= 1).astype(np.float64)
    elif ker_shape == "gaussian":
        p1, p2 = float(ker_param[0]), float(ker_param[1])
        n = int(np.ceil(10 * p1)) + 1
        g = _fspecial_gaussian(n, p1)
        zt = np.exp(-_colon(-3 * p2, 3 * p2) ** 2 / 4 / p2 ** 2)
        k = np.reshape(np.outer(g.reshape(-1, order="F"), zt), (n, n, len(zt)), order="F")
    elif ker_shape == "lorentz":
        p1, p2 = float(ker_param[0]), float(ker_param[1])
        a, c = np.ceil(5 * p1), np.ceil(5 * p2)
        Xg, Yg, Zg = _meshgrid3(_colon(-a, a), _colon(-a, a), _colon(-c, c))
        k = 1.0 / (1 + (p1 * (Xg ** 2 + Yg ** 2) + p2 * Zg ** 2))
    elif ker_shape == "user":
        k = np.array(ker_param, dtype=np.float64)
    else:
        raise ValueError(f"generate_kernel: unknown shape {ker_shape!r}")
    k = np.asfortranarray(k.reshape(k.shape + (1,) * (3 - k.ndim)))
    return k / np.linalg.norm(k.ravel())


def reconstruct_S(S, psf_ballistic, opts=None):
    """recon_nnmf = reconstruct_S(S, psf_ballistic, opts) (reconstruct_S.m:1),
    the GPU branch (:158-211): the components S(ii, :, :) reconstructed on
    one resident plan, in groups of up to 64 (sid_reconstruct_components).  S: (n, X, Y); psf_ballistic: dict or object with H;
    opts: q, lamb_L1, lamb_L2, whichSolver, max_iter, microlenses.  Returns a
    list of X x Y x Z CUDA tensors.  With opts.ker_param (and opts.ker_shape,
    default 'user'), the projector is composed with convn(., kernel, 'same')
    both ways (:110-114, :188-189)."""
    opts = dict(opts or {})
    kernel = generate_kernel(opts.get("ker_shape", "user"), opts["ker_param"]) if "ker_param" in opts else None
    tv = np.asarray(opts.get("lamb_TV_L2", 0.0))
    if np.any(tv != 0) or opts.get("lamb_TV_L1", 0):
        raise NotImplementedError("reconstruct_S: TV regularisers do not run natively")
    H = psf_ballistic["H"] if isinstance(psf_ballistic, dict) else psf_ballistic.H
    S = S if isinstance(S, torch.Tensor) else np.asarray(S)
    n, X, Y = S.shape
    method = opts.get("method", _DEFAULT_METHOD)
    # many components: the mixed form's tensor-core batched projections
    P = _plan_for(H, (X, Y), None, method, batched=(method == "spectral_mixed" and n > 1))
    P.set_kernel(kernel)
    try:
        out = P.reconstruct_components([S[ii] for ii in range(n)], opts.get("microlenses"), opts, method=method)
    finally:
        P.set_kernel(None)
    return out


def library_boxes(centers, neur_rad, axial, size):
    """Crop boxes of generate_LFM_library_GPU.m:68-88 as 0-based half-open
    (x0, x1, y0, y1, z0, z1) rows, computed by libsid's host code."""
    c = np.asfortranarray(np.asarray(centers, dtype=np.float64).reshape(-1, 3))
    n = c.shape[0]
    out = np.zeros((n, 6), dtype=np.int32)
    X, Y, Z = size
    _lib.call("sid_library_boxes", c.ctypes.data, n, int(neur_rad), float(axial), X, Y, Z, out.ctypes.data)
    return out


def generate_LFM_library_GPU(recon, centers, neur_id, psf, options, layout="rows", method="direct"):
    """forward_model = generate_LFM_library_GPU(recon, centers, neur_id, psf, options)
    (generate_LFM_library_GPU.m:1).  recon: list of (X, Y, Z) volumes; centers:
    (n, 3) 1-based; neur_id: (n, n_comp) logical; psf: dict with 'H';
    options: dict with 'neur_rad', 'axial'.  Returns the (n, X*Y) library on
    the GPU ('rows', the reference's layout) or its transpose (X*Y, n)
    ('columns', the layout the NNLS solvers take).  method 'direct': FP32
    lenslet taps (sid_library); 'spectral': the tensor-core spectral
    projector on lenslet windows around the boxes (sid_library_spectral,
    about 1e-5 relative per row)."""
    if method not in ("direct", "spectral"):
        raise ValueError(f"method must be 'direct' or 'spectral', not {method!r}")
    H = psf["H"] if isinstance(psf, dict) else psf
    vols = [to_device(r) for r in recon]
    X, Y, Z = vols[0].shape
    proj = _plan_for(H, (X, Y), None, "direct")
    c = np.asfortranarray(np.asarray(centers, dtype=np.float64).reshape(-1, 3))
    n = c.shape[0]
    ids = np.asfortranarray(np.asarray(neur_id).reshape(n, len(vols)).astype(np.uint8))
    ptrs = (ctypes.c_void_p * len(vols))(*[v.data_ptr() for v in vols])
    if layout == "rows":
        out = _fortran_tensor((n, X * Y), vols[0].device)
    else:
        out = _fortran_tensor((X * Y, n), vols[0].device)
    fn = "sid_library" if method == "direct" else "sid_library_spectral"
    _lib.call(fn, proj._plan, ctypes.cast(ptrs, ctypes.c_void_p), len(vols), c.ctypes.data,
              ids.ctypes.data, n, int(options["neur_rad"]), float(options["axial"]), out.data_ptr(),
              0 if layout == "rows" else 1, _stream_ptr())
    return out


def _kernel_args(kernel):
    if kernel is None:
        return None, 0, 0, 0, None
    W = np.asfortranarray(np.asarray(kernel, dtype=np.float32))
    if W.ndim == 2:
        W = W[:, :, None]
    return W.ctypes.data, W.shape[0], W.shape[1], W.shape[2], W


def library_kernel_voxels(centers, r, dim, m, Z, kernel=None):
    """The voxels generate_LFM_library_CPU.m:39-49 paints per neuron: a list of
    (count, 3) 0-based (x, y, z) arrays and their kernel values, computed by
    libsid's host code."""
    c = np.asfortranarray(np.asarray(centers, dtype=np.float64).reshape(-1, 3))
    n = c.shape[0]
    kp, kx, ky, kz, keep = _kernel_args(kernel)
    dz = float(np.asarray(dim, dtype=np.float64).ravel()[2]) if kernel is None else 1.0
    counts = np.zeros(n, dtype=np.int64)
    _lib.call("sid_library_kernel_voxels", c.ctypes.data, n, float(r), dz, kp, kx, ky, kz, int(m[0]), int(m[1]),
              int(Z), counts.ctypes.data, None, None, 0)
    tot = int(counts.sum())
    xyz = np.zeros((max(tot, 1), 3), dtype=np.int32)
    vals = np.zeros(max(tot, 1), dtype=np.float32)
    _lib.call("sid_library_kernel_voxels", c.ctypes.data, n, float(r), dz, kp, kx, ky, kz, int(m[0]), int(m[1]),
              int(Z), counts.ctypes.data, xyz.ctypes.data, vals.ctypes.data, tot)
    del keep
    out, at = [], 0
    for k in counts:
        out.append((xyz[at:at + k].copy(), vals[at:at + k].copy()))
        at += int(k)
    return out


def generate_LFM_library_CPU(centers, psf, r, dim, m, kernel=None, layout="rows", method="direct"):
    """forward_model = generate_LFM_library_CPU(centers, psf_ballistic, r, dim, m, kernel)
    (generate_LFM_library_CPU.m:1): every neuron is the kernel (or the ball of
    radius r, axial radius r / dim(3)) painted at its centre, forward-projected
    and L2-normalised.  Returns the dense (n, X*Y) rows on the GPU ('rows') or
    their transpose ('columns'); the reference's sparse matrix holds their
    nonzeros.  method 'direct' (FP32 lenslet taps) or 'spectral'
    (tensor-core windows)."""
    if method not in ("direct", "spectral"):
        raise ValueError(f"method must be 'direct' or 'spectral', not {method!r}")
    H = psf["H"] if isinstance(psf, dict) else psf
    X, Y = int(m[0]), int(m[1])
    proj = _plan_for(H, (X, Y), None, "direct")
    c = np.asfortranarray(np.asarray(centers, dtype=np.float64).reshape(-1, 3))
    n = c.shape[0]
    kp, kx, ky, kz, keep = _kernel_args(kernel)
    dz = float(np.asarray(dim, dtype=np.float64).ravel()[2]) if kernel is None else 1.0
    out = _fortran_tensor((n, X * Y) if layout == "rows" else (X * Y, n), "cuda")
    _lib.call("sid_library_kernel", proj._plan, _lib.METHODS["direct" if method == "direct" else "spectral_mixed"],
              c.ctypes.data, n, float(r), dz, kp, kx, ky, kz, out.data_ptr(), 0 if layout == "rows" else 1,
              _stream_ptr())
    del keep
    return out
