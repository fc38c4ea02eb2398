"""FP64 CPU restatement of SID's hot path (test infrastructure only).

This module is the checker.  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline / reference arm may import it; the product package
``sid_gb300`` never does.

Parity status: parity unpinned against the real reference.  The reference is
MATLAB R2017b code whose arithmetic lives in MATLAB built-ins (conv2, mtimes,
quantile, linsolve, inv); neither MATLAB nor GNU Octave exists here and the
reference ships no golden vectors.  The projector part is cross-checked against
an independent NumPy/SciPy transcription of the reference's loop structure
(tests/golden/make_golden.py).

Arrays follow MATLAB semantics: column-major (Fortran-order) NumPy arrays with
MATLAB's shapes, e.g. H is (M, M, Nnum, Nnum, Z), a volume is (X, Y, Z), a
movie is (P, F).  The projector and the Lawson-Hanson NQP run in C
(oracle/sid_oracle.c); the solvers below are NumPy restatements of the cited
MATLAB lines.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build() -> str:
    """Compile oracle/sid_oracle.c into oracle/_build/liboracle.so."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return os.path.join(_HERE, "_build", "liboracle.so")


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        p = ctypes.c_void_p
        i = ctypes.c_int64
        lib.oracle_forward.argtypes = [p, i, i, i, p, p, i, i, p]
        lib.oracle_adjoint.argtypes = [p, i, i, i, p, p, i, i, p]
        lib.oracle_forward_pixels.argtypes = [p, i, i, i, p, p, i, i, p, i, p]
        lib.oracle_adjoint_voxels.argtypes = [p, i, i, i, p, p, i, i, p, i, p]
        lib.baseline_forward_f32.argtypes = [p, i, i, i, p, i, i, p, i, i, ctypes.c_int]
        lib.oracle_nqp.argtypes = [p, p, i, p, p, p]
        lib.oracle_nqp.restype = ctypes.c_int
        _LIB = lib
    return _LIB


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _psf(H):
    H = np.asfortranarray(H, dtype=np.float32)
    assert H.ndim == 5 and H.shape[0] == H.shape[1] and H.shape[2] == H.shape[3]
    return H


def _ca(CAindex, Z):
    if CAindex is None:
        return None
    ca = np.asfortranarray(np.asarray(CAindex, dtype=np.int32).reshape(Z, 2))
    return ca


# ----------------------------------------------------------------------------
# L2 operators: forwardProjectACC.m:14-29 / backwardProjectACC_new.m:14-26
# (and the GPU FFT forms, which equal them with CAindex = [1, M]).
# ----------------------------------------------------------------------------
def forward_project(H, V, CAindex=None):
    """Sensor image A V, FP64.  H (M,M,N,N,Z) float32, V (X,Y,Z)."""
    H = _psf(H)
    M, _, N, _, Z = H.shape
    V = np.asfortranarray(V, dtype=np.float64)
    X, Y = V.shape[0], V.shape[1]
    assert V.shape[2] == Z
    ca = _ca(CAindex, Z)
    out = np.zeros((X, Y), dtype=np.float64, order="F")
    _lib().oracle_forward(_ptr(H), M, N, Z, _ptr(ca), _ptr(V), X, Y, _ptr(out))
    return out


def backward_project(H, I, CAindex=None):
    """Back projection A^T I, FP64 (the reference's imrotate(.,180) form)."""
    H = _psf(H)
    M, _, N, _, Z = H.shape
    I = np.asfortranarray(I, dtype=np.float64)
    X, Y = I.shape
    ca = _ca(CAindex, Z)
    out = np.zeros((X, Y, Z), dtype=np.float64, order="F")
    _lib().oracle_adjoint(_ptr(H), M, N, Z, _ptr(ca), _ptr(I), X, Y, _ptr(out))
    return out


def forward_project_pixels(H, V, pixels, CAindex=None):
    """(A V) at 0-based sensor pixels, pixels: (n, 2) int."""
    H = _psf(H)
    M, _, N, _, Z = H.shape
    V = np.asfortranarray(V, dtype=np.float64)
    X, Y = V.shape[0], V.shape[1]
    pix = np.ascontiguousarray(pixels, dtype=np.int64)
    out = np.zeros(pix.shape[0], dtype=np.float64)
    _lib().oracle_forward_pixels(_ptr(H), M, N, Z, _ptr(_ca(CAindex, Z)), _ptr(V), X, Y,
                                 _ptr(pix), pix.shape[0], _ptr(out))
    return out


def backward_project_voxels(H, I, voxels, CAindex=None):
    """(A^T I) at 0-based voxels, voxels: (n, 3) int."""
    H = _psf(H)
    M, _, N, _, Z = H.shape
    I = np.asfortranarray(I, dtype=np.float64)
    X, Y = I.shape
    vox = np.ascontiguousarray(voxels, dtype=np.int64)
    out = np.zeros(vox.shape[0], dtype=np.float64)
    _lib().oracle_adjoint_voxels(_ptr(H), M, N, Z, _ptr(_ca(CAindex, Z)), _ptr(I), X, Y,
                                 _ptr(vox), vox.shape[0], _ptr(out))
    return out


def baseline_forward_f32(H, V, y_begin=0, y_end=None, nthreads=0):
    """FP32 lenslet-sparse forward projection on the host cores (the timed CPU
    baseline), optionally restricted to sensor columns [y_begin, y_end)."""
    H = _psf(H)
    M, _, N, _, Z = H.shape
    V = np.asfortranarray(V, dtype=np.float32)
    X, Y = V.shape[0], V.shape[1]
    y_end = Y if y_end is None else y_end
    out = np.zeros((X, Y), dtype=np.float32, order="F")
    _lib().baseline_forward_f32(_ptr(H), M, N, Z, _ptr(V), X, Y, _ptr(out),
                                y_begin, y_end, int(nthreads))
    return out


# ----------------------------------------------------------------------------
# MATLAB helpers restated
# ----------------------------------------------------------------------------
def matlab_quantile(v, p):
    """MATLAB quantile of a vector: NaNs dropped, sorted data at positions
    (k-0.5)/n with linear interpolation, clamped to the extremes (NumPy's
    'hazen' rule); NaN when no value is left."""
    v = np.asarray(v, dtype=np.float64).ravel()
    v = np.sort(v[~np.isnan(v)])
    n = v.size
    if n == 0:
        return np.nan
    t = n * p + 0.5  # 1-based fractional position
    if t <= 1:
        return v[0]
    if t >= n:
        return v[-1]
    lo = int(np.floor(t))
    f = t - lo
    return v[lo - 1] + f * (v[lo] - v[lo - 1])


# ----------------------------------------------------------------------------
# L3 deconvolution: deconvRL.m:46-93 (ISRA) and LS_deconv.m:49-93
# ----------------------------------------------------------------------------
def deconvRL(forward, backward, Htf, maxIter, Xguess, opts=None):
    """ISRA multiplicative update X <- X .* Htf ./ (A^T A X [+ lambda]).
    Implements opts.mode 'basic' with lambda == 0 and p == 1 (deconvRL.m:49-60);
    'basic' with p != 1 reads an undefined variable in the reference and is
    rejected here too.  'TV' p = 1 / p = 2 follow deconvRL.m:61-83."""
    if opts is None:
        opts = {"lambda": 0.0, "p": 1, "mode": "basic"}
    X = np.array(Xguess, dtype=np.float64, order="F")
    Htf = np.asarray(Htf, dtype=np.float64)
    mode = opts.get("mode", "basic")
    lam = opts.get("lambda", 0.0)
    p = opts.get("p", 1)
    for _ in range(int(maxIter)):
        HX = forward(X)
        with np.errstate(divide="ignore", invalid="ignore"):
            if mode == "basic":
                if np.all(np.asarray(lam) == 0):
                    err = Htf / backward(HX)
                elif p == 1:
                    err = Htf / (backward(HX) + lam)
                else:
                    raise ValueError("deconvRL: mode 'basic' with p != 1 is undefined in the reference")
            elif mode == "TV":
                lam3 = np.broadcast_to(np.asarray(lam, dtype=np.float64), (3,))
                if np.all(lam3 == 0):
                    err = Htf / backward(HX)
                elif p == 1:
                    # convn(X, center-left, 'same') = X(i) - X(i+1) along each
                    # axis; convn(dx, right, 'same') = dx(i-1)
                    dx = np.sign(X - _shift(X, 0, +1))
                    dy = np.sign(X - _shift(X, 1, +1))
                    dz = np.sign(X - _shift(X, 2, +1))
                    den = backward(HX) + lam3[0] * dx + lam3[1] * dy + lam3[2] * dz + lam3.sum()
                    num = (Htf + lam3[0] * _shift(dx, 0, -1) + lam3[1] * _shift(dy, 1, -1)
                           + lam3[2] * _shift(dz, 2, -1) + lam3.sum())
                    err = num / den
                elif p == 2:
                    den = backward(HX) + 2.0 * lam3.sum() * X
                    num = Htf + sum(lam3[d] * (_shift(X, d, -1) + _shift(X, d, +1)) for d in range(3))
                    err = num / den
                else:
                    # deconvRL.m:79-81 prints 'p>2 not supported' and returns Xguess
                    return X
            else:
                raise ValueError("deconvRL: unknown mode")
            err[np.isinf(err)] = 0.0
            X = X * err
            X[np.isnan(X)] = 0.0
    return X


def rl_poisson(forward, backward, y, maxIter, Xguess):
    """Poisson-likelihood Richardson-Lucy (Richardson 1972, Lucy 1974):
    X <- X .* A'(y ./ AX) ./ A'1, ratios that are not finite -> 0, then the zero
    rules of deconvRL.m:85-87 (inf -> 0 in the factor, NaN -> 0 in X)."""
    X = np.array(Xguess, dtype=np.float64, order="F")
    y = np.asarray(y, dtype=np.float64)
    norm = backward(np.ones_like(y))
    for _ in range(int(maxIter)):
        with np.errstate(divide="ignore", invalid="ignore"):
            r = y / forward(X)
            r[~np.isfinite(r)] = 0.0
            e = backward(r) / norm
            e[np.isinf(e)] = 0.0
            X = X * e
            X[np.isnan(X)] = 0.0
    return X


def _shift(X, axis, direction):
    """Zero-filled neighbour: direction -1 returns X at index-1 (0 at the lower
    edge), +1 returns X at index+1.  convn(X, e_k, 'same') with a 3-tap unit
    filter is such a shift."""
    out = np.zeros_like(X)
    src = [slice(None)] * X.ndim
    dst = [slice(None)] * X.ndim
    if direction < 0:
        src[axis] = slice(0, -1)
        dst[axis] = slice(1, None)
    else:
        src[axis] = slice(1, None)
        dst[axis] = slice(0, -1)
    out[tuple(dst)] = X[tuple(src)]
    return out


def LS_deconv(forward, backward, df, opts=None):
    """Projected gradient with exact line search (LS_deconv.m:49-93), the
    default solver of reconstruct_S.  TV/L2 terms are the reference's 3-D
    7-point filters (LS_deconv.m:52-71)."""
    opts = dict(opts or {})
    lamb_TV_L1 = opts.get("lamb_TV_L1", 0.0)
    lamb_TV_L2 = np.asarray(opts.get("lamb_TV_L2", [0, 0, 0]), dtype=np.float64).ravel()
    if lamb_TV_L2.size != 3:
        if np.any(lamb_TV_L2):
            # LS_deconv.m:53-55 assigns the broadcast to opts.p, so a scalar
            # weight then fails on lamb_TV_L2(3)
            raise ValueError("LS_deconv: lamb_TV_L2 must have 3 entries")
        lamb_TV_L2 = np.zeros(3)
    lamb_L1 = opts.get("lamb_L1", 0.0)
    lamb_L2 = opts.get("lamb_L2", 0.0)
    max_iter = int(opts.get("max_iter", 8))

    def tv(X):
        if not np.any(lamb_TV_L2):
            return 0.0
        out = -lamb_TV_L2.sum() * X
        for d in range(3):
            out = out + lamb_TV_L2[d] * (_shift(X, d, -1) + _shift(X, d, +1))
        return out

    def Q(X):
        return backward(forward(X)) + tv(X) + (lamb_L2 * X if lamb_L2 else 0.0)

    X = np.array(df, dtype=np.float64, order="F")
    d = Q(X) - X + lamb_L1
    use_q = bool(np.all(lamb_TV_L1 * lamb_TV_L2 * lamb_L2))
    for _ in range(max_iter):
        passive = (X > 0) | (d < 0)
        d_ = passive * d
        with np.errstate(divide="ignore", invalid="ignore"):
            if use_q:
                alpha = np.sum(d_ * d_) / np.sum(d_ * Q(d_))
            else:
                v = forward(d_)
                alpha = np.sum(d_ * d_) / np.sum(v * v)
        if not np.isfinite(alpha):
            alpha = 0.0
        Xn = X - alpha * d_
        Xn[Xn < 0] = 0.0
        d = d + Q(Xn - X)
        X = Xn
    return X


def reconstruct_S_one(img, forward, backward, opts=None, microlenses=None):
    """One component of reconstruct_S (GPU branch, reconstruct_S.m:168-205;
    the CPU branch :130-148 computes the same): background clip at quantile q
    of the non-microlens pixels, normalise by max then by the L2 norm,
    back-project, cap lamb_L1 by the (1-1e-4) quantile of Htf, solve with
    max_iter iterations, rescale by the norm."""
    opts = dict(opts or {})
    q = opts.get("q", 0.8)
    img = np.asarray(img, dtype=np.float64)
    mask = np.ones(img.shape, dtype=bool) if microlenses is None else (np.asarray(microlenses) == 0)
    img = np.maximum(img - matlab_quantile(img[mask], q), 0.0)
    img = img / img.max()
    nrm = np.sqrt(np.sum(img * img))
    Htf = backward(img / nrm)
    opts["lamb_L1"] = min(matlab_quantile(Htf, 1 - 1e-4), opts.get("lamb_L1", 0.0))
    solver = opts.get("whichSolver", "fast_nnls")
    if solver == "ISRA":
        X = deconvRL(forward, backward, Htf, opts.get("max_iter", 8), Htf, opts)
    elif solver == "fast_nnls":
        X = LS_deconv(forward, backward, Htf, opts)
    else:
        raise ValueError("unknown solver")
    return nrm * X


# ----------------------------------------------------------------------------
# Library generation: generate_LFM_library_GPU.m:63-109
# ----------------------------------------------------------------------------
def library_boxes(centers, image_size, Z, neur_rad, axial):
    """Per-neuron crop box (0-based, inclusive-exclusive) and z window,
    generate_LFM_library_GPU.m:68-88: x = round(center), lateral window
    [max(x-r,1), min(x+r,size)], z window [max(z-ceil(r/axial),1),
    min(z+ceil(r/axial),Z)] (1-based inclusive)."""
    boxes = []
    zr = int(np.ceil(neur_rad / axial))
    for c in np.asarray(centers, dtype=np.float64):
        x, y, z = (int(_mround(v)) for v in c[:3])
        x0, x1 = max(x - neur_rad, 1), min(x + neur_rad, image_size[0])
        y0, y1 = max(y - neur_rad, 1), min(y + neur_rad, image_size[1])
        z0, z1 = max(z - zr, 1), min(z + zr, Z)
        boxes.append((x0 - 1, x1, y0 - 1, y1, z0 - 1, z1))
    return np.asarray(boxes, dtype=np.int64)


def _mround(v):
    """MATLAB round: half away from zero."""
    return np.sign(v) * np.floor(np.abs(v) + 0.5)


def generate_library(recon, centers, neur_id, H, neur_rad, axial, image_size=None):
    """forward_model (n_neurons, X*Y): each row is the forward projection of the
    averaged, cropped reconstructions (generate_LFM_library_GPU.m:63-109)."""
    H = _psf(H)
    Z = H.shape[4]
    X, Y = recon[0].shape[:2] if image_size is None else image_size
    boxes = library_boxes(centers, (X, Y), Z, neur_rad, axial)
    out = np.zeros((len(boxes), X * Y), dtype=np.float64)
    for n, (x0, x1, y0, y1, z0, z1) in enumerate(boxes):
        ids = np.flatnonzero(np.asarray(neur_id)[n])
        vol = np.zeros((X, Y, z1 - z0), dtype=np.float64, order="F")
        for k in ids:
            vol[x0:x1, y0:y1, :] += np.asarray(recon[k], dtype=np.float64)[x0:x1, y0:y1, z0:z1]
        vol = vol / len(ids)
        out[n] = forward_project(H[..., z0:z1], vol).ravel(order="F")
    return out


def library_kernel_shape(r, dim, kernel=None):
    """(W, r, rr) of generate_LFM_library_CPU.m:18,27-36: the given kernel with
    r = (size(W,1)-1)/2, rr = (size(W,3)-1)/2, or the ball
    X.^2 + Y.^2 + (Z*r/rr).^2 <= r^2 over meshgrid(-r:r, -r:r, -rr:rr),
    rr = r/dim(3)."""
    if kernel is not None:
        W = np.asarray(kernel, dtype=np.float32)
        if W.ndim == 2:
            W = W[:, :, None]
        return np.asfortranarray(W), (W.shape[0] - 1) / 2.0, (W.shape[2] - 1) / 2.0
    r = float(r)
    rr = r / float(dim[2])
    xs = np.arange(-r, r + 0.5, 1.0)
    zs = -rr + np.arange(int(np.floor(2 * rr + 1e-10)) + 1, dtype=np.float64)
    X, Y, Z = np.meshgrid(xs, xs, zs)  # MATLAB meshgrid: X along columns, Y along rows
    W = (X ** 2 + Y ** 2 + (Z * r / rr) ** 2 <= r ** 2).astype(np.float32)
    return np.asfortranarray(W), r, rr


def library_kernel_voxels(centers, r, dim, m, Z, kernel=None):
    """Per neuron the 0-based voxels and kernel values generate_LFM_library_CPU.m
    :39-49 paints: bbb = round(BWW - [r+1, r+1, rr+1] + centre) for the nonzero
    kernel entries BWW in find() order, kept inside [1, m(1)] x [1, m(2)] x [1, Z]."""
    W, rk, rr = library_kernel_shape(r, dim, kernel)
    flat = W.ravel(order="F")
    idx = np.flatnonzero(flat != 0)
    i, j, k = np.unravel_index(idx, W.shape, order="F")
    BWW = np.stack([i + 1, j + 1, k + 1], 1).astype(np.float64)
    out = []
    for c in np.asarray(centers, dtype=np.float64).reshape(-1, 3):
        bbb = _mround((BWW - np.array([rk + 1, rk + 1, rr + 1])) + c)
        keep = ((bbb[:, 0] <= m[0]) & (bbb[:, 0] > 0) & (bbb[:, 1] <= m[1]) & (bbb[:, 1] > 0)
                & (bbb[:, 2] <= Z) & (bbb[:, 2] > 0))
        out.append((bbb[keep].astype(np.int64) - 1, flat[idx][keep]))
    return out


def project_forward_patched(pixels, values, dims, Nnum, H):
    """project_forward_patched.m:8-73 in FP64: paint the 1-based voxels into a
    patch of an odd number of lenslets, conv2 'full' every (phase, depth) slice
    with its PSF, paste the result centred on the patch, clipped to the sensor."""
    from scipy.signal import convolve2d
    pixels = np.asarray(pixels, dtype=np.int64)
    N = int(Nnum)
    px_min, px_max = pixels.min(0), pixels.max(0)
    off_ml = (px_min[:2] - 1) // N
    off_px = off_ml * N
    n_ml = -(-px_max[:2] // N) - off_ml
    n_ml = n_ml + (n_ml % 2 == 0)
    off_z = px_min[2] - 1
    n_z = px_max[2] - off_z
    vol = np.zeros((n_ml[0] * N, n_ml[1] * N, n_z))
    for (x, y, z), v in zip(pixels, values):
        vol[x - off_px[0] - 1, y - off_px[1] - 1, z - off_z - 1] = v
    total = None
    for i in range(N):
        for j in range(N):
            for k in range(n_z):
                t = np.zeros(vol.shape[:2])
                t[i::N, j::N] = vol[i::N, j::N, k]
                if not t.any():
                    continue
                c = convolve2d(t, np.asarray(H[:, :, i, j, off_z + k], dtype=np.float64), mode="full")
                total = c if total is None else total + c
    img = np.zeros((int(dims[0]), int(dims[1])))
    if total is None:
        return img
    pj = total.shape
    center = off_px + np.ceil((n_ml / 2.0) * N).astype(np.int64)
    x0, x1 = max(1, center[0] - pj[0] // 2), min(int(dims[0]), center[0] + pj[0] // 2)
    y0, y1 = max(1, center[1] - pj[1] // 2), min(int(dims[1]), center[1] + pj[1] // 2)
    p0, p1 = x0 - (center[0] - pj[0] // 2 - 1), x1 - (center[0] - pj[0] // 2 - 1)
    q0, q1 = y0 - (center[1] - pj[1] // 2 - 1), y1 - (center[1] - pj[1] // 2 - 1)
    img[x0 - 1:x1, y0 - 1:y1] = total[p0 - 1:p1, q0 - 1:q1]
    return img


def generate_library_cpu(centers, H, r, dim, m, kernel=None):
    """forward_model rows of generate_LFM_library_CPU.m:37-54 (dense, FP64):
    each neuron's painted kernel through project_forward_patched, divided by
    its L2 norm."""
    H = _psf(H)
    Z, N = H.shape[4], H.shape[2]
    rows = []
    for vox, vals in library_kernel_voxels(centers, r, dim, m, Z, kernel):
        Q = project_forward_patched(vox + 1, vals.astype(np.float64), m[:2], N, H).ravel(order="F")
        rows.append(Q / np.linalg.norm(Q))
    return np.asarray(rows)


# ----------------------------------------------------------------------------
# NNLS: LS_nnls.m:59-172 and fast_nnls.m:21-199
# ----------------------------------------------------------------------------
def _fit_matrix(sample):
    Xd = np.stack([np.arange(1, 2 * sample, 2, dtype=np.float64), np.ones(sample)], axis=1)
    Xi = np.linalg.inv(Xd.T @ Xd) @ Xd.T
    return Xd, Xi


def LS_nnls(A, Y, opts=None, G=None, x=None, return_iters=False):
    """argmin_{x>=0} ||Y - A x||^2 column-wise by projected gradient with exact
    line search, recomputing the gradient from the Gram each iteration.
    Column retirement follows LS_nnls.m:132-172 verbatim in meaning, including
    its use of the squared column sum of the step and of the first active
    column's slope k(1)."""
    opts = dict(opts or {})
    use_std = opts.get("use_std", False)
    lam = opts.get("lambda", 0.0)
    sample = int(opts.get("sample", 300))
    tol = opts.get("tol", 1e-7)
    tol_ = opts.get("tol_", 1e-2)
    max_iter = int(opts.get("max_iter", 2000))
    A = np.asarray(A, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    F = Y.shape[1]
    h = A.T @ Y - lam
    if G is None:
        G = A.T @ A
    if x is None:
        x = np.zeros((A.shape[1], F))
    x = np.array(x, dtype=np.float64)
    Xout = x.copy()
    rds = np.arange(F)
    if use_std:
        Gm = G
        Gf = lambda v: Gm @ v - (Gm @ v.sum(axis=1, keepdims=True)) / F  # noqa: E731
        h = h - (A.T @ Y.sum(axis=1, keepdims=True)) / F
    else:
        Gf = lambda v: G @ v  # noqa: E731
    dn, Xi = _fit_matrix(sample)
    test = np.zeros((0, F))
    it = 0
    iters = np.zeros(F, dtype=np.int64)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        while x.shape[1] > 0:
            it += 1
            x_ = x.copy()
            df = -h + Gf(x)
            passive = (x > 0) | (df < 0)
            d_ = df * passive
            alpha = np.sum(d_ * d_, axis=0) / np.sum(d_ * Gf(d_), axis=0)
            alpha[np.isnan(alpha)] = 0.0
            x = x - d_ * alpha
            x[x < 0] = 0.0
            ids = None
            if it > max_iter:
                ids = np.ones(x.shape[1], dtype=bool)
            elif not use_std:
                if it % 2 == 1:
                    row = np.log(np.sum(x - x_, axis=0) ** 2 / np.sum(x_ ** 2, axis=0)) / 2
                    test = np.vstack([test, row])
                    if test.shape[0] > sample:
                        test = test[1:]
                    if it > 2 * sample:
                        k = Xi @ test
                        c1 = np.exp(test[-1]) / (1 - np.exp(k[0, 0])) < tol
                        c2 = np.sum(np.abs(dn @ k - test), axis=0) < tol_ * sample
                        c3 = np.exp(k[0]) < 1
                        ids = (c1 & c2 & c3) | (test[-1] == -np.inf)
                    else:
                        ids = np.zeros(x.shape[1], dtype=bool)
            if ids is not None and ids.any():
                Xout[:, rds[ids]] = x[:, ids]
                iters[rds[ids]] = it
                keep = ~ids
                rds, x, h, test = rds[keep], x[:, keep], h[:, keep], test[:, keep]
    if return_iters:
        return Xout, G, iters
    return Xout, G


def fast_nnls(A, Y, opts=None, Q=None, df=None, h=None, return_iters=False):
    """Multi-RHS NNLS on the diagonally normalised Gram with incremental
    gradient updates (fast_nnls.m:53-199), default per-column line search
    (opts.total = 0), log-l1 (tol_p = 1) or log-l2 (tol_p = 2) step test."""
    opts = dict(opts or {})
    tol_p = opts.get("tol_p", 1)
    max_iter = int(opts.get("max_iter", 2000))
    tol = opts.get("tol", 1e-6)
    tol_ = opts.get("tol_", 1e-1)
    sample = int(opts.get("sample", 30))
    warm = opts.get("warm_start", None)
    lam = opts.get("lambda", 0.0)
    total = opts.get("total", 0)
    A = np.asarray(A, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    if Q is None:
        Q = A.T @ A
        dq = np.sqrt(np.diag(Q))
        h = 1.0 / dq
        Q = Q / np.outer(dq, dq)
        df = h[:, None] * (-(A.T @ Y) + lam)
    elif df is None:
        df = h[:, None] * (-(A.T @ Y) + lam)
    df = np.array(df, dtype=np.float64)
    K, F = A.shape[1], Y.shape[1]
    if warm is None or (np.ndim(warm) == 2 and np.size(warm) == 0):
        x = np.zeros((K, F))
    elif np.isscalar(warm) and warm == 1:
        x = np.linalg.inv(Q) @ (-df)
        x[x < 0] = 0.0
        df = df + Q @ x
    else:
        x = np.asarray(warm, dtype=np.float64) / h[:, None]
        df = df + Q @ x
    passive = (x > 0) | (df < 0)
    h_ = np.max(h)
    rds = np.arange(F)
    xx = np.ones((K, F))
    iters = np.zeros(F, dtype=np.int64)
    s = 1
    test = np.zeros((0, F))
    Xd, Xi = _fit_matrix(sample)
    ids = None
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        while x.shape[1] > 0:
            s += 1
            d_ = df * passive
            if total:
                alpha = np.sum(d_ * d_) / np.sum(d_ * (Q @ d_))
                if np.isnan(alpha):
                    alpha = 0.0
                x_ = x - d_ * alpha
                x_[x_ < 0] = 0.0
                df = df + Q @ (x_ - x)
                x = x_
                passive = (x > 0) | (df < 0)
                if s > max_iter:
                    # fast_nnls.m:112-116 breaks without copying x into xx, so
                    # the reference returns diag(h) * ones in total mode
                    iters[rds] = s
                    break
                continue
            alpha = np.sum(d_ * d_, axis=0) / np.sum(d_ * (Q @ d_), axis=0)
            alpha[np.isnan(alpha)] = 0.0
            x_ = x - d_ * alpha
            x_[x_ < 0] = 0.0
            if s % 2 == 1:
                if tol_p == 2:
                    row = np.log(np.sqrt(np.sum((x_ - x) ** 2, axis=0)))
                else:
                    row = np.log(np.sum(np.abs(x_ - x), axis=0))
                test = np.vstack([test, row])
                if test.shape[0] > sample:
                    test = test[1:]
                if s > 2 * sample:
                    k = Xi @ test
                    no_passive = ~passive.any(axis=0)
                    c1 = h_ * np.exp(test[-1]) / (1 - np.exp(k[0])) < tol * x.shape[0] * np.max(x, axis=0)
                    c2 = np.sum(np.abs(Xd @ k - test), axis=0) < tol_ * sample
                    c3 = np.exp(k[0]) < 1
                    ids = no_passive | (c1 & c2 & c3)
                # odd s <= 2*sample keeps ids from the previous (even) step: empty
            else:
                ids = None
            df = df + Q @ (x_ - x)
            if s > max_iter:
                ids = np.ones(x.shape[1], dtype=bool)
            x = x_
            passive = (x > 0) | (df < 0)
            if ids is not None and ids.any():
                xx[:, rds[ids]] = x[:, ids]
                iters[rds[ids]] = s
                keep = ~ids
                rds, x, df, passive, test = rds[keep], x[:, keep], df[:, keep], passive[:, keep], test[:, keep]
    if h is not None:
        xx = h[:, None] * xx
    if return_iters:
        return xx, Q, df, h, iters
    return xx, Q, df, h


# ----------------------------------------------------------------------------
# NMF steps: T_update.m:5-78 and S_update.m:4-80
# ----------------------------------------------------------------------------
def convn_same(V, k):
    """MATLAB convn(V, k, 'same') in FP64: the central part of the full
    convolution, starting at floor(size(k) / 2) along each axis."""
    from scipy.signal import convolve
    V = np.asarray(V, dtype=np.float64)
    k = np.asarray(k, dtype=np.float64)
    k = k.reshape(k.shape + (1,) * (V.ndim - k.ndim))
    full = convolve(V, k, mode="full", method="direct")
    sl = tuple(slice(kn // 2, kn // 2 + vn) for vn, kn in zip(V.shape, k.shape))
    return np.asfortranarray(full[sl])


def merge_filters(forward_model, timeseries, template, indices_in_orig, limit=0.9, bg_sub=True):
    """merge_filters.m:19-50 with MATLAB's types: corrcoef and the overlap
    normalisation in single, the comparisons with 1/3 and 1 + limit in double,
    the two bg_sub crops, and the sequential merge loop."""
    b = 1 if bg_sub else 0
    ts = np.asarray(timeseries, dtype=np.float64)
    K = ts.shape[0]
    corr = (np.corrcoef(ts).astype(np.float32) - np.eye(K, dtype=np.float32))[:K - b, :K - b]
    tp = np.array(template, dtype=np.float32)
    ssum = tp.sum(axis=1, dtype=np.float64).astype(np.float32)
    gram = (tp.astype(np.float64) @ tp.T.astype(np.float64)).astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        ov = (np.float32(1) / np.minimum(ssum[:, None], ssum[None, :])) * gram - np.eye(K - b, dtype=np.float32)
        v = (ov.astype(np.float64) > 1.0 / 3.0).astype(np.float32) + corr
    v = v[:K - 2 * b, :K - 2 * b]
    mat = np.tril(v.astype(np.float64) > 1.0 + limit)
    for ii in np.flatnonzero(mat.sum(axis=0)):
        src = np.flatnonzero(mat[:, ii])
        tp[ii, :] = ((tp[ii, :] + tp[src, :].sum(axis=0)) > 0).astype(np.float32)
        tp[src, :] = 0
    nz = np.flatnonzero(tp.sum(axis=1) > 0)
    rows = np.concatenate([nz, [K - 1]]) if b else nz
    return (np.asarray(forward_model)[rows], ts[rows], tp[nz], np.asarray(indices_in_orig)[rows])


def matlab_smooth(y, span=5):
    """MATLAB smooth(y, span) (moving average): an even span is reduced by one;
    the window shrinks symmetrically at the ends."""
    y = np.asarray(y, dtype=np.float64)
    if span % 2 == 0:
        span -= 1
    n = len(y)
    out = np.empty(n)
    for i in range(n):
        h = min(i, n - 1 - i, span // 2)
        out[i] = y[i - h:i + h + 1].mean()
    return out


def snr_order(traces, bg_sub=True):
    """SNR_order.m:13-28 (0-based order): FFT of [trace flip(trace)], bins 1..6
    and their mirrors zeroed, inverse (real part), first half, zscore; ratio of
    the range of smooth(., 5) to std(smooth(., 8) - .); sorted by decreasing
    ratio (stable), the background row last."""
    tr = np.asarray(traces, dtype=np.float64)
    K = tr.shape[0]
    b = 1 if bg_sub else 0
    pp = np.empty(K - b)
    for k in range(K - b):
        x = tr[k]
        hh = np.fft.fft(np.concatenate([x, x[::-1]]))
        hh[1:7] = 0
        hh[-6:] = 0
        t = np.real(np.fft.ifft(hh))[:len(x)]
        t = (t - t.mean()) / t.std(ddof=1)
        sn = np.std(matlab_smooth(t, 8) - t, ddof=1)
        sm = matlab_smooth(t)
        pp[k] = (sm.max() - sm.min()) / sn
    order = np.argsort(-pp, kind="stable")
    return (np.concatenate([order, [K - 1]]) if b else order), pp


def _colon(a, step, b):
    """MATLAB a:step:b."""
    if step == 0 or (step > 0 and a > b) or (step < 0 and a < b):
        return np.zeros(0)
    n = int(np.floor((b - a) / step + 1e-10)) + 1
    return a + step * np.arange(n)


def image_rect(img, xCenter, yCenter, dx, M, crop=True, cuts=(0, 0, 0, 0)):
    """ImageRect.m:7-45 in FP64: the resample grid (MATLAB colon steps dx/M
    around the centre, started on a lenslet boundary, trimmed to whole
    lenslets, cropped by cuts = XcutLeft, XcutRight, YcutUp, YcutDown) and
    interp2's bilinear rule, NaN outside the image."""
    img = np.asarray(img, dtype=np.float64)
    rows, cols = img.shape
    s = dx / M

    def axis(c, size):
        lo = _colon(c + 1, -s, 1.0)
        hi = _colon(c + 1 + s, s, float(size))
        allv = np.concatenate([lo[::-1], hi])
        centre = len(lo) - M // 2
        init = centre - M * int(np.floor(centre / M)) + M
        return allv[init - 1:], init

    xq, xi = axis(xCenter, cols)
    yq, yi = axis(yCenter, rows)
    nr = M * int(np.floor((len(yq) - yi) / M))
    nc = M * int(np.floor((len(xq) - xi) / M))
    xq, yq = xq[:nc], yq[:nr]
    if crop:
        xs, ys = nc // M, nr // M
        xq = xq[cuts[0] * M:(xs - cuts[1]) * M]
        yq = yq[cuts[2] * M:(ys - cuts[3]) * M]
    out = np.full((len(yq), len(xq)), np.nan)
    for r, y in enumerate(yq):
        if not (1 <= y <= rows):
            continue
        iy = min(int(np.floor(y)), rows - 1)
        fy = y - iy
        for c, x in enumerate(xq):
            if not (1 <= x <= cols):
                continue
            ix = min(int(np.floor(x)), cols - 1)
            fx = x - ix
            v00, v10 = img[iy - 1, ix - 1], img[iy - 1, ix]
            v01, v11 = img[iy, ix - 1], img[iy, ix]
            out[r, c] = (1 - fy) * ((1 - fx) * v00 + fx * v10) + fy * ((1 - fx) * v01 + fx * v11)
    return out


def rank_1_factorization(Y, maxIter=1):
    """[bg_spatial, bg_temporal] = rank_1_factorization(Y, maxIter)
    (rank_1_factorization.m:30-39): alternate t = s'Y / ||.||, s = Y t', s
    normalised except after the last iteration; s starts at ones/sqrt(P)."""
    Y = np.asarray(Y, dtype=np.float64)
    s = np.ones(Y.shape[0]) / np.sqrt(Y.shape[0])
    t = None
    for it in range(1, int(maxIter) + 1):
        t = s @ Y
        t = t / np.linalg.norm(t)
        s = Y @ t
        if it < maxIter:
            s = s / np.linalg.norm(s)
    return s, t


def compute_std_image(Y, y_1=None, y_2=None):
    """compute_std_image.m:17-26: sqrt((A - y1.^2)/F - B.^2 + 2 B.*y1*C -
    y1.^2*C^2) with A = sum(Y.^2, 2), B = mean(Y, 2), C = mean(y2); a negative
    value (rounding) gives 0 where MATLAB would return a complex root."""
    Y = np.asarray(Y, dtype=np.float64)
    P, F = Y.shape
    y1 = np.zeros(P) if y_1 is None else np.asarray(y_1, dtype=np.float64).reshape(-1)
    y2 = np.zeros(F) if y_2 is None else np.asarray(y_2, dtype=np.float64).reshape(-1)
    A = np.sum(Y ** 2, axis=1)
    B = Y.mean(axis=1)
    C = y2.mean()
    v = (A - y1 ** 2) / len(y2) - B ** 2 + 2 * B * y1 * C - y1 ** 2 * C ** 2
    return np.sqrt(np.maximum(v, 0.0))


def _matlab_zscore(T):
    """MATLAB zscore(T): along the first non-singleton dimension (columns of
    an R x F matrix with R > 1), N-1 normalisation, a zero standard deviation
    replaced by 1."""
    ax = 0 if T.shape[0] > 1 else 1
    mu = T.mean(axis=ax, keepdims=True)
    sd = T.std(axis=ax, ddof=1, keepdims=True)
    sd[sd == 0] = 1.0
    return (T - mu) / sd


def T_update(Y, T, S, opts):
    """One projected-gradient step on T with exact line search."""
    Y = np.asarray(Y, dtype=np.float64)
    T = np.nan_to_num(np.array(T, dtype=np.float64), nan=0.0)
    S = np.nan_to_num(np.array(S, dtype=np.float64), nan=0.0)
    lamb_corr = opts.get("lamb_corr", 0.0)
    active = np.asarray(opts.get("active", np.ones(Y.shape[0], dtype=bool)), dtype=bool).ravel()
    if lamb_corr > 0:
        for u in range(T.shape[0]):
            platz = np.linalg.norm(T[u])
            T[u] /= platz
            S[:, u] *= platz
    Sa = S[active]
    Q_S = Sa.T @ Sa
    q_T = Sa.T @ Y[active]
    F = T.shape[1]
    if opts.get("use_std", False):
        Qf = lambda v: Q_S @ v - (Q_S @ v.sum(axis=1, keepdims=True)) / F  # noqa: E731
        q_T = q_T - (Sa.T @ np.asarray(opts["Y"], dtype=np.float64)[active].reshape(-1, 1)) / F
    else:
        Qf = lambda v: Q_S @ v  # noqa: E731
    lamb_temp = opts.get("lamb_temp", 0.0)
    if lamb_corr:
        zsc = _matlab_zscore(T)  # T_update.m:38
        d = T.std(axis=1, ddof=1)
        hilf = (zsc @ zsc.T) @ zsc - zsc
        hilf = (1.0 / d)[:, None] * (hilf - (hilf.sum(axis=1, keepdims=True) * np.ones_like(T)) / F
                                     - (np.diag(hilf @ zsc.T)[:, None] * zsc) / F)
        df = -q_T + Qf(T) + lamb_temp + lamb_corr * hilf
    else:
        df = -q_T + Qf(T) + lamb_temp
    lamb_temp_TV = opts.get("lamb_temp_TV", 0.0)
    if lamb_temp_TV:
        pad = np.zeros((T.shape[0], F + 2))
        pad[:, 1:-1] = T
        pad[:, 0] = T[:, 1]
        pad[:, -1] = T[:, -2]
        tv = -pad[:, :-2] + 2 * pad[:, 1:-1] - pad[:, 2:]
        df = df + lamb_temp_TV * tv
    passive = (T > 0) | (df < 0)
    d_ = passive * df
    with np.errstate(divide="ignore", invalid="ignore"):
        if opts.get("pointwise", False):
            alpha = np.sum(d_ * d_, axis=0) / np.sum(d_ * Qf(d_), axis=0)
        else:
            alpha = np.array(np.sum(d_ * d_) / np.sum(d_ * Qf(d_)))
    alpha = np.where(np.isfinite(alpha), alpha, 0.0)
    T = T - d_ * alpha
    T[T < 0] = 0.0
    return S, T


def S_update(Y, S, T, opts):
    """One projected-gradient step on S with exact line search (spatial TV is
    not supported: the reference reads an undefined `laplace` there)."""
    Y = np.asarray(Y, dtype=np.float64)
    T = np.nan_to_num(np.array(T, dtype=np.float64), nan=0.0)
    S = np.nan_to_num(np.array(S, dtype=np.float64), nan=0.0)
    Q_T = T @ T.T
    q_S = Y @ T.T
    F = T.shape[1]
    if opts.get("use_std", False):
        tsum = T.sum(axis=1)
        Q_T = Q_T - np.outer(tsum, tsum) / F
        q_S = q_S - np.asarray(opts["Y"], dtype=np.float64).reshape(-1, 1) * tsum[None, :] / F
    l1o = opts.get("lamb_orth_L1", 0.0)
    l2o = opts.get("lamb_orth_L2", 0.0)
    if l1o:
        Q_T = Q_T + l1o * np.asarray(opts["hilf"], dtype=np.float64)
    if opts.get("lamb_spat_TV", 0.0):
        raise ValueError("S_update: lamb_spat_TV uses an undefined filter in the reference")
    df = -q_S + S @ Q_T + opts.get("lamb_spat", 0.0)
    if l1o + l2o > 0:
        if l2o:
            v = df + l2o * (S @ (np.asarray(opts["hilf"], dtype=np.float64) @ (S.T @ S)))
        else:
            v = df
        z = np.sum(S * v, axis=1, keepdims=True)
        v = v - S * z
        passive = (S > 0) | (v < 0)
        v = passive * v
    else:
        passive = (S > 0) | (df < 0)
        v = passive * df
    with np.errstate(divide="ignore", invalid="ignore"):
        if opts.get("pointwise", False):
            alpha = (np.sum(v * df, axis=1) / np.sum(v * (v @ Q_T), axis=1))[:, None]
        else:
            alpha = np.array(np.sum(v * df) / np.sum(v * (v @ Q_T)))
            if l2o != 0:
                alpha = np.fmax(alpha, 1e-6)  # MATLAB max ignores NaN (S_update.m:63)
    alpha = np.where(np.isfinite(alpha), alpha, 0.0)
    S = S - alpha * v
    S[S < 0] = 0.0
    if l1o + l2o > 0:
        platz = np.sqrt(np.sum(S * S, axis=0))
        T = platz[:, None] * T
        S = S / platz[None, :]
    return S, T


# ----------------------------------------------------------------------------
# Spatial NNLS: reg_nnls.m:40-69, NQP.m (in C), update_spatial_component.m:45-131
# ----------------------------------------------------------------------------
def NQP(Q, b):
    """argmin_{x>=0} 0.5 x'Qx + b'x (Lawson-Hanson, default options)."""
    Q = np.asfortranarray(Q, dtype=np.float64)
    b = np.ascontiguousarray(np.ravel(b), dtype=np.float64)
    n = b.size
    x = np.zeros(n)
    w = np.zeros(n)
    it = np.zeros(1, dtype=np.int64)
    rc = _lib().oracle_nqp(_ptr(Q), _ptr(b), n, _ptr(x), _ptr(w), _ptr(it))
    if rc != 0:
        raise RuntimeError(f"nnls Failed to converge in {int(it[0])} iterations")
    return x, w, int(it[0])


def reg_nnls(A, d, opts=None):
    """Regularised NNLS reduced to an NQP (reg_nnls.m:40-69)."""
    opts = dict(opts or {})
    A = np.asarray(A, dtype=np.float64)
    d = np.asarray(d, dtype=np.float64).reshape(A.shape[0], -1)
    n = A.shape[1]
    hilf = opts.get("hilf")
    if hilf is None:
        hilf = np.ones((n, n)) - np.eye(n)
        if opts.get("bg_sub", 0):
            hilf[:, -1] = 0
            hilf[-1, :] = 0
    Q = A.T @ A
    q = -(A.T @ d)
    if opts.get("use_std", False):
        tt = A.sum(axis=0)
        Q = Q - np.outer(tt, tt) / A.shape[0]
        q = q + tt[:, None] * d.sum(axis=0)[None, :] / A.shape[0]
    if opts.get("lamb_L1", 0):
        q = q + opts["lamb_L1"]
    if opts.get("lamb_L2", 0):
        Q = Q + opts["lamb_L2"] * np.eye(n)
    if opts.get("lamb_orth_L1", 0):
        Q = Q + opts["lamb_orth_L1"] * hilf
    x, _, _ = NQP(Q, q[:, 0])
    return x


def update_spatial_component(timeseries, sensor_movie, template, opts=None):
    """Per-neuron, per-pixel regularised NNLS over the template support
    (update_spatial_component.m:45-131).  Returns the dense forward model
    (n_components, P)."""
    opts = dict(opts or {})
    bg_sub = opts.get("bg_sub", 1)
    T = np.asarray(timeseries, dtype=np.float64)
    Ymov = np.asarray(sensor_movie, dtype=np.float64)
    tmpl = np.array(template, dtype=bool)
    order = np.argsort(tmpl.sum(axis=1), kind="stable")
    outside = ~tmpl.any(axis=0)
    out = np.zeros((T.shape[0], Ymov.shape[0]))
    for neuron in order:
        space = np.flatnonzero(tmpl[neuron])
        if space.size == 0:
            continue
        involved = np.flatnonzero(tmpl[:, space].any(axis=1))
        if bg_sub:
            temp = np.vstack([tmpl[np.ix_(involved, space)], np.ones((1, space.size), dtype=bool)])
            involved = np.append(involved, T.shape[0] - 1)
        else:
            temp = tmpl[np.ix_(involved, space)]
        A = T[involved].T
        Fm = np.zeros((involved.size, space.size))
        for k_ in range(space.size):
            idx = np.flatnonzero(temp[:, k_])
            y = Ymov[space[k_]]
            nrm = np.linalg.norm(y)
            if nrm > 0:
                Fm[idx, k_] = reg_nnls(A[:, idx], y / nrm, opts) * nrm
        tmpl[:, space] = False
        nz = np.nonzero(Fm)
        out[involved[nz[0]], space[nz[1]]] = Fm[nz]
    if bg_sub and outside.any():
        out[-1, outside] = Ymov[outside] @ T[-1]
    return out


# ----------------------------------------------------------------------------
# Timeseries extraction: incremental_temporal_update_gpu.m:76-100 (LS branch)
# ----------------------------------------------------------------------------
def pinv_extract(forward_model, chunks):
    """Q = inv(F F') F once, then Q * chunk for each chunk of frames."""
    Fm = np.asarray(forward_model, dtype=np.float64)
    Q = np.linalg.inv(Fm @ Fm.T) @ Fm
    return [Q @ np.asarray(c, dtype=np.float64) for c in chunks]
