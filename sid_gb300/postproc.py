"""Post-processing of the demixing, mirroring the reference's MATLAB functions:

* ``[forward_model, timeseries, template, indices_in_orig] =
  merge_filters(forward_model, timeseries, template, indices_in_orig, opts)``
  merge_filters.m:1
* ``n = SNR_order(traces, opts)``   SNR_order.m:1 (0-based order here)

Matrices are K x (F or P) with one component per row, MATLAB column-major.
The arithmetic runs in libsid (``sid_merge_filters`` / ``sid_snr_order``);
this module only gathers the surviving rows.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .lfm import _stream_ptr, to_device
from .nnls import _ctx


def merge_filters(forward_model, timeseries, template, indices_in_orig, opts=None):
    """Merge components whose templates overlap by more than a third and whose
    traces correlate above opts.limit (default 0.9); opts.bg_sub (default
    True): the last row is the background, kept and never merged."""
    opts = dict(opts or {})
    limit = float(opts.get("limit", 0.9))
    bg_sub = 1 if opts.get("bg_sub", True) else 0
    ts = to_device(timeseries)
    K, F = ts.shape
    tp = to_device(template).clone()
    Kt, P = tp.shape
    if Kt != K - bg_sub:
        raise ValueError(f"merge_filters: template has {Kt} rows, expected {K - bg_sub}")
    keep = np.zeros(K, dtype=np.int32)
    _lib.call("sid_merge_filters", _ctx()._ctx, ts.data_ptr(), K, F, tp.data_ptr(), P, limit, bg_sub,
              keep.ctypes.data, _stream_ptr())
    rows = np.flatnonzero(keep)
    trows = np.flatnonzero(keep[:Kt])
    ri = torch.as_tensor(rows, device=ts.device)
    fm = to_device(forward_model)
    return (to_device(fm[ri]), to_device(ts[ri]), to_device(tp[torch.as_tensor(trows, device=ts.device)]),
            np.asarray(indices_in_orig)[rows])


def SNR_order(traces, opts=None):
    """Row order by decreasing peak-to-noise ratio (0-based); with opts.bg_sub
    (default 1) the last row is left last."""
    opts = dict(opts or {})
    bg_sub = 1 if opts.get("bg_sub", 1) else 0
    tr = to_device(traces)
    K, F = tr.shape
    order = np.zeros(K, dtype=np.int32)
    _lib.call("sid_snr_order", _ctx()._ctx, tr.data_ptr(), K, F, bg_sub, order.ctypes.data, _stream_ptr())
    return order


def _sensor_movie_means(files, idx, x_offset, y_offset, dx, Nnum, do_rectify, cuts, nfiles):
    """frames.mean (read_sensor_movie.m:65-90): column j of the movie is the
    mean of the rectified frames idx[j] .. idx[j+1] (both ends included, the
    mask not applied, as the reference's branch does), j < len(idx) - 1."""
    from .tiff import read_tiff
    if not do_rectify:
        raise NotImplementedError("read_sensor_movie: frames.mean without rectification (the reference's crop "
                                  "subscript there selects a single column, read_sensor_movie.m:77-79)")
    cols, size = [], None
    for j in range(len(idx) - 1):
        grp = list(range(idx[j], idx[j + 1] + 1))
        imgs = np.stack([read_tiff(files[i - 1]) for i in grp], axis=2)
        mov, (R, C) = rectify_frames(imgs if imgs.dtype == np.uint16 else imgs.astype(np.float32), x_offset, y_offset,
                                     dx, Nnum, True, cuts, None)
        cols.append(mov.mean(dim=1, keepdim=True))
        size = (R, C)
    if not cols:
        raise ValueError("read_sensor_movie: frames.mean needs at least two frame indices")
    movie = to_device(torch.cat(cols, dim=1))
    return movie, (size[0], size[1], nfiles)


def _rect_size(rows, cols, xCenter, yCenter, dx, M, crop, cuts):
    c = np.asarray(cuts, dtype=np.int32)
    r_ = np.zeros(1, dtype=np.int64)
    c_ = np.zeros(1, dtype=np.int64)
    _lib.call("sid_image_rect_size", rows, cols, float(xCenter), float(yCenter), float(dx), int(M), 1 if crop else 0,
              c.ctypes.data, r_.ctypes.data, c_.ctypes.data)
    return int(r_[0]), int(c_[0])


def rectify_frames(frames, xCenter, yCenter, dx, M, crop=True, cuts=(0, 0, 0, 0), mask=None):
    """ImageRect (ImageRect.m:1) of every frame of frames (rows, cols, n) --
    uint16 or single, NumPy or CUDA -- on the GPU, optionally times mask
    (rows, cols).  Returns the (out_rows * out_cols, n) movie as a CUDA tensor."""
    if isinstance(frames, np.ndarray) and frames.dtype == np.uint16:
        # the raw 16-bit words travel as int16 (same bits); the kernel reads them as uint16
        f = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(frames).T).view(np.int16)).to("cuda")
        f = f.permute(*reversed(range(f.dim())))
        dtype = 2
    elif isinstance(frames, torch.Tensor) and frames.dtype == torch.int16:
        raise TypeError("rectify_frames: uint16 frames must be passed as NumPy arrays")
    else:
        f = to_device(frames)
        dtype = 0
    if f.dim() == 2:
        f = f.unsqueeze(2)
    rows, cols, n = f.shape
    R, C = _rect_size(rows, cols, xCenter, yCenter, dx, M, crop, cuts)
    out = torch.empty((n, R * C), device=f.device, dtype=torch.float32).t()
    m = to_device(mask) if mask is not None else None
    c = np.asarray(cuts, dtype=np.int32)
    _lib.call("sid_image_rect", _ctx()._ctx, f.data_ptr(), dtype, rows, cols, n,
              m.data_ptr() if m is not None else None, float(xCenter), float(yCenter), float(dx), int(M),
              1 if crop else 0, c.ctypes.data, out.data_ptr(), _stream_ptr())
    return out, (R, C)


def ImageRect(IMG_BW, xCenter, yCenter, dx, M, Crop=True, XcutLeft=0, XcutRight=0, YcutUp=0, YcutDown=0):
    """IMG_RESAMPLE_crop2 = ImageRect(IMG_BW, xCenter, yCenter, dx, M, Crop, XcutLeft,
    XcutRight, YcutUp, YcutDown) (ImageRect.m:1) on the GPU; a CUDA tensor."""
    out, (R, C) = rectify_frames(IMG_BW, xCenter, yCenter, dx, M, Crop, (XcutLeft, XcutRight, YcutUp, YcutDown))
    return out[:, 0].reshape(C, R).t()


def read_sensor_movie(in_folder, x_offset, y_offset, dx, Nnum, do_rectify=True, frames=None, mask=None,
                      crop_border_microlenses=(0, 0, 0, 0), batch=64):
    """[sensor_movie, movie_size] = read_sensor_movie(in_folder, x_offset, y_offset,
    dx, Nnum, do_rectify, frames, mask, crop_border_microlenses)
    (read_sensor_movie.m:1), the frames.mean = 0 branch (:82-113): the folder's
    *.tif* files in name order, frames.start:frames.step:frames.end (1-based) or
    frames.list, each frame times mask, rectified on the GPU in batches.
    Returns the (P, F) single movie (CUDA) and (rows, cols, n_files)."""
    import glob
    import os
    from .tiff import read_tiff
    files = sorted(glob.glob(os.path.join(in_folder, "*.tif*")), key=os.path.basename)
    nfiles = len(files)
    fr = dict(frames or {})
    if fr.get("list") is not None and len(fr["list"]):
        idx = [int(i) for i in fr["list"] if int(i) <= nfiles]
    else:
        idx = list(range(int(fr.get("start", 1)), min(int(fr.get("end", nfiles)), nfiles) + 1, int(fr.get("step", 1))))
    cuts = tuple(int(c) for c in crop_border_microlenses)
    if fr.get("mean", 0):
        return _sensor_movie_means(files, idx, x_offset, y_offset, dx, Nnum, do_rectify, cuts, nfiles)
    cols_out = []
    size = None
    for b0 in range(0, len(idx), batch):
        imgs = np.stack([read_tiff(files[i - 1]) for i in idx[b0:b0 + batch]], axis=2)
        if do_rectify:
            mov, (R, C) = rectify_frames(imgs if imgs.dtype == np.uint16 else imgs.astype(np.float32), x_offset,
                                         y_offset, dx, Nnum, True, cuts, mask)
        else:
            f = imgs.astype(np.float32) * (np.asarray(mask, dtype=np.float32)[:, :, None] if mask is not None else 1)
            f = f[cuts[0] * Nnum:f.shape[0] - cuts[1] * Nnum, cuts[2] * Nnum:f.shape[1] - cuts[3] * Nnum]
            R, C = f.shape[:2]
            mov = to_device(f.reshape(R * C, -1, order="F"))
        size = (R, C)
        cols_out.append(mov)
    movie = torch.cat(cols_out, dim=1) if len(cols_out) > 1 else cols_out[0]
    movie = to_device(movie)
    return movie, (size[0], size[1], nfiles)
