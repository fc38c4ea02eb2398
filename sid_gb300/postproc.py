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
