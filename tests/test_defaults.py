"""The option defaults libsid fills in are the reference's (host only): the
values each MATLAB function assigns to a missing opts field, and struct
layouts that the Python mirrors share with the C header."""
import ctypes

import pytest

from sid_gb300.lfm import ReconOpts
from sid_gb300.nmf import NmfOpts
from sid_gb300.nnls import NnlsOpts


def _filled(sidlib, fn, cls):
    """Fill a cls through fn inside a larger sentinel buffer: the C struct must
    not write past the Python mirror's size."""
    pad = 64
    raw = (ctypes.c_ubyte * (ctypes.sizeof(cls) + pad))(*([0xA5] * (ctypes.sizeof(cls) + pad)))
    getattr(sidlib, fn)(ctypes.byref(raw))
    assert all(b == 0xA5 for b in raw[ctypes.sizeof(cls):]), f"{fn} writes past the {cls.__name__} layout"
    return cls.from_buffer_copy(bytes(raw[:ctypes.sizeof(cls)]))


def test_ls_nnls_defaults(sidlib):
    o = _filled(sidlib, "sid_ls_nnls_defaults", NnlsOpts)
    assert o.use_std == 0            # LS_nnls.m:48
    assert o.lambda_ == 0.0          # LS_nnls.m:52
    assert o.sample == 300           # LS_nnls.m:60
    assert o.tol == pytest.approx(1e-7, rel=0)   # LS_nnls.m:64
    assert o.tol_ == pytest.approx(1e-2, rel=0)  # LS_nnls.m:68
    assert o.max_iter == 2000        # LS_nnls.m:72


def test_fast_nnls_defaults(sidlib):
    o = _filled(sidlib, "sid_fast_nnls_defaults", NnlsOpts)
    assert o.tol_p == 1              # fast_nnls.m:22
    assert o.max_iter == 2000        # fast_nnls.m:30
    assert o.tol == pytest.approx(1e-6, rel=0)   # fast_nnls.m:34 (1e-12 only for the two-argument call, :12-15)
    assert o.tol_ == pytest.approx(1e-1, rel=0)  # fast_nnls.m:38
    assert o.sample == 30            # fast_nnls.m:42
    assert o.lambda_ == 0.0          # fast_nnls.m:50


def test_recon_defaults(sidlib):
    o = _filled(sidlib, "sid_recon_defaults", ReconOpts)
    assert o.lamb_L1 == 0.0          # reconstruct_S.m:66
    assert o.lamb_L2 == 0.0          # reconstruct_S.m:69
    assert o.max_iter == 8           # reconstruct_S.m:72 (and maxIter, :88)
    assert o.solver == 0             # 'fast_nnls', reconstruct_S.m:80
    assert o.q == 0.8                # reconstruct_S.m:92


def test_nmf_defaults_are_off(sidlib):
    """fast_NMF.m:71-107 sets every penalty to 0 and use_std / pointwise to
    false; the orthogonality weights are read only when given."""
    o = _filled(sidlib, "sid_nmf_defaults", NmfOpts)
    for name, _ in NmfOpts._fields_:
        assert getattr(o, name) == 0, name


def test_python_mirrors_start_from_the_c_defaults():
    from sid_gb300.nmf import _nmf_opts
    from sid_gb300.nnls import _opts
    f = _opts("fast_nnls", {"tol": 1e-9})
    assert (f.sample, f.max_iter, f.tol_p, f.tol) == (30, 2000, 1, 1e-9)
    ls = _opts("ls_nnls", {"lambda": 0.5, "use_std": True})
    assert (ls.sample, ls.lambda_, ls.use_std) == (300, 0.5, 1)
    n = _nmf_opts({"lamb_temp": 0.01, "pointwise": 1})
    assert n.lamb_temp == 0.01 and n.pointwise == 1 and n.lamb_spat == 0.0
    with pytest.raises(ValueError):
        _nmf_opts({"lamb_typo": 1.0})
