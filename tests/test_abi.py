"""Host-side checks of the C ABI: the library loads, exports every function the
header declares, and rejects bad arguments before touching the GPU."""
import ctypes

import numpy as np
import pytest

from sid_gb300 import _lib


def test_header_lists_functions():
    names = _lib.header_functions()
    assert "sid_plan_create" in names and "sid_forward" in names and "sid_adjoint" in names
    assert len(names) >= 12


def test_library_exports_every_declared_symbol(sidlib):
    missing = [n for n in _lib.header_functions() if not hasattr(sidlib, n)]
    assert not missing, f"declared in include/sid.h but not exported: {missing}"


def test_signatures_cover_header(sidlib):
    assert set(_lib.header_functions()) <= set(_lib.SIGNATURES), \
        set(_lib.header_functions()) - set(_lib.SIGNATURES)


def test_version(sidlib):
    assert sidlib.sid_version() >= 10000


@pytest.mark.parametrize("M,N,Z,X,Y", [(0, 3, 2, 9, 9), (9, 0, 2, 9, 9), (9, 3, 0, 9, 9), (9, 3, 2, 0, 9),
                                       (9, 33, 2, 9, 9)])
def test_plan_create_rejects_bad_sizes(sidlib, M, N, Z, X, Y):
    H = np.ones(max(1, M * M * N * N * Z), dtype=np.float32)
    plan = ctypes.c_void_p()
    rc = sidlib.sid_plan_create(H.ctypes.data, M, N, Z, None, X, Y, _lib.PLAN_DIRECT, ctypes.byref(plan))
    assert rc == _lib.SID_EINVAL
    assert plan.value is None
    assert sidlib.sid_last_error()


def test_plan_create_rejects_bad_caindex(sidlib):
    M, N, Z = 9, 3, 2
    H = np.ones(M * M * N * N * Z, dtype=np.float32)
    ca = np.asfortranarray(np.array([[1, 9], [0, 9]], dtype=np.int32))  # 0 is out of range
    plan = ctypes.c_void_p()
    rc = sidlib.sid_plan_create(H.ctypes.data, M, N, Z, ca.ctypes.data, 9, 9, _lib.PLAN_DIRECT, ctypes.byref(plan))
    assert rc == _lib.SID_EINVAL
    assert b"CAindex" in sidlib.sid_last_error()


def test_null_arguments_rejected(sidlib):
    rc = sidlib.sid_forward(None, 0, None, None, None)
    assert rc == _lib.SID_EINVAL
    rc = sidlib.sid_plan_create(None, 9, 3, 2, None, 9, 9, 1, None)
    assert rc == _lib.SID_EINVAL


def test_destroy_null_is_ok(sidlib):
    assert sidlib.sid_plan_destroy(None) == 0


_NO_STATUS = {"sid_version", "sid_last_error", "sid_plan_destroy", "sid_ctx_destroy", "sid_pinv_destroy",
              "sid_ls_nnls_defaults", "sid_fast_nnls_defaults", "sid_nmf_defaults", "sid_recon_defaults"}


def test_every_entry_point_rejects_null_arguments(sidlib):
    """Every computing entry point the header declares checks its pointers and
    sizes first: all-NULL / zero arguments give SID_EINVAL and a message, with
    no CUDA call (this machine has no GPU)."""
    names = [n for n in _lib.header_functions() if n not in _NO_STATUS]
    assert len(names) >= 30
    for name in names:
        args = []
        for t in _lib.SIGNATURES[name]:
            if t in (ctypes.c_double, ctypes.c_float):
                args.append(0.0)
            elif t in (ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.c_long, ctypes.c_longlong,
                       ctypes.c_uint32):
                args.append(0)
            else:
                args.append(None)
        rc = getattr(sidlib, name)(*args)
        assert rc == _lib.SID_EINVAL, (name, rc)
        assert sidlib.sid_last_error(), name


def test_projector_mirror_checks_sizes_before_calling_libsid():
    """The Python mirror refuses host arrays of the wrong element count before
    any libsid call (the C side reads exactly the plan's volume or image)."""
    from sid_gb300.lfm import Projector
    P = Projector.__new__(Projector)  # geometry only: no plan, so any libsid call would fail differently
    P.X, P.Y, P.Z, P.default_method = 6, 5, 3, "direct"
    vol, img = np.zeros((6, 5, 3), np.float32), np.zeros((6, 5), np.float32)
    P._need("t", "v", vol)
    P._need("t", "i", img)
    with pytest.raises(ValueError, match="volume"):
        P.forward_host(np.zeros((6, 5, 2), np.float32))
    with pytest.raises(ValueError, match="image"):
        P.adjoint_host(np.zeros((5, 5), np.float32))
    with pytest.raises(ValueError, match="volume"):
        P.isra_host(vol, np.zeros((6, 5, 4), np.float32), 1)
