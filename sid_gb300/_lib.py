"""ctypes binding of libsid.so (the C ABI declared in include/sid.h).

The library is built in-tree by ``sid_gb300.build`` and loaded from
``sid_gb300/_build/libsid.so``.  There is no fallback: if the shared library is
missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsid.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "sid.h")

SID_OK, SID_EINVAL, SID_ENOMEM, SID_ECUDA, SID_ETIMEOUT, SID_ENOCONV, SID_ENOTSUP = 0, -1, -2, -3, -4, -5, -6
PLAN_DIRECT, PLAN_SPECTRAL_F32, PLAN_SPECTRAL_I16, PLAN_SPECTRAL_F24, PLAN_SPECTRAL_TC = 0x1, 0x2, 0x4, 0x8, 0x10
METHODS = {"direct": 0, "spectral_f32": 1, "spectral_i16": 2, "spectral_mixed": 3, "spectral_mixed_f32": 4}
PLAN_FLAG_FOR_METHOD = {"direct": PLAN_DIRECT, "spectral_f32": PLAN_SPECTRAL_F32, "spectral_i16": PLAN_SPECTRAL_I16,
                        "spectral_mixed": PLAN_SPECTRAL_I16 | PLAN_SPECTRAL_F24,
                        "spectral_mixed_f32": PLAN_SPECTRAL_I16 | PLAN_SPECTRAL_F32}

_CODES = {SID_EINVAL: "SID_EINVAL", SID_ENOMEM: "SID_ENOMEM", SID_ECUDA: "SID_ECUDA",
          SID_ETIMEOUT: "SID_ETIMEOUT", SID_ENOCONV: "SID_ENOCONV", SID_ENOTSUP: "SID_ENOTSUP"}


class SidError(RuntimeError):
    """A libsid call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"{_CODES.get(code, code)}: {msg}")
        self.code = code


P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int
F32 = ctypes.c_float
F64 = ctypes.c_double
PP = ctypes.POINTER(ctypes.c_void_p)

# name -> argtypes; restype is int unless listed in _RESTYPES
SIGNATURES = {
    "sid_last_error": [],
    "sid_version": [],
    "sid_plan_create": [P, I64, I64, I64, P, I64, I64, I32, PP],
    "sid_plan_destroy": [P],
    "sid_plan_info": [P, P],
    "sid_plan_release_workspaces": [P],
    "sid_plan_set_weak_fraction": [P, ctypes.c_double],
    "sid_plan_set_kernel": [P, P, I64, I64, I64],
    "sid_forward": [P, I32, P, P, P],
    "sid_adjoint": [P, I32, P, P, P],
    "sid_forward_host": [P, I32, P, P],
    "sid_adjoint_host": [P, I32, P, P],
    "sid_plan_sync": [P, P],
    "sid_deconv_isra": [P, I32, P, P, I32, F32, P],
    "sid_deconv_ls": [P, I32, P, I32, F32, F32, P],
    "sid_deconv_isra_ex": [P, I32, P, P, I32, I32, I32, P, P, P],
    "sid_forward_batched": [P, I32, I64, P, P, P],
    "sid_adjoint_batched": [P, I32, I64, P, P, P],
    "sid_deconv_isra_batched": [P, I32, I64, P, P, I32, F32, P],
    "sid_deconv_ls_batched": [P, I32, I64, P, I32, P, F32, P],
    "sid_reconstruct_components": [P, I32, I64, P, P, P, P, P, P],
    "sid_deconv_ls_ex": [P, I32, P, I32, F32, F32, P, F32, P],
    "sid_deconv_isra_host": [P, I32, P, P, I32, F32],
    "sid_deconv_rl_poisson": [P, I32, P, P, I32, P],
    "sid_plan_timing_enable": [P, I32],
    "sid_plan_timing_read": [P, P, P],
    "sid_ctx_create": [PP],
    "sid_ctx_destroy": [P],
    "sid_ctx_sync": [P, P],
    "sid_gram": [P, P, I64, I64, P, I32, P],
    "sid_rank1_background": [P, P, I32, I64, I64, I32, P, P, P, P],
    "sid_std_image": [P, P, I32, I64, I64, P, P, P, P],
    "sid_merge_filters": [P, P, I64, I64, P, I64, ctypes.c_double, I32, P, P],
    "sid_snr_order": [P, P, I64, I64, I32, P, P],
    "sid_image_rect_size": [I64, I64, ctypes.c_double, ctypes.c_double, ctypes.c_double, I64, I32, P, P, P],
    "sid_image_rect": [P, P, I32, I64, I64, I64, P, ctypes.c_double, ctypes.c_double, ctypes.c_double, I64, I32, P,
                       P, P],
    "sid_cross": [P, P, P, I32, I64, I64, I64, P, I32, P],
    "sid_ls_nnls_defaults": [P],
    "sid_fast_nnls_defaults": [P],
    "sid_ls_nnls": [P, P, P, I32, I64, I64, I64, P, P, I32, P, I32, I32, P, P],
    "sid_fast_nnls": [P, P, P, I32, I64, I64, I64, P, P, P, P, I32, P, P],
    "sid_fast_nnls_ex": [P, P, P, I32, I64, I64, I64, P, I32, I32, P, P, P, P, P, P, P, P, I32, P, P],
    "sid_gram_noalloc": [P, I64, I64, P, P],
    "sid_selftest_wait_timeout": [ctypes.c_uint32, I32],
    "sid_library": [P, P, I64, P, P, I64, I64, F64, P, I32, P],
    "sid_library_spectral": [P, P, I64, P, P, I64, I64, F64, P, I32, P],
    "sid_ctx_timing_enable": [P, I32],
    "sid_gemm_tile_plan": [I64, I64, I64, I32, I32, P, P],
    "sid_weak_runs_plan": [P, I64, I64, I64, I64, P, I64, P, P],
    "sid_ctx_timing_read": [P, P, P],
    "sid_library_kernel": [P, I32, P, I64, F64, F64, P, I64, I64, I64, P, I32, P],
    "sid_library_kernel_voxels": [P, I64, F64, F64, P, I64, I64, I64, I64, I64, I64, P, P, P, I64],
    "sid_library_boxes": [P, I64, I64, F64, I64, I64, I64, P],
    "sid_spatial_update": [P, P, P, I32, P, I64, I64, I64, F64, F64, F64, I32, I32, P, P, P],
    "sid_nqp_batched": [P, P, P, I32, I64, P, P, P, P, P],
    "sid_reg_nnls": [P, P, I64, I32, P, F64, F64, F64, I32, I32, P, P, P],
    "sid_nmf_defaults": [P],
    "sid_t_update": [P, P, I32, P, P, I64, I64, I64, P, P, P, I32, P],
    "sid_s_update": [P, P, I32, P, P, I64, I64, I64, P, P, P, I32, P],
    "sid_pinv_create": [P, P, I64, I64, I32, I32, PP, P],
    "sid_pinv_apply": [P, P, I32, I64, P, P, I64, P],
    "sid_pinv_destroy": [P],
    "sid_quantile": [P, P, I64, P, P, I32, P, P],
    "sid_recon_defaults": [P],
    "sid_reconstruct_component": [P, I32, P, P, P, P, P, P],
}
PREC = {"fp32": 0, "split": 1, "bf16": 2}
DTYPE_F32, DTYPE_F16 = 0, 1
_RESTYPES = {"sid_last_error": ctypes.c_char_p, "sid_ls_nnls_defaults": None,
             "sid_fast_nnls_defaults": None, "sid_nmf_defaults": None,
             "sid_recon_defaults": None}

_lib = None


def header_functions(path: str = HEADER):
    """Names of the functions declared in include/sid.h."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(sid_\w+)\s*\(", text, flags=re.M)))


def load(path: str = LIB_PATH):
    """Load libsid.so and attach signatures (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libsid.so not built ({path}); run sid_gb300.build.build() first")
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, ctypes.c_int)
    _lib = lib
    return lib


def check(rc: int, what: str):
    if rc != SID_OK:
        msg = load().sid_last_error()
        raise SidError(rc, f"{what}: {msg.decode() if msg else ''}")


def call(name: str, *args):
    rc = getattr(load(), name)(*args)
    check(rc, name)
    return rc
