"""ctypes binding of libbbdg.so, the C-ABI CUDA library declared in include/bbdg.h.

There is no fallback: if the library is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

BB_OK, BB_ERR_ARG, BB_ERR_CUDA, BB_ERR_TIMEOUT, BB_ERR_NONFINITE, BB_ERR_STATE, \
    BB_ERR_NOMEM, BB_ERR_DEVICE = range(8)
BB_F32, BB_F64 = 0, 1
BB_WAVE, BB_MAXWELL, BB_ADVECTION, BB_ADVECTION3 = 0, 1, 2, 3
GEO_STRIDE = 24

_STATUS_NAMES = {0: "BB_OK", 1: "BB_ERR_ARG", 2: "BB_ERR_CUDA", 3: "BB_ERR_TIMEOUT",
                 4: "BB_ERR_NONFINITE", 5: "BB_ERR_STATE", 6: "BB_ERR_NOMEM",
                 7: "BB_ERR_DEVICE"}


class BBError(RuntimeError):
    """A libbbdg call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")


_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double

# name -> (restype, argtypes); mirrors include/bbdg.h
SIGNATURES = {
    "bb_version": (_I, []),
    "bb_ctx_create": (_I, [_I, ctypes.POINTER(_P)]),
    "bb_ctx_destroy": (_I, [_P]),
    "bb_ctx_last_error": (ctypes.c_char_p, [_P]),
    "bb_ctx_launch_count": (_I64, [_P]),
    "bb_deriv_apply": (_I, [_P, _I, _I, _I64, _I, _P, _P, _P]),
    "bb_grad_apply": (_I, [_P, _I, _I64, _I, _P, _P, _P, _P, _P]),
    "bb_lift_apply": (_I, [_P, _I, _I64, _I, _P, _P, _P]),
    "bb_face_lift_apply": (_I, [_P, _I, _I64, _I, _P, _P, _P]),
    "bb_elevation_apply": (_I, [_P, _I, _I64, _I, _P, _P, _P]),
    "bb_reduction_apply": (_I, [_P, _I, _I64, _I, _P, _P, _P]),
    "bb_fused_apply": (_I, [_P, _I, _I64, _I, _P, _P, _P, _P, _P, _P, _P]),
    "bb_solver_create": (_I, [_P, _I, _I, _I64, _I, _P, _P, _D, ctypes.POINTER(_P)]),
    "bb_solver_destroy": (_I, [_P]),
    "bb_solver_set_tile": (_I, [_P, _I, _I]),
    "bb_solver_get_tile": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "bb_solver_set_kernel": (_I, [_P, _I]),
    "bb_solver_get_kernel": (_I, [_P]),
    "bb_fast_variant": (_I, [_I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                             ctypes.POINTER(_I)]),
    "bb_stage_tile_bytes": (_I, [_I, _I, _I, _I, ctypes.POINTER(_I64), ctypes.POINTER(_I)]),
    "bb_rhs": (_I, [_P, _P, _P, _P]),
    "bb_lsrk_run": (_I, [_P, _D, _I, _P, _P, _I, _P]),
    "bb_solver_check": (_I, [_P, _P]),
    "bb_lsrk_run_host": (_I, [_P, _D, _I, _P, _P, _P, _P, _I, _P]),
    "bb_host_schedule": (_I, [_I64, _I, _P, _P, _P, _P, _P, _P, _P]),
    "bb_norms": (_I, [_P, _I, _I64, _I, _I, _P, _P, ctypes.POINTER(_D), _P]),
    "bb_mass_norms": (_I, [_P, _I, _I64, _I, _I, _P, _P, _P, ctypes.POINTER(_D), _P]),
    "bb_norms_noalloc": (_I, [_I, _I64, _I, _I, _P, _P, _P, _P]),
    "bb_project": (_I, [_P, _I, _I, _I64, _I, _I, _P, _I, _P, _P]),
    "bb_conn_from_mapP": (_I, [_I, _I64, _P, _P, _P]),
    "bb_geo_from_meshdata": (_I, [_I64, _I, _P, _P, _P, _P]),
}

class BatchProblem(ctypes.Structure):
    """bb_batch_problem of include/bbdg.h."""
    _fields_ = [("physics", ctypes.c_int), ("N", ctypes.c_int), ("K", ctypes.c_int64),
                ("conn", ctypes.c_void_p), ("geo", ctypes.c_void_p), ("q", ctypes.c_void_p),
                ("res", ctypes.c_void_p), ("dt", ctypes.c_double), ("tau", ctypes.c_double)]


SIGNATURES.update({
    "bb_batch_create": (_I, [_P, _I, ctypes.POINTER(BatchProblem), _I, ctypes.POINTER(_P)]),
    "bb_batch_destroy": (_I, [_P]),
    "bb_batch_set_tile": (_I, [_P, _I, _I, _I]),
    "bb_batch_get_tile": (_I, [_P, _I, _I, ctypes.POINTER(_I)]),
    "bb_batch_run": (_I, [_P, _I, _I, _P]),
    "bb_gemm_bf16": (_I, [_P, _I64, _I, _I, _P, _P, ctypes.c_float, _P, _I, _P, _P, _P, _P, _P,
                          _I, _I, _I, _P]),
    "bb_device_status": (_I, [_P, _P, ctypes.POINTER(_I)]),
    "bb_ctx_set_wait_limit": (_I, [_P, ctypes.c_uint32]),
    "bb_ctx_set_test_fault": (_I, [_P, _I]),
    "bb_transpose_bf16": (_I, [_P, _I64, _I, _P, _P, _P]),
    "bb_mlp_create": (_I, [_P, _I, _I, _I, _I, _I64, ctypes.c_uint64, ctypes.POINTER(_P)]),
    "bb_mlp_destroy": (_I, [_P]),
    "bb_mlp_num_params": (_I64, [_P]),
    "bb_mlp_set_params": (_I, [_P, _P, _P]),
    "bb_mlp_get_params": (_I, [_P, _P, _P]),
    "bb_mlp_get_grads": (_I, [_P, _P, _P]),
    "bb_mlp_fwd": (_I, [_P, _I64, _P, _P, _P, _I, _P]),
    "bb_mlp_bwd": (_I, [_P, _I64, _P, _P, _P, _P]),
    "bb_mlp_step": (_I, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                         _P]),
    "bb_closure_features": (_I, [_P, _I, _I64, _I, _P, _I, _P, ctypes.c_float, _P, _P, _P]),
    "bb_closure_apply": (_I, [_P, _I, _I64, _I, _I, ctypes.c_float, _P, _P, _P]),
})

_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads libbbdg.so (building it first if needed) and binds every entry point."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(_build.LIB):
            raise RuntimeError(f"libbbdg.so not found at {_build.LIB}; run the build first")
        L = ctypes.CDLL(_build.LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return _lib


def check(rc: int, ctx_handle=None, what: str = "") -> None:
    if rc != BB_OK:
        msg = what
        if ctx_handle:
            err = load().bb_ctx_last_error(ctx_handle)
            msg = (what + ": " if what else "") + (err.decode() if err else "")
        raise BBError(rc, msg)
