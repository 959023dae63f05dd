"""ctypes binding of the C ABI declared in ``include/lightprop2d_gb300.h``.

The shared library is built in-tree by ``lightprop2d_gb300.build``.  There is
no fallback: if the library is missing or a call fails, an exception says why.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblightprop2d_gb300.so")

# lp_status codes (include/lightprop2d_gb300.h)
LP_OK = 0
LP_ERR_INVALID_ARGUMENT = 1
LP_ERR_UNSUPPORTED_SIZE = 2
LP_ERR_MISALIGNED = 3
LP_ERR_CUDA = 4
LP_ERR_OUT_OF_MEMORY = 5
LP_ERR_NOT_INITIALIZED = 6
LP_ERR_TIMEOUT = 7

# mask element types
LP_MASK_NONE = 0
LP_MASK_F32 = 1
LP_MASK_C64 = 2
LP_MASK_U8 = 3
LP_MASK_PHASE_F32 = 4
LP_MASK_F64 = 5
LP_MASK_C128 = 6
LP_MASK_SEP_F32 = 7
LP_MASK_SPAN_I32 = 8
LP_MASK_SEP_C64 = 9
LP_MASK_SEP_C128 = 10

# flags
LP_FLAG_PHASE_FP32 = 0x1
LP_FLAG_EVANESCENT_MASK = 0x2
LP_FLAG_ADJOINT = 0x4
LP_FLAG_SPECTRUM_READONLY = 0x8
LP_FLAG_DZ = 0x10
LP_FLAG_XMASK_AFTER = 0x20
LP_FLAG_PLAIN_FP64_H = 0x100

_vp, _i, _d, _u = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint32


class BeamDesc(ctypes.Structure):
    """lp_beam_desc"""
    _fields_ = [("field", ctypes.c_void_p), ("iprofile", ctypes.c_void_p), ("n", ctypes.c_int),
                ("area_size", ctypes.c_double), ("wl", ctypes.c_double), ("z", ctypes.c_double),
                ("lens_f", ctypes.c_double), ("flags", ctypes.c_uint32),
                ("moments", ctypes.c_void_p)]


class BatchOptions(ctypes.Structure):
    """lp_batch_options"""
    _fields_ = [("ctas_per_sm", ctypes.c_int), ("tiles_per_item", ctypes.c_int),
                ("group_points_log2", ctypes.c_int), ("spin_limit", ctypes.c_longlong),
                ("debug_unsatisfiable", ctypes.c_int)]

# name -> argtypes (restype is lp_status = int unless listed in _RESTYPES)
SIGNATURES = {
    "lp_abi_version": [],
    "lp_last_error": [],
    "lp_status_string": [_i],
    "lp_is_supported_n": [_i],
    "lp_init": [_i],
    "lp_workspace_release": [],
    "lp_profile_events": [ctypes.POINTER(ctypes.c_void_p), _i],
    "lp_tune_ctas_per_sm": [_i, _i, _i],
    "lp_async_status": [_vp],
    "lp_fft2": [_vp, _vp, _i, _i, _vp],
    "lp_propagate": [_vp, _vp, _i, _d, _d, _d, _vp, _i, _u, _vp],
    "lp_propagate_field": [_vp, _vp, _vp, _vp, _i, _d, _d, _d, _d, _vp, _i, _vp, _i,
                           _u, _vp],
    "lp_lens": [_vp, _vp, _i, _d, _d, _d, _vp],
    "lp_coordinate_filter": [_vp, _vp, _i, _vp, _i, _vp],
    "lp_spectral_filter": [_vp, _vp, _i, _vp, _i, _vp],
    "lp_iprofile": [_vp, _vp, _i, _vp],
    "lp_beam_moments": [_vp, _i, _vp, _vp],
    "lp_intensity_mse": [_vp, _vp, ctypes.c_longlong, _vp, _vp],
    "lp_intensity_mse_grad": [_vp, _vp, ctypes.c_longlong, _vp, ctypes.c_float, _vp, _vp],
    "lp_phase_grad": [_vp, _vp, ctypes.c_longlong, _vp, _vp],
    "lp_expand": [_vp, _i, _vp, _i, _vp],
    "lp_coarse": [_vp, _i, _vp, _i, _vp],
    "lp_crop": [_vp, _i, _i, _i, _d, _d, _vp, _i, _d, _vp],
    "lp_modes_project": [_vp, _i, _i, _vp, _i, _vp, _vp],
    "lp_modes_combine": [_vp, _i, _i, _vp, _vp, _i, _vp],
    "lp_apply_transfer": [_vp, _i, _d, _d, _d, _u, _vp],
    "lp_fft2_c128": [_vp, _vp, _i, _i, _vp],
    "lp_propagate_c128": [_vp, _vp, _i, _d, _d, _d, _vp, _i, _u, _vp],
    "lp_propagate_field_c128": [_vp, _vp, _vp, _vp, _i, _d, _d, _d, _d, _vp, _i, _vp, _i,
                                _u, _vp],
    "lp_lens_c128": [_vp, _vp, _i, _d, _d, _d, _vp],
    "lp_coordinate_filter_c128": [_vp, _vp, _i, _vp, _i, _vp],
    "lp_spectral_filter_c128": [_vp, _vp, _i, _vp, _i, _vp],
    "lp_apply_transfer_c128": [_vp, _i, _d, _d, _d, _u, _vp],
    "lp_iprofile_c128": [_vp, _vp, _i, _vp],
    "lp_plain_propagate_field": [_vp, _vp, _i, _d, _d, _d, _u, _vp],
    "lp_plain_propagate_field_noalloc": [_vp, _vp, _i, _d, _d, _d, _u, _vp],
    "lp_batch_create": [ctypes.POINTER(BeamDesc), _i, ctypes.POINTER(BatchOptions),
                        ctypes.POINTER(ctypes.c_void_p)],
    "lp_batch_run": [_vp, _vp],
    "lp_batch_status": [_vp, _vp],
    "lp_batch_info": [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)],
    "lp_batch_plan": [ctypes.POINTER(BeamDesc), _i, ctypes.POINTER(BatchOptions),
                      ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_longlong),
                      ctypes.POINTER(ctypes.c_longlong)],
    "lp_batch_destroy": [_vp],
}
_RESTYPES = {"lp_last_error": ctypes.c_char_p, "lp_status_string": ctypes.c_char_p}

_lib = None
_lock = threading.Lock()


class BackendError(RuntimeError):
    """A CUDA-side failure reported by the backend."""


def load():
    """Load the shared library (once) and declare every ABI signature."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import lightprop2d_gb300.build as b; b.build()'` "
                "(the GB300 backend has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = L
        return _lib


def last_error() -> str:
    return load().lp_last_error().decode(errors="replace")


def check(status: int, what: str) -> None:
    """Raise the exception that matches an lp_status (reference-style errors:
    ValueError for bad arguments, RuntimeError for device failures)."""
    if status == LP_OK:
        return
    msg = f"{what}: {load().lp_status_string(status).decode()}: {last_error()}"
    if status in (LP_ERR_INVALID_ARGUMENT, LP_ERR_UNSUPPORTED_SIZE, LP_ERR_MISALIGNED):
        raise ValueError(msg)
    if status == LP_ERR_OUT_OF_MEMORY:
        raise MemoryError(msg)
    raise BackendError(msg)
