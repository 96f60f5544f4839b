"""ctypes binding of the native C ABI (``include/nanopyx_gb300.h``).

The library is the only compute path of this package: if it is missing or
cannot be loaded, every op raises ``NativeLibraryError`` -- there is no CPU
fallback.  Build it with ``python -m nanopyx_gb300._build`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

NX_OK = 0
NX_ERR_INVALID_ARG = -1
NX_ERR_UNSUPPORTED = -2
NX_ERR_OUT_OF_MEMORY = -3
NX_ERR_CUDA = -4
NX_ERR_DEVICE_TIMEOUT = -5
NX_ERR_WORKSPACE = -6
NX_ERR_INDEX = -7

NX_CORR_AVG = 1
NX_CORR_VAR = 2
NX_CORR_TAC2 = 4

CORR_BITS = {"AVG": NX_CORR_AVG, "VAR": NX_CORR_VAR, "TAC2": NX_CORR_TAC2}


class EsrrfItem(C.Structure):
    """nx_esrrf_item of include/nanopyx_gb300.h."""

    _fields_ = [("plan", C.c_void_p), ("d_in", C.c_void_p), ("T", C.c_int),
                ("frames_per_timepoint", C.c_int), ("corr_mask", C.c_int),
                ("macro_pixel_correction", C.c_int), ("n_sens", C.c_int),
                ("sens", C.c_float * 4), ("frames_per_unit", C.c_int), ("d_out", C.c_void_p)]


class NativeLibraryError(RuntimeError):
    """The CUDA library is missing or failed to load."""


class DeviceTimeoutError(RuntimeError):
    """A bounded device-side wait ran out; the kernel returned early."""


_P = C.c_void_p
_F = C.POINTER(C.c_float)
_I = C.c_int
_FL = C.c_float
_SZ = C.c_size_t
_LL = C.c_longlong

# name -> (restype, argtypes)
_SIGS = {
    "nx_abi_version": (_I, []),
    "nx_last_error": (C.c_char_p, []),
    "nx_esrrf_plan_create": (_I, [C.POINTER(_P), _I, _I, _I, _FL, _FL, _I]),
    "nx_esrrf_plan_destroy": (_I, [_P]),
    "nx_esrrf_plan_set_tile_variant": (_I, [_P, _I]),
    "nx_esrrf_plan_tile_variant": (_I, [_P]),
    "nx_esrrf_weight_table": (_I, [_I, _FL, _P, _SZ]),
    "nx_esrrf_st_workspace_bytes": (_SZ, [_P, _I]),
    "nx_esrrf_st": (_I, [_P, _P, _I, _P, _P, _SZ, _P]),
    "nx_esrrf_workspace_bytes": (_SZ, [_P, _I, _I, _I]),
    "nx_esrrf_run": (_I, [_P, _P, _I, _I, _I, _I, _P, _P, _SZ, _P]),
    "nx_esrrf_run_stage1": (_I, [_P, _P, _I, _I, _I, _P, _SZ, _P]),
    "nx_esrrf_run_stage2": (_I, [_P, _I, _I, _I, _I, _P, _P, _SZ, _P]),
    "nx_selftest_wait_timeout": (_I, [_P, _SZ, C.c_ulonglong, _P]),
    "nx_selftest_fused_abort": (_I, [_P, _P, _I, _P, _P, _SZ, C.c_ulonglong, _P]),
    "nx_probe_ffma": (_I, [_P, _I, _I, _P]),
    "nx_probe_ffma2": (_I, [_P, _I, _I, _P]),
    "nx_esrrf_accum_bytes": (_SZ, [_P]),
    "nx_esrrf_push_workspace_bytes": (_SZ, [_P, _I]),
    "nx_esrrf_accum_push": (_I, [_P, _P, _I, _I, _P, _P, _SZ, _P]),
    "nx_esrrf_accum_finalize": (_I, [_P, _P, _I, _I, _I, _P, _P, _SZ, _P]),
    "nx_workspace_status": (_I, [_P, _P]),
    "nx_esrrf_batch_create": (_I, [C.POINTER(_P), _P, _I]),
    "nx_esrrf_batch_workspace_bytes": (_SZ, [_P]),
    "nx_esrrf_batch_bind": (_I, [_P, _P, _SZ, _P]),
    "nx_esrrf_batch_launch": (_I, [_P, _P]),
    "nx_esrrf_batch_destroy": (_I, [_P]),
    "nx_cr_shift_magnify": (_I, [_P, _I, _I, _I, _P, _P, _FL, _FL, _P, _P]),
    "nx_roberts_cross": (_I, [_P, _I, _I, _I, _P, _P, _P]),
    "nx_rgc": (_I, [_P, _P, _P, _I, _I, _I, _I, _FL, _FL, _I, _I, _P, _P]),
    "nx_radiality_workspace_bytes": (_SZ, [_I, _I, _I]),
    "nx_radiality": (_I, [_P, _P, _I, _I, _I, _I, _FL, _I, _I, _I, _P, _P, _SZ, _P]),
    "nx_srrf_workspace_bytes": (_SZ, [_I, _I, _I, _I]),
    "nx_srrf": (_I, [_P, _I, _I, _I, _I, _FL, _I, _I, _I, _I, _P, _P, _SZ, _P]),
    "nx_temporal_correlation": (_I, [_P, _I, _LL, _I, _P, _P]),
    "nx_srrf_temporal_correlation": (_I, [_P, _I, _LL, _I, _P, _P]),
    "nx_srrf_acrf_workspace_bytes": (_SZ, [_I, _LL]),
    "nx_srrf_acrf_integrated": (_I, [_P, _I, _LL, _I, _P, _P, _SZ, _P]),
    "nx_fht_plan_create": (_I, [C.POINTER(_P), _I, _I, _I]),
    "nx_fht_plan_create_ex": (_I, [C.POINTER(_P), _I, _I, _I, _I]),
    "nx_fht_plan_destroy": (_I, [_P]),
    "nx_fht_workspace_bytes": (_SZ, [_P, _I]),
    "nx_fht_interpolate": (_I, [_P, _P, _I, _P, _P, _SZ, _P]),
    "nx_esrrf3d_workspace_bytes": (_SZ, [_I, _I, _I, _I, _I, _I]),
    "nx_esrrf3d_st": (_I, [_P, _I, _I, _I, _I, _I, _I, C.c_double, C.c_double, C.c_float, _I, _I,
                           _P, _P, _SZ, _P]),
    "nx_gaussian_blur_workspace_bytes": (_SZ, [_I, _I]),
    "nx_gaussian_blur": (_I, [_P, _I, _I, C.c_double, _I, C.c_float, C.c_float, _P, _P, _SZ, _P]),
    "nx_gaussian_blur_batch_workspace_bytes": (_SZ, [_I, _I, _I]),
    "nx_gaussian_blur_batch": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "nx_gaussian_blur_batch_ex": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _I, _P, _P, _SZ, _P]),
    "nx_decorr_prepare_workspace_bytes": (_SZ, [_I, _I]),
    "nx_decorr_prepare": (_I, [_P, _I, _I, _P, _I, _P, _SZ, _P]),
    "nx_decorr_coefs_workspace_bytes": (_SZ, [_P, _I, _I]),
    "nx_decorr_coefs": (_I, [_P, _P, _P, _I, _I, C.c_float, C.c_float, _I, _P, _P, _P, _SZ, _P]),
    "nx_moment_sums_workspace_bytes": (_SZ, [_I]),
    "nx_moment_sums": (_I, [_P, _P, C.c_longlong, _I, _P, _P, _SZ, _P]),
    "nx_frc_plan_create": (_I, [C.POINTER(_P), _I]),
    "nx_frc_plan_destroy": (_I, [_P]),
    "nx_frc_rings": (_I, [_P]),
    "nx_frc_workspace_bytes": (_SZ, [_P, _I]),
    "nx_frc_ring_sums": (_I, [_P, _P, _P, _I, C.c_longlong, _I, _I, _I, _P, _P, _SZ, _P]),
    "nx_macro_pixel_workspace_bytes": (_SZ, [_I, _I]),
    "nx_macro_pixel_correct": (_I, [_P, _I, _I, _I, _I, _P, _SZ, _P]),
    "nx_macro_pixel_correct_static": (_I, [_P, _I, _I, _I, _I, _P]),
}

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return os.environ.get("NANOPYX_GB300_LIB", _build.LIB)


def lib():
    """Load (once) and return the ctypes library; raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise NativeLibraryError(
                f"native library not found at {path}; build it with "
                "`python -m nanopyx_gb300._build` (nvcc, sm_103a)")
        try:
            h = C.CDLL(path)
        except OSError as e:
            raise NativeLibraryError(f"cannot load {path}: {e}") from e
        for name, (res, args) in _SIGS.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        if h.nx_abi_version() != 1:
            raise NativeLibraryError("native library ABI version mismatch")
        _lib = h
        return _lib


def exported_symbols():
    return list(_SIGS)


def check(rc: int, what: str = "") -> None:
    """Raise the Python exception matching a C-ABI status code."""
    if rc == NX_OK:
        return
    msg = lib().nx_last_error().decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if rc == NX_ERR_INVALID_ARG:
        raise ValueError(text)
    if rc == NX_ERR_OUT_OF_MEMORY:
        raise MemoryError(text)
    if rc == NX_ERR_DEVICE_TIMEOUT:
        raise DeviceTimeoutError(text)
    if rc == NX_ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    if rc == NX_ERR_INDEX:
        raise IndexError(text)
    raise RuntimeError(f"{text} (status {rc})")
