"""ctypes binding of libscir_gb300.so (the C ABI declared in include/scir_gb300.h).

The library is built in-tree by ``scir_gb300.build``.  Loading never falls
back to anything: a missing library raises ``NativeLibraryError``.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_i64 = ctypes.c_int64
_int = ctypes.c_int
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_dp = ctypes.c_void_p  # double* / float* passed as raw addresses

# name -> (restype, argtypes); the C-ABI contract, one entry per SCIR_API symbol
SIGNATURES = {
    "scir_abi_version": (_int, []),
    "scir_status_string": (ctypes.c_char_p, [_int]),
    "scir_last_error": (_int, [ctypes.c_char_p, _sz]),
    "scir_init": (_int, [_int]),
    "scir_device_count": (_int, [ctypes.POINTER(_int)]),
    "scir_device_errors": (_int, [ctypes.POINTER(ctypes.c_uint)]),
    "scir_release_scratch": (_int, []),
    "scir_probe_fma_peak": (_int, [_int, ctypes.POINTER(ctypes.c_double)]),
    "scir_selftest_pipeline": (_int, [_vp, _i64, _i64, ctypes.c_longlong, _vp, _vp]),
    "scir_scratch_usage": (_int, [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "scir_fir_out_len": (_i64, [_i64, _i64, _int]),
    "scir_fir_batched_f32": (_int, [_vp, _i64, _i64, _i64, _vp, _i64, _int, _int, _vp, _i64, _vp]),
    "scir_ragged_plan_create": (_int, [_vp, _i64, _int, _int, ctypes.POINTER(_vp)]),
    "scir_ragged_plan_destroy": (_int, [_vp]),
    "scir_ragged_plan_tensor_cores": (_int, [_vp, ctypes.POINTER(_int), ctypes.POINTER(_i64)]),
    "scir_ragged_plan_stats": (_int, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(_i64)]),
    "scir_fir_ragged_f32": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "scir_ragged_plan_autotune": (_int, [_vp, _vp, _vp, _vp, _vp, ctypes.POINTER(_int),
                                         ctypes.POINTER(ctypes.c_double)]),
    "scir_autotune_fir": (_int, [_i64, _i64, _i64, _int, _int, ctypes.POINTER(ctypes.c_double),
                                 ctypes.c_char_p, _sz]),
    "scir_autotune_resample_poly": (_int, [_i64, _i64, _int, _int, _i64,
                                           ctypes.POINTER(ctypes.c_double), ctypes.c_char_p, _sz]),
    "scir_autotune_clear": (_int, []),
    "scir_add_vec_f32": (_int, [_vp, _vp, _vp, _i64, _vp]),
    "scir_add_scalar_f32": (_int, [_vp, ctypes.c_float, _vp, _i64, _vp]),
    "scir_mul_scalar_f32": (_int, [_vp, ctypes.c_float, _vp, _i64, _vp]),
    "scir_resize2d_f32": (_int, [_vp, _i64, _i64, _vp, _i64, _i64, _int, _vp]),
    "scir_graph_capture_begin": (_int, [_vp]),
    "scir_graph_capture_end": (_int, [_vp, ctypes.POINTER(_vp)]),
    "scir_graph_launch": (_int, [_vp, _vp]),
    "scir_graph_destroy": (_int, [_vp]),
    "scir_autotune_save": (_int, [ctypes.c_char_p]),
    "scir_autotune_load": (_int, [ctypes.c_char_p]),
    "scir_upfirdn_out_len": (_i64, [_i64, _i64, _int, _int]),
    "scir_upfirdn_f32": (_int, [_vp, _i64, _i64, _i64, _vp, _i64, _int, _int, _int, _vp, _i64, _vp]),
    "scir_resample_poly_out_len": (_i64, [_i64, _int, _int]),
    "scir_resample_poly_default_taps": (_int, [_int, _int, _int, _vp, _i64, ctypes.POINTER(_i64)]),
    "scir_resample_poly_f32": (_int, [_vp, _i64, _i64, _i64, _int, _int, _vp, _i64, _int, _vp,
                                      _i64, _vp]),
    "scir_sosfilt_f32": (_int, [_vp, _i64, _i64, _i64, _vp, _int, _vp, _vp, _int, _vp, _i64, _vp]),
    "scir_sosfilt_f64": (_int, [_vp, _i64, _i64, _i64, _vp, _int, _vp, _vp, _int, _vp, _i64, _vp]),
    "scir_sosfilt_zi": (_int, [_vp, _int, _vp]),
    "scir_lfilter_f32": (_int, [_vp, _i64, _i64, _i64, _vp, _int, _vp, _int, _vp, _vp, _vp, _i64,
                                _vp]),
    "scir_lfilter_f64": (_int, [_vp, _i64, _i64, _i64, _vp, _int, _vp, _int, _vp, _vp, _vp, _i64,
                                _vp]),
    "scir_lfilter_zi": (_int, [_vp, _int, _vp, _int, _vp]),
    "scir_iirfilter_zpk": (_int, [_int, _int, _int, _vp, ctypes.c_double, ctypes.c_double, _vp, _vp,
                                  _int, _vp, _vp, _vp]),
    "scir_zpk2sos": (_int, [_vp, _int, _vp, _int, ctypes.c_double, _int, _vp, _int, _vp]),
    "scir_iirfilter_sos": (_int, [_int, _int, _int, _vp, ctypes.c_double, ctypes.c_double, _vp, _int,
                                  _vp]),
    "scir_firwin": (_int, [_i64, _vp, _int, _int, ctypes.c_double, _int, _int, ctypes.c_double,
                           _vp]),
    "scir_sosfiltfilt_default_padlen": (_i64, [_vp, _int]),
    "scir_sosfiltfilt_f32": (_int, [_vp, _i64, _i64, _i64, _vp, _int, _int, _i64, _int, _vp, _i64,
                                    _vp]),
    "scir_sosfiltfilt_f64": (_int, [_vp, _i64, _i64, _i64, _vp, _int, _int, _i64, _int, _vp, _i64,
                                    _vp]),
    "scir_sosfiltfilt_f32_noalloc": (_int, [_vp, _i64, _i64, _i64, _vp, _int, _int, _i64, _int,
                                            _vp, _i64, _vp]),
    "scir_fir1d_batched_f32_cuda": (_int, [_vp, _sz, _sz, _vp, _sz, _vp]),
    "scir_host_chunk_plan": (_int, [_i64, _sz, _sz, _i64, _vp, _i64, ctypes.POINTER(_i64)]),
    "scir_fir_batched_f32_host": (_int, [_vp, _i64, _i64, _vp, _i64, _int, _int, _vp]),
    "scir_sosfilt_f64_host": (_int, [_vp, _int, _vp, _sz, _sz, _vp]),
    "scir_filtfilt_f64_host": (_int, [_vp, _int, _vp, _sz, _sz, _vp]),
    "scir_resample_poly_f64_host": (_int, [_vp, _sz, _sz, _sz, _sz, _vp]),
    "scir_resample_poly_f32_host": (_int, [_vp, _i64, _i64, _int, _int, _vp, _i64, _int, _vp]),
}


class NativeLibraryError(RuntimeError):
    """The compiled library is missing or does not export the C ABI."""


_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads (and on first use, builds) the native library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise NativeLibraryError(f"{path} is missing; run scir_gb300.build.build()")
            _build.build()
        try:
            L = ctypes.CDLL(path)
        except OSError as e:  # pragma: no cover - environment specific
            raise NativeLibraryError(f"cannot load {path}: {e}") from e
        for name, (res, args) in SIGNATURES.items():
            try:
                fn = getattr(L, name)
            except AttributeError as e:
                raise NativeLibraryError(f"{path} does not export {name}") from e
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().scir_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def status_string(code: int) -> str:
    return load().scir_status_string(int(code)).decode()
