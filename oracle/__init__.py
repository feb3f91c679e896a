"""CPU oracle for the batched-filtering path (test infrastructure only).

Loads ``oracle/_build/libscir_oracle.so`` (built from ``scir_oracle.c`` by
``oracle/Makefile``) and wraps it with numpy.  Only the test suite, the smoke
check and the CPU-baseline leg of ``bench.py`` use this module; the library
itself never imports it.  Function-by-function citations of the reference
lines each routine restates are in ``scir_oracle.c``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libscir_oracle.so")
_lock = threading.Lock()
_lib = None

MODE_REF, MODE_LFILTER, MODE_FULL, MODE_VALID = 0, 1, 2, 3

_i64 = ctypes.c_int64
_int = ctypes.c_int
_vp = ctypes.c_void_p


def build(force: bool = False) -> str:
    """Compile the oracle with make (gcc, a few seconds)."""
    src = os.path.join(_HERE, "scir_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            sig = {
                "orc_set_threads": (_int, [_int]),
                "orc_fir1d_batched_f32": (None, [_vp, _i64, _i64, _vp, _i64, _vp]),
                "orc_fir1d_batched_f64": (None, [_vp, _i64, _i64, _vp, _i64, _vp]),
                "orc_fir_out_len": (_i64, [_i64, _i64, _int]),
                "orc_fir_mode_f64": (_int, [_vp, _i64, _i64, _vp, _i64, _int, _vp]),
                "orc_fir_ragged_f64": (_int, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _int, _vp, _vp]),
                "orc_sosfilt_f64": (None, [_vp, _int, _vp, _i64, _i64, _vp, _vp, _vp]),
                "orc_filtfilt_ref_f64": (None, [_vp, _int, _vp, _i64, _i64, _vp]),
                "orc_sosfilt_zi": (_int, [_vp, _int, _vp]),
                "orc_sosfiltfilt_default_padlen": (_i64, [_vp, _int]),
                "orc_sosfiltfilt_f64": (_int, [_vp, _int, _vp, _i64, _i64, _int, _i64, _vp]),
                "orc_upfirdn_out_len": (_i64, [_i64, _i64, _i64, _i64]),
                "orc_upfirdn_f64": (None, [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _i64]),
                "orc_resample_poly_out_len": (_i64, [_i64, _i64, _i64]),
                "orc_resample_poly_ref_f64": (_i64, [_vp, _i64, _i64, _i64, _i64, _vp, _i64, _vp]),
                "orc_resample_poly_fast_f64": (_i64, [_vp, _i64, _i64, _i64, _i64, _vp, _i64, _vp]),
                "orc_resize2d_f32": (None, [_vp, _i64, _i64, _vp, _i64, _i64, _int]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> int:
    return lib().orc_set_threads(int(n))


def fir1d_batched_f32(x, taps):
    """Reference ``fir1d_batched_f32`` (f32 in, f32 out, bit-exact restatement)."""
    x = _c(np.atleast_2d(x), np.float32)
    taps = _c(taps, np.float32)
    y = np.empty_like(x)
    lib().orc_fir1d_batched_f32(_p(x), x.shape[0], x.shape[1], _p(taps), taps.size, _p(y))
    return y


def fir1d_batched_f64(x, taps):
    x = _c(np.atleast_2d(x), np.float64)
    taps = _c(taps, np.float64)
    y = np.empty_like(x)
    lib().orc_fir1d_batched_f64(_p(x), x.shape[0], x.shape[1], _p(taps), taps.size, _p(y))
    return y


def fir_out_len(n: int, k: int, mode: int) -> int:
    return int(lib().orc_fir_out_len(n, k, mode))


def fir_mode_f64(x, taps, mode: int):
    x = _c(np.atleast_2d(x), np.float64)
    taps = _c(taps, np.float64)
    n_out = fir_out_len(x.shape[1], taps.size, mode)
    if n_out < 0:
        raise ValueError("invalid FIR mode/shape")
    y = np.empty((x.shape[0], n_out), np.float64)
    rc = lib().orc_fir_mode_f64(_p(x), x.shape[0], x.shape[1], _p(taps), taps.size, mode, _p(y))
    if rc:
        raise ValueError(f"orc_fir_mode_f64 failed ({rc})")
    return y


def sosfilt_f64(sos, x, zi=None, return_zf=False):
    sos = _c(sos, np.float64)
    x = _c(np.atleast_2d(x), np.float64)
    b, n = x.shape
    nsec = sos.shape[0]
    y = np.empty_like(x)
    zf = np.empty((b, nsec, 2), np.float64) if return_zf else None
    zi_c = _c(np.broadcast_to(zi, (b, nsec, 2)), np.float64) if zi is not None else None
    lib().orc_sosfilt_f64(_p(sos), nsec, _p(x), b, n,
                          _p(zi_c) if zi_c is not None else None,
                          _p(zf) if zf is not None else None, _p(y))
    return (y, zf) if return_zf else y


def filtfilt_ref_f64(sos, x):
    sos = _c(sos, np.float64)
    x = _c(np.atleast_2d(x), np.float64)
    y = np.empty_like(x)
    lib().orc_filtfilt_ref_f64(_p(sos), sos.shape[0], _p(x), x.shape[0], x.shape[1], _p(y))
    return y


def sosfilt_zi(sos):
    sos = _c(sos, np.float64)
    zi = np.empty((sos.shape[0], 2), np.float64)
    if lib().orc_sosfilt_zi(_p(sos), sos.shape[0], _p(zi)) != 0:
        raise ValueError("section with a pole at z = 1")
    return zi


def sosfiltfilt_default_padlen(sos) -> int:
    sos = _c(sos, np.float64)
    return int(lib().orc_sosfiltfilt_default_padlen(_p(sos), sos.shape[0]))


def sosfiltfilt_f64(sos, x, padtype: str | None = "odd", padlen: int | None = None):
    sos = _c(sos, np.float64)
    x = _c(np.atleast_2d(x), np.float64)
    y = np.empty_like(x)
    pt = 0 if padtype == "odd" else -1
    rc = lib().orc_sosfiltfilt_f64(_p(sos), sos.shape[0], _p(x), x.shape[0], x.shape[1], pt,
                                   -1 if padlen is None else int(padlen), _p(y))
    if rc:
        raise ValueError(f"orc_sosfiltfilt_f64 failed ({rc})")
    return y


def upfirdn_f64(h, x, up: int, down: int):
    h = _c(h, np.float64)
    x = _c(np.atleast_2d(x), np.float64)
    nout = int(lib().orc_upfirdn_out_len(h.size, x.shape[1], up, down))
    y = np.empty((x.shape[0], nout), np.float64)
    lib().orc_upfirdn_f64(_p(h), h.size, _p(x), x.shape[0], x.shape[1], up, down, _p(y), nout)
    return y


def resample_poly_out_len(n: int, up: int, down: int) -> int:
    return int(lib().orc_resample_poly_out_len(n, up, down))


def resample_poly_ref_f64(x, up: int, down: int, h):
    """The reference algorithm (zero-stuff, full convolution, decimate)."""
    h = _c(h, np.float64)
    x = _c(np.atleast_2d(x), np.float64)
    b, n = x.shape
    nc = n * up + h.size - 1
    off = (h.size - 1) // 2
    nout = max(0, -(-(nc - 2 * off) // down))
    y = np.empty((b, nout), np.float64)
    got = lib().orc_resample_poly_ref_f64(_p(x), b, n, up, down, _p(h), h.size, _p(y))
    assert got == nout
    return y


def resample_poly_fast_f64(x, up: int, down: int, h):
    """scipy.signal.resample_poly with explicit taps h (already scaled by up)."""
    h = _c(h, np.float64)
    x = _c(np.atleast_2d(x), np.float64)
    b, n = x.shape
    nout = resample_poly_out_len(n, up, down)
    y = np.empty((b, nout), np.float64)
    got = lib().orc_resample_poly_fast_f64(_p(x), b, n, up, down, _p(h), h.size, _p(y))
    assert got == nout
    return y


def resize2d_f32(img, out_h, out_w, mode):
    """Reference ``DeviceArray::resize2d_f32`` (mode 0 nearest, 1 bilinear),
    f32 arithmetic in the reference's order."""
    img = _c(img, np.float32)
    out = np.empty((out_h, out_w), np.float32)
    lib().orc_resize2d_f32(_p(img), img.shape[0], img.shape[1], _p(out), out_h, out_w, int(mode))
    return out
