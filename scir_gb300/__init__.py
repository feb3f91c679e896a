"""scir_gb300 -- GB300 (sm_103a) batched filtering for SciR.

Python face of the C ABI in ``include/scir_gb300.h``.  Two layers:

* Host-array functions named after the reference's Rust API
  (``fir1d_batched_f32_cuda``, ``fir1d_batched_f32_auto``, ``sosfilt``,
  ``filtfilt``, ``resample_poly``): numpy in, numpy out, synchronous, the
  reference's semantics (crates/scir-gpu/src/lib.rs:515-531, 1036-1152;
  crates/scir-signal/src/lib.rs:260-362).  Failures raise ``GpuError``, the
  mirror of ``scir_gpu::GpuError`` (lib.rs:58-63); there is no CPU fallback.
* Device functions on CUDA tensors (``fir_batched``, ``upfirdn``,
  ``resample_poly_f32``, ``sosfilt_f32``, ``sosfiltfilt_f32``,
  ``RaggedPlan``): stream-ordered, caller-owned buffers.  torch only supplies
  the device memory and the stream handle.
"""
from __future__ import annotations

import ctypes
import enum
from typing import Optional

import numpy as np

from ._native import NativeLibraryError, last_error, load, status_string

__all__ = [
    "Device", "GpuError", "NativeLibraryError", "FirMode", "Precision", "SosPrecision", "PadType",
    "fir1d_batched_f32_cuda", "fir1d_batched_f32_auto", "fir_batched_host", "sosfilt", "filtfilt",
    "resample_poly", "resample_poly_host", "fir_batched", "fir_out_len", "upfirdn",
    "upfirdn_out_len", "resample_poly_f32", "resample_poly_out_len", "resample_poly_default_taps",
    "sosfilt_f32", "sosfilt_f64", "sosfiltfilt_f32", "sosfiltfilt_f64", "sosfilt_zi",
    "sosfiltfilt_default_padlen", "RaggedPlan", "load", "device_errors", "FilterFamily", "BandType",
    "SosPairing", "iirfilter", "butter", "cheby1", "bessel", "zpk2sos", "firwin",
]

OK, ERR_INVALID_ARG, ERR_SHAPE, ERR_ALIGN, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_UNSUPPORTED, \
    ERR_NO_DEVICE = range(9)


class FirMode(enum.IntEnum):
    REF_CORR = 0  # reference fir1d_batched_f32: y[i] = sum_j taps[k-1-j] x[i-j]
    LFILTER = 1   # scipy.signal.lfilter(taps, 1, x)
    FULL = 2      # numpy.convolve(x, taps, 'full')
    VALID = 3     # numpy.convolve(x, taps, 'valid')


class Precision(enum.IntEnum):
    AUTO = -1
    REF_EXACT = 0  # FP32, reference order, no FMA (bit-identical to the reference loop)
    FP32 = 1       # FP32 FMA on CUDA cores ("plain")
    BF16X3 = 2     # tensor cores, bf16 hi+lo operands, 3 products
    BF16X6 = 3     # tensor cores, 3-term bf16 operands, 6 products
    FP16X3 = 4     # tensor cores, power-of-two scaled fp16 hi+lo operands, 3 products


class SosPrecision(enum.IntEnum):
    FP64_EXACT = 0    # FP64 state + coefficients, reference operation order
    FP64 = 1          # FP64 state + coefficients, FMA
    FP32 = 2          # all FP32 (DF2T)
    FP32_COUPLED = 3  # FP32 state, complex-pole sections in coupled form (FP64-derived)


class PadType(enum.IntEnum):
    NONE = 0  # reference filtfilt: no padding, zero state
    ODD = 1   # scipy.signal.sosfiltfilt default


class Device(enum.Enum):
    """Mirror of ``scir_gpu::Device`` (crates/scir-gpu/src/lib.rs:26-35)."""
    Cpu = "cpu"
    Cuda = "cuda"


class GpuError(RuntimeError):
    """Mirror of ``scir_gpu::GpuError``: kind is ``"ShapeMismatch"`` for shape
    errors and ``"BackendUnavailable"`` for everything else."""

    def __init__(self, status: int, message: str):
        self.status = int(status)
        self.kind = "ShapeMismatch" if status == ERR_SHAPE else "BackendUnavailable"
        super().__init__(f"{self.kind} [{status_string(status) if status else 'ok'}]: {message}")


def _check(rc: int) -> None:
    if rc != OK:
        raise GpuError(rc, last_error())


def _ptr(a) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data if isinstance(a, np.ndarray) else int(a))


# --------------------------------------------------------------------------- host layer

def fir1d_batched_f32_cuda(x, taps) -> np.ndarray:
    """crates/scir-gpu/src/lib.rs:1036 ``fir1d_batched_f32_cuda``: rows of x
    filtered with the reference's causal correlation, on the GPU, bit-identical
    to the reference CPU loop."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    if x.ndim != 2:
        raise GpuError(ERR_SHAPE, "x must be 2-D (batch, n)")
    taps = np.ascontiguousarray(taps, dtype=np.float32).reshape(-1)
    y = np.empty_like(x)
    _check(load().scir_fir1d_batched_f32_cuda(_ptr(x), x.shape[0], x.shape[1], _ptr(taps),
                                               taps.size, _ptr(y)))
    return y


def fir1d_batched_f32_auto(x, taps, device: Device) -> np.ndarray:
    """crates/scir-gpu/src/lib.rs:515 ``fir1d_batched_f32_auto``.  Only the CUDA
    device is served by this library (the CPU device stays in scir-gpu);
    there is no silent fallback -- errors raise ``GpuError``."""
    if device is Device.Cuda:
        return fir1d_batched_f32_cuda(x, taps)
    raise GpuError(ERR_UNSUPPORTED, "Device.Cpu is served by scir-gpu's own CPU loop")


def host_chunk_plan(rows: int, in_row_bytes: int, out_row_bytes: int,
                    quantum: int = 1) -> list:
    """Row counts of the pipelined chunks the host-buffer entry points cut a
    call into (host arithmetic only)."""
    count = ctypes.c_int64(0)
    _check(load().scir_host_chunk_plan(rows, in_row_bytes, out_row_bytes, quantum, None, 0,
                                       ctypes.byref(count)))
    sizes = np.zeros(max(count.value, 1), np.int64)
    _check(load().scir_host_chunk_plan(rows, in_row_bytes, out_row_bytes, quantum, _ptr(sizes),
                                       count.value, ctypes.byref(count)))
    return sizes[:count.value].tolist()


def fir_batched_host(x, taps, mode: FirMode = FirMode.LFILTER,
                     precision: Precision = Precision.AUTO, out=None) -> np.ndarray:
    """Any FIR mode/precision on host rows (pipelined copies + kernel);
    `out` may be a preallocated (e.g. pinned) float32 array."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    taps = np.ascontiguousarray(taps, dtype=np.float32).reshape(-1)
    n_out = fir_out_len(x.shape[1], taps.size, mode)
    y = np.empty((x.shape[0], n_out), np.float32) if out is None else out
    if y.shape != (x.shape[0], n_out) or y.dtype != np.float32 or not y.flags.c_contiguous:
        raise GpuError(ERR_SHAPE, "out must be a C-contiguous float32 (batch, n_out) array")
    _check(load().scir_fir_batched_f32_host(_ptr(x), x.shape[0], x.shape[1], _ptr(taps), taps.size,
                                             int(mode), int(precision), _ptr(y)))
    return y


def _sos_array(sos) -> np.ndarray:
    sos = np.ascontiguousarray(sos, dtype=np.float64)
    if sos.ndim != 2 or sos.shape[1] != 6:
        raise GpuError(ERR_SHAPE, "sos must have shape (n_sections, 6)")
    return sos


def sosfilt(sos, x) -> np.ndarray:
    """crates/scir-signal/src/lib.rs:260 ``sosfilt`` (f64, zero state, DF2T);
    1-D or (batch, n) input."""
    sos = _sos_array(sos)
    x = np.ascontiguousarray(x, dtype=np.float64)
    x2 = x.reshape(1, -1) if x.ndim == 1 else x
    y = np.empty_like(x2)
    _check(load().scir_sosfilt_f64_host(_ptr(sos), sos.shape[0], _ptr(x2), x2.shape[0],
                                        x2.shape[1], _ptr(y)))
    return y.reshape(x.shape)


def filtfilt(sos, x) -> np.ndarray:
    """crates/scir-signal/src/lib.rs:278 ``filtfilt`` (no padding, zero state)."""
    sos = _sos_array(sos)
    x = np.ascontiguousarray(x, dtype=np.float64)
    x2 = x.reshape(1, -1) if x.ndim == 1 else x
    y = np.empty_like(x2)
    _check(load().scir_filtfilt_f64_host(_ptr(sos), sos.shape[0], _ptr(x2), x2.shape[0],
                                         x2.shape[1], _ptr(y)))
    return y.reshape(x.shape)


def resample_poly(x, up: int, down: int) -> np.ndarray:
    """crates/scir-signal/src/lib.rs:313 ``resample_poly`` (the reference's
    design, 2/3 only, f64)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    x2 = x.reshape(1, -1) if x.ndim == 1 else x
    n_out = resample_poly_out_len(x2.shape[1], up, down)
    y = np.empty((x2.shape[0], n_out), np.float64)
    _check(load().scir_resample_poly_f64_host(_ptr(x2), x2.shape[0], x2.shape[1], up, down, _ptr(y)))
    return y.reshape(-1) if x.ndim == 1 else y


def resample_poly_host(x, up: int, down: int, h=None,
                       precision: Precision = Precision.AUTO, out=None) -> np.ndarray:
    """SciPy-semantics resample_poly on f32 host rows (default Kaiser design
    when h is None; explicit h must include the gain up).  `out` may be a
    preallocated (e.g. pinned) float32 array."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    n_out = resample_poly_out_len(x.shape[1], up, down)
    y = np.empty((x.shape[0], n_out), np.float32) if out is None else out
    if y.shape != (x.shape[0], n_out) or y.dtype != np.float32 or not y.flags.c_contiguous:
        raise GpuError(ERR_SHAPE, "out must be a C-contiguous float32 (batch, n_out) array")
    hh = None if h is None else np.ascontiguousarray(h, dtype=np.float32).reshape(-1)
    _check(load().scir_resample_poly_f32_host(_ptr(x), x.shape[0], x.shape[1], up, down,
                                              _ptr(hh) if hh is not None else None,
                                              0 if hh is None else hh.size, int(precision),
                                              _ptr(y)))
    return y


def device_errors() -> int:
    """Reads and clears the device error word (non-zero: a kernel's bounded
    wait gave up).  Synchronises the device."""
    code = ctypes.c_uint(0)
    _check(load().scir_device_errors(ctypes.byref(code)))
    return int(code.value)


def autotune_fir(batch: int, n: int, k: int, mode: FirMode = FirMode.LFILTER,
                 precision: Precision = Precision.AUTO):
    """Times the batched-FIR variants for this shape on the current device and
    records the fastest; returns (choice, ms per call)."""
    ms = ctypes.c_double()
    buf = ctypes.create_string_buffer(64)
    _check(load().scir_autotune_fir(batch, n, k, int(mode), int(precision), ctypes.byref(ms), buf, 64))
    return buf.value.decode(), ms.value


def autotune_resample_poly(batch: int, n: int, up: int, down: int, kh: int = 0):
    """Times the polyphase schedules for this shape (kh = 0: the default
    design) and records the fastest; returns (choice, ms per call)."""
    ms = ctypes.c_double()
    buf = ctypes.create_string_buffer(64)
    _check(load().scir_autotune_resample_poly(batch, n, up, down, kh, ctypes.byref(ms), buf, 64))
    return buf.value.decode(), ms.value


def init(device: int = 0) -> None:
    """Creates the library's per-device state for ``device`` and makes it
    current (needed before a CUDA-graph capture)."""
    _check(load().scir_init(device))


class ResizeMode(enum.IntEnum):
    NEAREST = 0
    BILINEAR = 1


def _f32_flat(t, name):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32:
        raise GpuError(ERR_INVALID_ARG, f"{name} must be a float32 CUDA tensor")
    if not t.is_contiguous():
        raise GpuError(ERR_INVALID_ARG, f"{name} must be contiguous")
    return t


def add_vec(a, b, out=None, stream=None):
    """DeviceArray::add_auto on the GPU: out = a + b (same shape, float32)."""
    a, b = _f32_flat(a, "a"), _f32_flat(b, "b")
    if a.shape != b.shape:
        raise GpuError(ERR_SHAPE, "shape mismatch")
    out = _torch().empty_like(a) if out is None else _f32_flat(out, "out")
    _check(load().scir_add_vec_f32(a.data_ptr(), b.data_ptr(), out.data_ptr(), a.numel(),
                                   _stream(stream)))
    return out


def add_scalar(a, alpha: float, out=None, stream=None):
    a = _f32_flat(a, "a")
    out = _torch().empty_like(a) if out is None else _f32_flat(out, "out")
    _check(load().scir_add_scalar_f32(a.data_ptr(), float(alpha), out.data_ptr(), a.numel(),
                                      _stream(stream)))
    return out


def mul_scalar(a, alpha: float, out=None, stream=None):
    a = _f32_flat(a, "a")
    out = _torch().empty_like(a) if out is None else _f32_flat(out, "out")
    _check(load().scir_mul_scalar_f32(a.data_ptr(), float(alpha), out.data_ptr(), a.numel(),
                                      _stream(stream)))
    return out


def resize2d(img, out_h: int, out_w: int, mode: ResizeMode = ResizeMode.BILINEAR, stream=None):
    """DeviceArray::resize2d_f32 on a [height, width] float32 CUDA tensor."""
    img = _f32_flat(img, "img")
    if img.dim() != 2:
        raise GpuError(ERR_SHAPE, "resize2d needs a 2-D [height, width] tensor")
    out = _torch().empty((out_h, out_w), device=img.device, dtype=img.dtype)
    _check(load().scir_resize2d_f32(img.data_ptr(), img.shape[0], img.shape[1], out.data_ptr(),
                                    out_h, out_w, int(mode), _stream(stream)))
    return out


class GraphCapture:
    """Records the library calls made on ``stream`` inside the ``with`` block
    into a CUDA graph; ``launch()`` replays them with one launch.  Call
    ``init()`` and make one call of each operation before capturing."""

    def __init__(self, stream):
        self.stream = stream
        self._h = ctypes.c_void_p()

    def __enter__(self):
        _check(load().scir_graph_capture_begin(_stream(self.stream)))
        return self

    def __exit__(self, exc_type, exc, tb):
        rc = load().scir_graph_capture_end(_stream(self.stream), ctypes.byref(self._h))
        if exc_type is None:
            _check(rc)
        return False

    def launch(self, stream=None):
        _check(load().scir_graph_launch(self._h, _stream(self.stream if stream is None else stream)))

    def close(self):
        if self._h:
            load().scir_graph_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_save(path: str) -> None:
    _check(load().scir_autotune_save(path.encode()))


def autotune_load(path: str) -> None:
    _check(load().scir_autotune_load(path.encode()))


def autotune_clear() -> None:
    _check(load().scir_autotune_clear())


def release_scratch() -> None:
    """Returns the unused memory of the library's scratch pool on the current
    device (synchronises the device)."""
    _check(load().scir_release_scratch())


def probe_fma_peak(fp64: bool = False) -> float:
    """Measured FP32 (or FP64) FMA throughput of the current device, TFLOP/s."""
    v = ctypes.c_double(0.0)
    _check(load().scir_probe_fma_peak(1 if fp64 else 0, ctypes.byref(v)))
    return float(v.value)


def scratch_usage() -> tuple:
    """(reserved, used) bytes of the library's scratch pool on the current
    device; (0, 0) before any call needed scratch."""
    r, u = ctypes.c_uint64(0), ctypes.c_uint64(0)
    _check(load().scir_scratch_usage(ctypes.byref(r), ctypes.byref(u)))
    return int(r.value), int(u.value)


def fir_out_len(n: int, k: int, mode: FirMode) -> int:
    v = int(load().scir_fir_out_len(n, k, int(mode)))
    if v < 0:
        raise GpuError(ERR_SHAPE, f"invalid FIR geometry n={n} k={k} mode={mode!r}")
    return v


def upfirdn_out_len(kh: int, n: int, up: int, down: int) -> int:
    return int(load().scir_upfirdn_out_len(kh, n, up, down))


def resample_poly_out_len(n: int, up: int, down: int) -> int:
    v = int(load().scir_resample_poly_out_len(n, up, down))
    if v < 0:
        raise GpuError(ERR_INVALID_ARG, "bad resample_poly sizes")
    return v


def resample_poly_default_taps(up: int, down: int, design: int = 0) -> np.ndarray:
    kh = ctypes.c_int64(0)
    _check(load().scir_resample_poly_default_taps(up, down, design, None, 0, ctypes.byref(kh)))
    h = np.empty(kh.value, np.float64)
    _check(load().scir_resample_poly_default_taps(up, down, design, _ptr(h), h.size, ctypes.byref(kh)))
    return h


def sosfilt_zi(sos) -> np.ndarray:
    sos = _sos_array(sos)
    zi = np.empty((sos.shape[0], 2), np.float64)
    _check(load().scir_sosfilt_zi(_ptr(sos), sos.shape[0], _ptr(zi)))
    return zi


def lfilter_zi(b, a) -> np.ndarray:
    """scipy.signal.lfilter_zi (max(len(a), len(b)) - 1 values)."""
    b = np.ascontiguousarray(np.atleast_1d(b), np.float64)
    a = np.ascontiguousarray(np.atleast_1d(a), np.float64)
    zi = np.empty(max(max(b.size, a.size) - 1, 1), np.float64)
    _check(load().scir_lfilter_zi(_ptr(b), b.size, _ptr(a), a.size, _ptr(zi)))
    return zi[:max(b.size, a.size) - 1]


def sosfiltfilt_default_padlen(sos) -> int:
    sos = _sos_array(sos)
    return int(load().scir_sosfiltfilt_default_padlen(_ptr(sos), sos.shape[0]))


# --------------------------------------------------------------------------- IIR design (host)

class FilterFamily(enum.IntEnum):
    """scir_iir_family: the prototype (and Bessel normalisation)."""
    BUTTER = 0
    CHEBY1 = 1
    BESSEL_PHASE = 2
    BESSEL_DELAY = 3
    BESSEL_MAG = 4


class BandType(enum.IntEnum):
    LOWPASS = 0
    HIGHPASS = 1
    BANDPASS = 2
    BANDSTOP = 3


class SosPairing(enum.IntEnum):
    """SosPairing (crates/scir-iir-filters/src/sos.rs:22-35)."""
    NEAREST = 0
    KEEP_ODD = 1
    MINIMAL = 2


_BTYPE_NAMES = {"low": BandType.LOWPASS, "lowpass": BandType.LOWPASS,
                "high": BandType.HIGHPASS, "highpass": BandType.HIGHPASS,
                "band": BandType.BANDPASS, "bandpass": BandType.BANDPASS,
                "bandstop": BandType.BANDSTOP, "stop": BandType.BANDSTOP}


def _cplx_pairs(v) -> np.ndarray:
    v = np.asarray(v, np.complex128).ravel()
    return np.ascontiguousarray(np.stack([v.real, v.imag], axis=1).ravel())


def iirfilter(order: int, wn, btype="low", family: FilterFamily = FilterFamily.BUTTER,
              rp: float = 0.0, fs: Optional[float] = None, output: str = "sos"):
    """Digital IIR design (iirfilter, crates/scir-iir-filters/src/filter_design.rs:216-314).

    ``wn`` is one edge or two increasing edges in the units of ``fs`` (normalised
    to Nyquist = 1 when ``fs`` is None).  ``output`` is ``"sos"`` ([nsec, 6]) or
    ``"zpk"`` (zeros, poles, gain).
    """
    bt = _BTYPE_NAMES[btype] if isinstance(btype, str) else BandType(btype)
    w = np.ascontiguousarray(np.atleast_1d(np.asarray(wn, np.float64)))
    need = 2 if bt >= BandType.BANDPASS else 1
    if w.size != need:
        raise GpuError(ERR_INVALID_ARG, f"{bt.name.lower()} needs {need} edge(s), got {w.size}")
    fsv = -1.0 if fs is None else float(fs)
    lib = load()
    if output == "sos":
        nsec = ctypes.c_int(0)
        _check(lib.scir_iirfilter_sos(int(order), int(family), int(bt), _ptr(w), float(rp), fsv,
                                      None, 0, ctypes.byref(nsec)))
        sos = np.empty((nsec.value, 6), np.float64)
        _check(lib.scir_iirfilter_sos(int(order), int(family), int(bt), _ptr(w), float(rp), fsv,
                                      _ptr(sos), nsec.value, ctypes.byref(nsec)))
        return sos
    if output != "zpk":
        raise GpuError(ERR_INVALID_ARG, f"unknown output {output!r}")
    nz, npl, k = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0.0)
    _check(lib.scir_iirfilter_zpk(int(order), int(family), int(bt), _ptr(w), float(rp), fsv,
                                  None, None, 0, ctypes.byref(nz), ctypes.byref(npl),
                                  ctypes.byref(k)))
    cap = max(nz.value, npl.value, 1)
    zb = np.empty(2 * cap, np.float64)
    pb = np.empty(2 * cap, np.float64)
    _check(lib.scir_iirfilter_zpk(int(order), int(family), int(bt), _ptr(w), float(rp), fsv,
                                  _ptr(zb), _ptr(pb), cap, ctypes.byref(nz), ctypes.byref(npl),
                                  ctypes.byref(k)))
    z = zb[0:2 * nz.value:2] + 1j * zb[1:2 * nz.value:2]
    p = pb[0:2 * npl.value:2] + 1j * pb[1:2 * npl.value:2]
    return z, p, k.value


def butter(order: int, wn, btype="low", fs: Optional[float] = None, output: str = "sos"):
    """butter (crates/scir-iir-filters/src/filter_design.rs:128)."""
    return iirfilter(order, wn, btype, FilterFamily.BUTTER, 0.0, fs, output)


def cheby1(order: int, rp: float, wn, btype="low", fs: Optional[float] = None,
           output: str = "sos"):
    """cheby1 (crates/scir-iir-filters/src/filter_design.rs:191)."""
    return iirfilter(order, wn, btype, FilterFamily.CHEBY1, rp, fs, output)


def bessel(order: int, wn, btype="low", fs: Optional[float] = None, norm: str = "phase",
           output: str = "sos"):
    """bessel / bessel_with_norm (crates/scir-iir-filters/src/filter_design.rs:154-175)."""
    fam = {"phase": FilterFamily.BESSEL_PHASE, "delay": FilterFamily.BESSEL_DELAY,
           "mag": FilterFamily.BESSEL_MAG}[norm]
    return iirfilter(order, wn, btype, fam, 0.0, fs, output)


_WINDOWS = {"hamming": 0, "kaiser": 1, "hann": 2, "hanning": 2, "blackman": 3, "boxcar": 4,
            "rectangular": 4}


def firwin(numtaps: int, cutoff, window="hamming", pass_zero=True, scale: bool = True,
           fs: Optional[float] = None) -> np.ndarray:
    """scipy.signal.firwin: window is a name or ("kaiser", beta); pass_zero is a
    bool or "lowpass" / "highpass" / "bandpass" / "bandstop"."""
    c = np.ascontiguousarray(np.atleast_1d(np.asarray(cutoff, np.float64)))
    beta = 0.0
    if isinstance(window, tuple):
        name, beta = window[0], float(window[1])
    else:
        name = window
    if name not in _WINDOWS:
        raise GpuError(ERR_INVALID_ARG, f"unsupported window {window!r}")
    if isinstance(pass_zero, str):
        pass_zero = pass_zero in ("lowpass", "bandstop")
    h = np.empty(int(numtaps), np.float64)
    _check(load().scir_firwin(int(numtaps), _ptr(c), c.size, _WINDOWS[name], beta,
                              1 if pass_zero else 0, 1 if scale else 0,
                              -1.0 if fs is None else float(fs), _ptr(h)))
    return h


def zpk2sos(z, p, k: float, pairing: SosPairing = SosPairing.NEAREST) -> np.ndarray:
    """zpk2sos (crates/scir-iir-filters/src/sos.rs:154-357)."""
    zb, pb = _cplx_pairs(z), _cplx_pairs(p)
    nz, npl = zb.size // 2, pb.size // 2
    nsec = ctypes.c_int(0)
    lib = load()
    _check(lib.scir_zpk2sos(_ptr(zb), nz, _ptr(pb), npl, float(k), int(pairing), None, 0,
                            ctypes.byref(nsec)))
    sos = np.empty((nsec.value, 6), np.float64)
    _check(lib.scir_zpk2sos(_ptr(zb), nz, _ptr(pb), npl, float(k), int(pairing), _ptr(sos),
                            nsec.value, ctypes.byref(nsec)))
    return sos


# --------------------------------------------------------------------------- device layer

def _torch():
    import torch  # plumbing for device memory and streams
    return torch


def _stream(stream) -> ctypes.c_void_p:
    if stream is None:
        stream = _torch().cuda.current_stream()
    return ctypes.c_void_p(int(getattr(stream, "cuda_stream", stream)))


def _rows(t, dtype, name: str):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise GpuError(ERR_INVALID_ARG, f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise GpuError(ERR_INVALID_ARG, f"{name} must be {dtype}")
    t2 = t.unsqueeze(0) if t.dim() == 1 else t
    if t2.dim() != 2:
        raise GpuError(ERR_SHAPE, f"{name} must be 1-D or 2-D")
    if t2.shape[1] > 1 and t2.stride(1) != 1:
        raise GpuError(ERR_INVALID_ARG, f"{name} rows must be contiguous")
    ld = t2.stride(0) if t2.shape[0] > 1 else max(t2.shape[1], 1)
    return t2, ld


def fir_batched(x, taps, mode: FirMode = FirMode.LFILTER, precision: Precision = Precision.AUTO,
                out=None, stream=None):
    """Batched FIR of the rows of CUDA float32 tensor x with CUDA float32 taps."""
    torch = _torch()
    x2, ldx = _rows(x, torch.float32, "x")
    taps = taps.contiguous()
    k = taps.numel()
    n_out = x2.shape[1] if k == 0 else fir_out_len(x2.shape[1], k, mode)
    if out is None:
        out = torch.empty((x2.shape[0], n_out), device=x.device, dtype=torch.float32)
    y2, ldy = _rows(out, torch.float32, "out")
    _check(load().scir_fir_batched_f32(x2.data_ptr(), ldx, x2.shape[0], x2.shape[1],
                                       taps.data_ptr(), k, int(mode), int(precision),
                                       y2.data_ptr(), ldy, _stream(stream)))
    return out


def upfirdn(h, x, up: int = 1, down: int = 1, precision: Precision = Precision.FP32, out=None,
            stream=None):
    """scipy.signal.upfirdn(h, x, up, down) along the rows of x."""
    torch = _torch()
    x2, ldx = _rows(x, torch.float32, "x")
    h = h.contiguous()
    n_out = upfirdn_out_len(h.numel(), x2.shape[1], up, down)
    if out is None:
        out = torch.empty((x2.shape[0], n_out), device=x.device, dtype=torch.float32)
    y2, ldy = _rows(out, torch.float32, "out")
    _check(load().scir_upfirdn_f32(x2.data_ptr(), ldx, x2.shape[0], x2.shape[1], h.data_ptr(),
                                   h.numel(), up, down, int(precision), y2.data_ptr(), ldy,
                                   _stream(stream)))
    return out


def resample_poly_f32(x, up: int, down: int, h=None, precision: Precision = Precision.AUTO,
                      out=None, stream=None):
    """scipy.signal.resample_poly along the rows of x (zero-padded edges).  h
    (CUDA float32, gain ``up`` included) defaults to SciPy's Kaiser design."""
    torch = _torch()
    x2, ldx = _rows(x, torch.float32, "x")
    n_out = resample_poly_out_len(x2.shape[1], up, down)
    if out is None:
        out = torch.empty((x2.shape[0], n_out), device=x.device, dtype=torch.float32)
    y2, ldy = _rows(out, torch.float32, "out")
    hp, kh = (None, 0) if h is None else (h.contiguous().data_ptr(), h.numel())
    _check(load().scir_resample_poly_f32(x2.data_ptr(), ldx, x2.shape[0], x2.shape[1], up, down,
                                         hp, kh, int(precision), y2.data_ptr(), ldy,
                                         _stream(stream)))
    return out


def _sosfilt_dev(fn, dtype, sos, x, zi, return_zf, precision, out, stream):
    torch = _torch()
    sos = _sos_array(sos)
    x2, ldx = _rows(x, dtype, "x")
    if out is None:
        out = torch.empty_like(x2)
    y2, ldy = _rows(out, dtype, "out")
    nsec = sos.shape[0]
    zip_ = None
    if zi is not None:
        zi = zi.to(device=x.device, dtype=torch.float64).expand(x2.shape[0], nsec, 2).contiguous()
        zip_ = zi.data_ptr()
    zf = torch.empty((x2.shape[0], nsec, 2), device=x.device, dtype=torch.float64) \
        if return_zf else None
    _check(fn(x2.data_ptr(), ldx, x2.shape[0], x2.shape[1], _ptr(sos), nsec, zip_,
              zf.data_ptr() if zf is not None else None, int(precision), y2.data_ptr(), ldy,
              _stream(stream)))
    return (out, zf) if return_zf else out


def lfilter(b, a, x, zi=None, return_zf: bool = False, out=None, stream=None):
    """scipy.signal.lfilter(b, a, x, axis=-1, zi) along the rows of CUDA tensor
    x (float32 or float64); zi / zf are (batch, max(len(a), len(b)) - 1)
    float64."""
    torch = _torch()
    b = np.ascontiguousarray(np.atleast_1d(b), np.float64)
    a = np.ascontiguousarray(np.atleast_1d(a), np.float64)
    dtype = x.dtype
    if dtype not in (torch.float32, torch.float64):
        raise GpuError(ERR_INVALID_ARG, "x must be float32 or float64")
    x2, ldx = _rows(x, dtype, "x")
    if out is None:
        out = torch.empty_like(x2)
    y2, ldy = _rows(out, dtype, "out")
    ns = max(a.size, b.size) - 1
    zip_ = None
    if zi is not None:
        zi = zi.to(device=x.device, dtype=torch.float64).expand(x2.shape[0], ns).contiguous()
        zip_ = zi.data_ptr()
    zf = torch.empty((x2.shape[0], ns), device=x.device, dtype=torch.float64) if return_zf else None
    fn = load().scir_lfilter_f32 if dtype == torch.float32 else load().scir_lfilter_f64
    _check(fn(x2.data_ptr(), ldx, x2.shape[0], x2.shape[1], _ptr(b), b.size, _ptr(a), a.size, zip_,
              zf.data_ptr() if zf is not None else None, y2.data_ptr(), ldy, _stream(stream)))
    return (out, zf) if return_zf else out


def sosfilt_f32(sos, x, zi=None, return_zf: bool = False,
                precision: SosPrecision = SosPrecision.FP64, out=None, stream=None):
    """Channel-parallel sosfilt of the float32 rows of x; zi/zf are
    (batch, n_sections, 2) float64 DF2T states."""
    return _sosfilt_dev(load().scir_sosfilt_f32, _torch().float32, sos, x, zi, return_zf, precision,
                        out, stream)


def sosfilt_f64(sos, x, zi=None, return_zf: bool = False,
                precision: SosPrecision = SosPrecision.FP64_EXACT, out=None, stream=None):
    return _sosfilt_dev(load().scir_sosfilt_f64, _torch().float64, sos, x, zi, return_zf, precision,
                        out, stream)


def _sosfiltfilt_dev(fn, dtype, sos, x, padtype, padlen, precision, out, stream):
    torch = _torch()
    sos = _sos_array(sos)
    x2, ldx = _rows(x, dtype, "x")
    if out is None:
        out = torch.empty_like(x2)
    y2, ldy = _rows(out, dtype, "out")
    _check(fn(x2.data_ptr(), ldx, x2.shape[0], x2.shape[1], _ptr(sos), sos.shape[0], int(padtype),
              -1 if padlen is None else int(padlen), int(precision), y2.data_ptr(), ldy,
              _stream(stream)))
    return out


def sosfiltfilt_f32(sos, x, padtype: PadType = PadType.ODD, padlen: Optional[int] = None,
                    precision: SosPrecision = SosPrecision.FP64, out=None, stream=None):
    """scipy.signal.sosfiltfilt on float32 rows (PadType.NONE: the reference's
    unpadded filtfilt)."""
    return _sosfiltfilt_dev(load().scir_sosfiltfilt_f32, _torch().float32, sos, x, padtype, padlen,
                            precision, out, stream)


def sosfiltfilt_f64(sos, x, padtype: PadType = PadType.ODD, padlen: Optional[int] = None,
                    precision: SosPrecision = SosPrecision.FP64_EXACT, out=None, stream=None):
    return _sosfiltfilt_dev(load().scir_sosfiltfilt_f64, _torch().float64, sos, x, padtype, padlen,
                            precision, out, stream)


class _Desc(ctypes.Structure):
    _fields_ = [("x_off", ctypes.c_int64), ("n", ctypes.c_int64), ("taps_off", ctypes.c_int64),
                ("k", ctypes.c_int64), ("y_off", ctypes.c_int64)]


class RaggedPlan:
    """A persistent-launch plan over signals of lengths ``n`` and tap counts
    ``k`` packed back to back in one input, one tap and one output buffer."""

    def __init__(self, n, k, mode: FirMode = FirMode.LFILTER,
                 precision: Precision = Precision.FP32, x_off=None, taps_off=None, y_off=None):
        n = np.asarray(n, np.int64)
        k = np.asarray(k, np.int64)
        count = n.size
        self.n_out = np.array([fir_out_len(int(a), int(b), mode) for a, b in zip(n, k)], np.int64)
        self.x_off = np.concatenate([[0], np.cumsum(n)[:-1]]) if x_off is None else np.asarray(x_off)
        self.taps_off = np.concatenate([[0], np.cumsum(k)[:-1]]) if taps_off is None else \
            np.asarray(taps_off)
        self.y_off = np.concatenate([[0], np.cumsum(self.n_out)[:-1]]) if y_off is None else \
            np.asarray(y_off)
        self.x_len = int(n.sum())
        self.taps_len = int(k.sum())
        self.y_len = int(self.n_out.sum())
        table = (_Desc * max(count, 1))()
        for i in range(count):
            table[i] = _Desc(int(self.x_off[i]), int(n[i]), int(self.taps_off[i]), int(k[i]),
                             int(self.y_off[i]))
        self._h = ctypes.c_void_p()
        _check(load().scir_ragged_plan_create(ctypes.cast(table, ctypes.c_void_p), count, int(mode),
                                              int(precision), ctypes.byref(self._h)))
        tiles = ctypes.c_int64()
        macs = ctypes.c_double()
        samples = ctypes.c_int64()
        _check(load().scir_ragged_plan_stats(self._h, ctypes.byref(tiles), ctypes.byref(macs),
                                             ctypes.byref(samples)))
        self.tiles, self.macs, self.samples_in = tiles.value, macs.value, samples.value

    def run(self, x, taps, y, stream=None):
        _check(load().scir_fir_ragged_f32(self._h, x.data_ptr(), taps.data_ptr(), y.data_ptr(),
                                          _stream(stream)))
        return y

    def tensor_cores(self):
        """(tap threshold of the tensor-core bucket or 0, signals in it)."""
        t, c = ctypes.c_int(), ctypes.c_int64()
        _check(load().scir_ragged_plan_tensor_cores(self._h, ctypes.byref(t), ctypes.byref(c)))
        return t.value, c.value

    def autotune(self, x, taps, y, stream=None):
        """Times the tile variants (and, with a tensor-core bucket, its tap
        threshold) on these buffers and rebuilds the plan with the fastest;
        returns (16-output tap threshold, ms per launch)."""
        thr = ctypes.c_int()
        ms = ctypes.c_double()
        _check(load().scir_ragged_plan_autotune(self._h, x.data_ptr(), taps.data_ptr(), y.data_ptr(),
                                                _stream(stream), ctypes.byref(thr), ctypes.byref(ms)))
        return thr.value, ms.value

    def close(self):
        if self._h:
            load().scir_ragged_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

