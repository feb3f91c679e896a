"""The allocation-free forward-backward entry point.

scir_sosfiltfilt_f32_noalloc serves callers that may not allocate device
memory while they filter (real-time frame loops, processes whose device
memory is reserved by another pool, FFI hosts that forbid hidden
allocations): it takes its scratch from a fixed device array instead of the
stream-ordered allocator.  It must give the same result as the allocating
entry point scir_sosfiltfilt_f32, call after call, and refuse work that does
not fit its fixed scratch.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import scipy.signal as ss

import scir_gb300 as S
from conftest import normwise_err

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the sosfiltfilt tolerance used by the other GPU tests
SOS = ss.butter(8, [0.001, 0.002], btype="bandpass", output="sos")


def _entry():
    fn = S.load().scir_sosfiltfilt_f32_noalloc
    i64, vp = ctypes.c_int64, ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [vp, i64, i64, i64, vp, ctypes.c_int, ctypes.c_int, i64, ctypes.c_int, vp, i64,
                   vp]
    return fn


def _call(fn, x, y, sos, padlen=-1, precision=S.SosPrecision.FP64):
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    return fn(x.data_ptr(), x.stride(0), x.shape[0], x.shape[1], sos.ctypes.data, sos.shape[0],
              int(S.PadType.ODD), padlen, int(precision), y.data_ptr(), y.stride(0), stream)


def test_noalloc_matches_allocating_entry_point(cuda):
    import torch
    fn = _entry()
    sos = np.ascontiguousarray(SOS)
    for call in range(2):  # the second call reuses the array the first one left behind
        g = torch.Generator(device=cuda).manual_seed(100 + call)
        x = torch.randn((96, 30000), device=cuda, generator=g)
        ref = S.sosfiltfilt_f32(sos, x).cpu().numpy()
        y = torch.full_like(x, float("nan"))
        assert _call(fn, x, y, sos) == 0, S.last_error()
        torch.cuda.synchronize()
        assert normwise_err(y.cpu().numpy(), ref) <= TOL


def test_noalloc_rejects_work_beyond_its_scratch(cuda):
    import torch
    fn = _entry()
    sos = np.ascontiguousarray(SOS)
    x = torch.zeros((2, 64), device=cuda)
    y = torch.empty_like(x)
    # batch * padlen above the fixed 4 Mi-float scratch: refused before any device work
    rc = fn(x.data_ptr(), 64, 100000, 63, sos.ctypes.data, sos.shape[0], int(S.PadType.ODD), 51,
            int(S.SosPrecision.FP64), y.data_ptr(), 64, None)
    assert rc == S.ERR_SHAPE
    assert "scratch" in S.last_error()
