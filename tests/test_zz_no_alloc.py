"""The allocation-free forward-backward entry point.

scir_sosfiltfilt_f32_noalloc serves callers that may not allocate device
memory while they filter (real-time frame loops, processes whose device
memory is reserved by another pool, FFI hosts that forbid hidden
allocations): it takes its scratch from a fixed device array instead of the
stream-ordered allocator.  It must give the same result as the allocating
entry point scir_sosfiltfilt_f32, call after call, for every precision and
padding, leave the library's scratch pool untouched, and refuse work that does
not fit its fixed scratch.  This file is collected last on purpose."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest
import scipy.signal as ss

import scir_gb300 as S
from conftest import ROOT, normwise_err

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the sosfiltfilt tolerance used by the other GPU tests
SOS = np.ascontiguousarray(ss.butter(8, [0.001, 0.002], btype="bandpass", output="sos"))
PRECISIONS = [S.SosPrecision.FP64, S.SosPrecision.FP32, S.SosPrecision.FP32_COUPLED]


def _entry():
    fn = S.load().scir_sosfiltfilt_f32_noalloc
    i64, vp = ctypes.c_int64, ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [vp, i64, i64, i64, vp, ctypes.c_int, ctypes.c_int, i64, ctypes.c_int, vp, i64,
                   vp]
    return fn


def _call(fn, x, y, sos, padtype=S.PadType.ODD, padlen=-1, precision=S.SosPrecision.FP64):
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    return fn(x.data_ptr(), x.stride(0), x.shape[0], x.shape[1], sos.ctypes.data, sos.shape[0],
              int(padtype), padlen, int(precision), y.data_ptr(), y.stride(0), stream)


@pytest.mark.parametrize("precision", PRECISIONS, ids=lambda p: p.name)
@pytest.mark.parametrize("padtype,padlen", [(S.PadType.ODD, -1), (S.PadType.ODD, 0),
                                            (S.PadType.NONE, 0)], ids=["odd", "odd0", "none"])
def test_noalloc_matches_allocating_entry_point(cuda, precision, padtype, padlen):
    import torch
    fn = _entry()
    for call in range(2):  # the second call reuses the array the first one left behind
        g = torch.Generator(device=cuda).manual_seed(100 + call)
        x = torch.randn((96, 30000), device=cuda, generator=g)
        ref = S.sosfiltfilt_f32(SOS, x, padtype=padtype, padlen=padlen,
                                precision=precision).cpu().numpy()
        torch.cuda.synchronize()
        before = S.scratch_usage()
        y = torch.full_like(x, float("nan"))
        assert _call(fn, x, y, SOS, padtype, padlen, precision) == 0, S.last_error()
        torch.cuda.synchronize()
        assert S.scratch_usage() == before  # the library's pool was not touched
        assert normwise_err(y.cpu().numpy(), ref) <= TOL


@pytest.mark.parametrize("precision", PRECISIONS, ids=lambda p: p.name)
def test_noalloc_in_place(cuda, precision):
    import torch
    fn = _entry()
    g = torch.Generator(device=cuda).manual_seed(7)
    x = torch.randn((40, 20000), device=cuda, generator=g)
    ref = S.sosfiltfilt_f32(SOS, x, precision=precision).cpu().numpy()
    assert _call(fn, x, x, SOS, precision=precision) == 0, S.last_error()  # y aliases x
    torch.cuda.synchronize()
    assert normwise_err(x.cpu().numpy(), ref) <= TOL


_FRESH = r"""
import ctypes, sys
import numpy as np, scipy.signal as ss, torch
sys.path.insert(0, {root!r})
import scir_gb300 as S
dev = torch.device("cuda:0")
torch.cuda.set_device(dev)
sos = np.ascontiguousarray(ss.butter(8, [0.001, 0.002], btype="bandpass", output="sos"))
x = torch.randn((64, 25000), device=dev, generator=torch.Generator(device=dev).manual_seed(3))
y = torch.empty_like(x)
torch.cuda.synchronize()
fn = S.load().scir_sosfiltfilt_f32_noalloc
i64, vp = ctypes.c_int64, ctypes.c_void_p
fn.restype = ctypes.c_int
fn.argtypes = [vp, i64, i64, i64, vp, ctypes.c_int, ctypes.c_int, i64, ctypes.c_int, vp, i64, vp]
# the very first library call of the process: FP32 coupled state, whose
# pipeline kernels report bounded-wait timeouts through the device error word
rc = fn(x.data_ptr(), x.stride(0), 64, 25000, sos.ctypes.data, sos.shape[0], int(S.PadType.ODD),
        -1, int(S.SosPrecision.FP32_COUPLED), y.data_ptr(), y.stride(0),
        torch.cuda.current_stream().cuda_stream)
assert rc == 0, S.last_error()
torch.cuda.synchronize()
assert S.scratch_usage() == (0, 0), S.scratch_usage()  # no scratch pool was ever created
ref = S.sosfiltfilt_f32(sos, x, precision=S.SosPrecision.FP32_COUPLED).cpu().numpy().astype(np.float64)
got = y.cpu().numpy().astype(np.float64)
err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
assert err <= {tol}, err
assert S.device_errors() == 0
print("fresh ok")
"""


def test_noalloc_first_call_in_a_fresh_process(cuda):
    # a process whose first library call is the allocation-free entry point
    code = _FRESH.format(root=ROOT, tol=TOL)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600,
                       cwd=ROOT, env=dict(os.environ))
    assert r.returncode == 0 and "fresh ok" in r.stdout, r.stdout + r.stderr


def test_noalloc_rejects_work_beyond_its_scratch(cuda):
    import torch
    fn = _entry()
    x = torch.zeros((2, 64), device=cuda)
    y = torch.empty_like(x)
    # batch * padlen above the fixed 4 Mi-float scratch: refused before any device work
    rc = fn(x.data_ptr(), 64, 100000, 63, SOS.ctypes.data, SOS.shape[0], int(S.PadType.ODD), 51,
            int(S.SosPrecision.FP64), y.data_ptr(), 64, None)
    assert rc == S.ERR_SHAPE
    assert "scratch" in S.last_error()
