"""C-ABI surface and host-side logic that needs no GPU: every symbol the
header declares is exported, sizes/geometry agree with the oracle and SciPy,
the FP64 design helpers match SciPy, and argument validation rejects bad
calls before any device work."""
import ctypes
import os
import re

import numpy as np
import pytest
import scipy.signal as ss

import oracle as O
import scir_gb300 as S
from scir_gb300 import _native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "scir_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"SCIR_API\s+[\w\s\*]+?\b(scir_\w+)\s*\(", text)))


def test_header_symbols_exported_and_bound():
    L = S.load()
    syms = declared_symbols()
    assert len(syms) >= 25
    for name in syms:
        assert hasattr(L, name), f"{name} declared in the header but not exported"
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"
    assert set(_native.SIGNATURES) == set(syms)
    assert L.scir_abi_version() == 1


def test_status_strings():
    assert S.status_string(0) == "ok"
    assert "shape" in S.status_string(2)
    assert S.status_string(99) == "unknown status"


@pytest.mark.parametrize("n,k", [(10, 3), (3, 10), (1, 1), (65536, 63), (0, 4)])
def test_fir_out_len(n, k):
    for mode in range(4):
        exp = O.fir_out_len(n, k, mode) if n > 0 or mode < 2 else None
        got = S.load().scir_fir_out_len(n, k, mode)
        if mode == 3 and n < k:
            assert got == -1
        elif exp is not None:
            assert got == exp


@pytest.mark.parametrize("kh,n,up,down", [(3201, 1048576, 160, 147), (31, 32, 2, 3), (9, 5, 1, 4),
                                          (22, 77, 5, 1)])
def test_poly_lengths(kh, n, up, down):
    assert S.upfirdn_out_len(kh, n, up, down) == O.lib().orc_upfirdn_out_len(kh, n, up, down)
    assert S.resample_poly_out_len(n, up, down) == O.resample_poly_out_len(n, up, down)


def test_resample_cfg_output_length():
    # 256 x 1,048,576 at 160/147 gives 1,141,308 outputs per channel
    assert S.resample_poly_out_len(1048576, 160, 147) == 1141308


def test_reference_design_is_the_reference_table(golden_resample23):
    # crates/scir-signal/src/lib.rs:315-347: the same 31 doubles, bit for bit
    h = S.resample_poly_default_taps(2, 3, design=1)
    assert h.size == 31
    assert [int(b) for b in h.view(np.uint64)] == golden_resample23["bits"]
    assert np.array_equal(h, np.array([float(s) for s in golden_resample23["literals"]]))
    # the table is a Hamming design; it agrees with SciPy's only to ~1e-16
    np.testing.assert_allclose(h, ss.firwin(31, 1 / 3, window="hamming") * 2, atol=1e-15, rtol=0)
    assert S.resample_poly_default_taps(4, 6, design=1).tobytes() == h.tobytes()


@pytest.mark.parametrize("up,down", [(160, 147), (2, 3), (3, 2), (1, 5), (4, 6)])
def test_scipy_default_design(up, down):
    import math
    g = math.gcd(up, down)
    u, d = up // g, down // g
    mr = max(u, d)
    ref = ss.firwin(2 * 10 * mr + 1, 1.0 / mr, window=("kaiser", 5.0)) * u
    h = S.resample_poly_default_taps(up, down, design=0)
    np.testing.assert_allclose(h, ref, atol=1e-15, rtol=1e-11)


def test_reference_design_rejects_other_rates():
    with pytest.raises(S.GpuError) as ei:
        S.resample_poly_default_taps(160, 147, design=1)
    assert ei.value.status == S.ERR_UNSUPPORTED


def test_sosfilt_zi_and_padlen():
    for sos in [ss.butter(8, [0.001, 0.002], btype="bandpass", output="sos"),
                ss.butter(4, 0.2, output="sos"), ss.cheby1(5, 1, 0.3, output="sos")]:
        np.testing.assert_allclose(S.sosfilt_zi(sos), ss.sosfilt_zi(sos), rtol=1e-12, atol=1e-14)
        assert S.sosfiltfilt_default_padlen(sos) == O.sosfiltfilt_default_padlen(sos)


def test_validation_before_device():
    L = S.load()
    f = ctypes.c_void_p(16)
    # VALID with n < k
    assert L.scir_fir_batched_f32(f, 4, 1, 4, f, 8, 3, 1, f, 4, None) == S.ERR_SHAPE
    # row stride shorter than the row
    assert L.scir_fir_batched_f32(f, 3, 2, 4, f, 2, 1, 1, f, 4, None) == S.ERR_SHAPE
    # null taps
    assert L.scir_fir_batched_f32(f, 4, 1, 4, None, 2, 1, 1, f, 4, None) == S.ERR_INVALID_ARG
    # unknown mode / precision
    assert L.scir_fir_batched_f32(f, 4, 1, 4, f, 2, 9, 1, f, 4, None) == S.ERR_INVALID_ARG
    assert L.scir_fir_batched_f32(f, 4, 1, 4, f, 2, 1, 7, f, 4, None) == S.ERR_INVALID_ARG
    # upfirdn with up = 0
    assert L.scir_upfirdn_f32(f, 4, 1, 4, f, 3, 0, 1, 1, f, 8, None) == S.ERR_INVALID_ARG
    assert "up and down" in S.last_error()
    # sos section count out of range
    sos = np.zeros((40, 6))
    assert L.scir_sosfilt_f32(f, 4, 1, 4, sos.ctypes.data, 40, None, None, 1, f, 4, None) \
        == S.ERR_INVALID_ARG
    # the ragged plan rejects a descriptor with k = 0 before any upload
    with pytest.raises(S.GpuError):
        S.RaggedPlan([10, 20], [3, 0])


MB = 1 << 20


@pytest.mark.parametrize("rows,in_row,out_row,quantum", [
    (1, 4, 4, 1),
    (64, 65536 * 4, 65536 * 4, 1),               # 64 x 65,536 short-tap FIR call
    (1024, 262144 * 4, 262144 * 4, 128),         # 1,024 x 262,144 long-tap FIR call
    (256, 1048576 * 4, 1141308 * 4, 1),          # resample 160/147, 256 x 1,048,576
    (600, 40000 * 4, 40000 * 4, 1),
    (7, 100, 100, 128),
    (1000, 8, 8, 1),
    (3, 100 * MB, 100 * MB, 1),                  # rows larger than a chunk's target
    (5000, 1 * MB, 1 * MB, 128),
])
def test_host_chunk_plan(rows, in_row, out_row, quantum):
    # the host-buffer layer's chunking: every row once, whole chunks of cr rows
    # in the middle, half-size first and last chunks when there are three or
    # more, cr from a sixth of the call's bytes within 4 .. 64 MB (at least one
    # row), rounded up to the quantum while a chunk stays within 512 MB
    sizes = S.host_chunk_plan(rows, in_row, out_row, quantum)
    assert sum(sizes) == rows and min(sizes) >= 1
    row = in_row + out_row + 1
    target = min(64 * MB, max(4 * MB, rows * row // 6))
    cr = max(1, target // row)
    if quantum > 1 and -(-cr // quantum) * quantum * row <= 512 * MB:
        cr = -(-cr // quantum) * quantum
    cr = min(cr, rows)
    assert max(sizes) == cr
    if rows > 2 * cr and cr >= 2:
        h = cr // 2
        assert sizes[0] == h and sizes[-1] <= h
        assert all(s == cr for s in sizes[1:-2]) and 1 <= sizes[-2] <= cr
    else:
        assert all(s == cr for s in sizes[:-1])


def test_host_chunk_plan_random_shapes():
    # seeded sweep: rows 1 .. 100,000, row bytes 4 B .. 256 MB, quantum 1 or 128
    rng = np.random.default_rng(21)
    for _ in range(300):
        rows = int(np.exp(rng.uniform(0, np.log(100000))))
        in_row = int(np.exp(rng.uniform(np.log(4), np.log(256 * MB))))
        out_row = int(in_row * rng.uniform(0.5, 2.0))
        quantum = int(rng.choice([1, 128]))
        sizes = S.host_chunk_plan(rows, in_row, out_row, quantum)
        cr = max(sizes)
        assert sum(sizes) == rows and min(sizes) >= 1
        row = in_row + out_row + 1
        # a full chunk stays within 64 MB (or is one row), or within 512 MB
        # when rounded up to the quantum
        assert cr == 1 or cr * row <= (512 if quantum > 1 else 64) * MB
        if len(sizes) >= 3 and cr >= 2:  # single-row chunks have no half size
            assert sizes[0] == cr // 2 and sizes[-1] <= cr // 2
            assert all(s == cr for s in sizes[1:-2])
        else:
            assert all(s == cr for s in sizes[:-1])


def test_host_chunk_plan_long_tap_call():
    # 1,024 rows of 1 MB in and 1 MB out with 128-row tensor-core tiles: a
    # 64-row chunk, seven of 128, a 64-row chunk
    assert S.host_chunk_plan(1024, 1 * MB, 1 * MB, 128) == [64] + [128] * 7 + [64]
    L = S.load()
    n = ctypes.c_int64(-1)
    assert L.scir_host_chunk_plan(0, 4, 4, 1, None, 0, ctypes.byref(n)) == S.ERR_INVALID_ARG
    assert L.scir_host_chunk_plan(4, 4, 4, 0, None, 0, ctypes.byref(n)) == S.ERR_INVALID_ARG
    assert L.scir_host_chunk_plan(4, 4, 4, 1, None, 3, ctypes.byref(n)) == S.ERR_INVALID_ARG
    assert L.scir_host_chunk_plan(4, 4, 4, 1, None, 0, ctypes.byref(n)) == S.OK and n.value == 1


def test_package_never_loads_the_oracle():
    # the oracle is test infrastructure: importing the package and loading its
    # library pulls in neither the oracle module nor libscir_oracle.so
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, scir_gb300 as S; S.load(); "
            "maps = open('/proc/self/maps').read(); "
            "print('oracle' in sys.modules, 'libscir_oracle' in maps, 'libscir_gb300' in maps)")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         timeout=120, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.split() == ["False", "False", "True"]
    # and no package source names it
    pkg = os.path.join(root, "scir_gb300")
    for dirpath, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(dirpath, fn)).read()
                assert "import oracle" not in text and "libscir_oracle" not in text, fn


def test_missing_or_foreign_library_fails_loudly():
    # no library, or a shared object without the C ABI: NativeLibraryError,
    # never a fallback (fresh process: the loaded library is cached)
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = """
import _ctypes
import scir_gb300.build as B, scir_gb300._native as N
for path, build in (("/nonexistent/libscir_gb300.so", False), (_ctypes.__file__, True)):
    B.LIB = path
    try:
        N.load(build_if_missing=build)
        print("loaded")
    except N.NativeLibraryError as e:
        print("missing" if "is missing" in str(e) else "no-abi" if "does not export" in str(e)
              else "other")
"""
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         timeout=120, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.split() == ["missing", "no-abi"]


def test_no_silent_cpu_path():
    with pytest.raises(S.GpuError) as ei:
        S.fir1d_batched_f32_auto(np.zeros((1, 4), np.float32), np.ones(3, np.float32), S.Device.Cpu)
    assert ei.value.kind == "BackendUnavailable"


def test_no_device_is_an_error_not_a_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(S.GpuError) as ei:
        S.fir1d_batched_f32_cuda(np.zeros((1, 4), np.float32), np.ones(3, np.float32))
    assert ei.value.status in (S.ERR_NO_DEVICE, S.ERR_CUDA)
