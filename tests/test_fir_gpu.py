"""Batched FIR on the GPU through the C ABI vs the oracle.

Tolerances: REF_EXACT is compared bit for bit with the f32 restatement of the
reference loop; FP32 (FMA, different summation order) must be within 1e-5
normwise (max|y - y64| / max|y64|) of the FP64 oracle on the same
f32-rounded inputs."""
import numpy as np
import pytest
import scipy.signal as ss

import oracle as O
import scir_gb300 as S
from conftest import normwise_err

pytestmark = pytest.mark.gpu
TOL_FP32 = 1e-5


def _dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def test_known_answer_host_api(cuda):
    # crates/scir-gpu/src/lib.rs:1300-1323 cuda_fir1d_batched_f32_parity_small
    x = np.array([[1.0, 2.0, 3.0, 4.0], [0.5, 0.0, -0.5, -1.0]], np.float32)
    taps = np.array([0.25, 0.5, 0.25], np.float32)
    y = S.fir1d_batched_f32_cuda(x, taps)
    np.testing.assert_allclose(y, [[0.25, 1, 2, 3], [0.125, 0.25, 0, -0.5]], atol=1e-7)
    assert np.array_equal(y, O.fir1d_batched_f32(x, taps))
    assert np.array_equal(S.fir1d_batched_f32_auto(x, taps, S.Device.Cuda), y)


@pytest.mark.parametrize("b,n,k", [(3, 1000, 5), (2, 100, 63), (4, 5000, 300), (2, 10, 20),
                                   (1, 1, 1), (2, 9000, 5000), (5, 4097, 128), (1, 70000, 17)])
def test_ref_exact_is_bit_identical(cuda, b, n, k):
    rng = np.random.default_rng(b * 7919 + n + k)
    x = rng.uniform(-1, 1, (b, n)).astype(np.float32)
    taps = rng.standard_normal(k).astype(np.float32)  # asymmetric: pins orientation
    ref = O.fir1d_batched_f32(x, taps)
    y = S.fir_batched(_dev(x, cuda), _dev(taps, cuda), S.FirMode.REF_CORR,
                      S.Precision.REF_EXACT).cpu().numpy()
    assert np.array_equal(y, ref)
    assert np.array_equal(S.fir1d_batched_f32_cuda(x, taps), ref)


@pytest.mark.parametrize("mode", list(S.FirMode))
@pytest.mark.parametrize("b,n,k", [(3, 3000, 63), (2, 20000, 700), (2, 500, 9)])
def test_fp32_modes_vs_fp64(cuda, mode, b, n, k):
    rng = np.random.default_rng(n + k + int(mode))
    x = rng.uniform(-1, 1, (b, n)).astype(np.float32)
    taps = rng.standard_normal(k).astype(np.float32)
    ref = O.fir_mode_f64(x.astype(np.float64), taps.astype(np.float64), int(mode))
    y = S.fir_batched(_dev(x, cuda), _dev(taps, cuda), mode, S.Precision.FP32).cpu().numpy()
    assert y.shape == ref.shape
    assert normwise_err(y, ref) < TOL_FP32


def test_strided_rows_and_out(cuda):
    import torch
    rng = np.random.default_rng(11)
    big = rng.uniform(-1, 1, (4, 3000)).astype(np.float32)
    taps = rng.standard_normal(31).astype(np.float32)
    xd = _dev(big, cuda)[:, 100:2100]            # ld = 3000, n = 2000
    out = torch.zeros((4, 2500), device=cuda)[:, :2000]
    S.fir_batched(xd, _dev(taps, cuda), S.FirMode.REF_CORR, S.Precision.REF_EXACT, out=out)
    ref = O.fir1d_batched_f32(np.ascontiguousarray(big[:, 100:2100]), taps)
    assert np.array_equal(out.cpu().numpy(), ref)


def test_cfg1_full_size(cuda):
    # 64 channels x 65,536 samples U[-1,1), 63-tap Hamming low-pass at 0.2 Nyquist
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (64, 65536)).astype(np.float32)
    taps = ss.firwin(63, 0.2, window="hamming").astype(np.float32)
    xd, td = _dev(x, cuda), _dev(taps, cuda)
    ref32 = O.fir1d_batched_f32(x, taps)
    y = S.fir_batched(xd, td, S.FirMode.REF_CORR, S.Precision.REF_EXACT).cpu().numpy()
    assert np.array_equal(y, ref32)
    x64, t64 = x.astype(np.float64), taps.astype(np.float64)
    for mode in (S.FirMode.FULL, S.FirMode.VALID):
        ref = O.fir_mode_f64(x64[:8], t64, int(mode))
        yd = S.fir_batched(xd, td, mode, S.Precision.FP32).cpu().numpy()
        assert yd.shape == (64, S.fir_out_len(65536, 63, mode))
        assert normwise_err(yd[:8], ref) < TOL_FP32


def test_cfg3_long_taps_fp32(cuda):
    # 4,095-tap Kaiser(8.6) band-pass 0.1-0.3 Nyquist on sinusoid mixtures, 2 channels
    rng = np.random.default_rng(0)
    n = 65536
    t = np.arange(n)
    x = np.zeros((2, n))
    for c in range(2):
        f = rng.uniform(0, 0.5, 32)
        ph = rng.uniform(0, 2 * np.pi, 32)
        x[c] = np.sum(np.sin(2 * np.pi * f[:, None] * t[None, :] + ph[:, None]), 0) / 32
        x[c] += rng.normal(0, 0.1, n)
    x = x.astype(np.float32)
    taps = ss.firwin(4095, [0.1, 0.3], window=("kaiser", 8.6), pass_zero=False).astype(np.float32)
    ref = O.fir_mode_f64(x.astype(np.float64), taps.astype(np.float64), int(S.FirMode.LFILTER))
    y = S.fir_batched(_dev(x, cuda), _dev(taps, cuda), S.FirMode.LFILTER, S.Precision.FP32)
    assert normwise_err(y.cpu().numpy(), ref) < TOL_FP32


def test_empty_taps_and_empty_batch(cuda):
    import torch
    x = _dev(np.ones((2, 5), np.float32), cuda)
    y = S.fir_batched(x, torch.empty(0, device=cuda), S.FirMode.REF_CORR, S.Precision.FP32)
    assert np.array_equal(y.cpu().numpy(), np.zeros((2, 5), np.float32))
    e = torch.empty((0, 7), device=cuda)
    assert S.fir_batched(e, _dev(np.ones(3, np.float32), cuda)).shape == (0, 7)


def test_shape_errors(cuda):
    x = _dev(np.ones((1, 4), np.float32), cuda)
    with pytest.raises(S.GpuError) as ei:
        S.fir_batched(x, _dev(np.ones(8, np.float32), cuda), S.FirMode.VALID)
    assert ei.value.kind == "ShapeMismatch"


def test_host_pipeline_many_chunks(cuda):
    # enough rows that the host layer splits into several pipelined chunks
    rng = np.random.default_rng(12)
    x = rng.uniform(-1, 1, (600, 40000)).astype(np.float32)
    taps = rng.standard_normal(15).astype(np.float32)
    y = S.fir_batched_host(x, taps, S.FirMode.REF_CORR, S.Precision.REF_EXACT)
    assert np.array_equal(y[::37], O.fir1d_batched_f32(x[::37], taps))


@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
def test_host_calls_back_to_back_new_taps(cuda, pinned):
    # the tap upload is queued on the upload stream without a wait of its own:
    # each call must still filter with its own taps, the caller may overwrite
    # them once a call returns, and a longer tap set grows the tap buffer
    import torch
    rng = np.random.default_rng(13)
    x = rng.uniform(-1, 1, (96, 30000)).astype(np.float32)
    tap_sets = [rng.standard_normal(k).astype(np.float32) for k in (15, 15, 63, 7, 301)]
    buf = torch.empty(301, dtype=torch.float32, pin_memory=pinned).numpy()
    outs = []
    for t in tap_sets:
        buf[:t.size] = t
        outs.append(S.fir_batched_host(x, buf[:t.size], S.FirMode.REF_CORR,
                                       S.Precision.REF_EXACT))
        buf[:] = np.nan  # overwritten as soon as the call returns
    for t, y in zip(tap_sets, outs):
        assert np.array_equal(y[::19], O.fir1d_batched_f32(x[::19], t))


# ---------------------------------------------------------------- tensor cores
# BF16X6 (three bf16 terms, six products) and FP16X3 (scaled fp16 hi+lo,
# three products, 22 significant bits per operand) must meet the FP32 bound
# of 1e-5; BF16X3 (bf16 hi+lo, three products) carries ~16 significant bits
# per product and is held to a stated bound of 3e-5 normwise (about 7e-6 on
# the long-tap band-pass workload).
TOL_BF16X3 = 3e-5
TC_FORMS = [(S.Precision.FP16X3, TOL_FP32), (S.Precision.BF16X6, TOL_FP32),
            (S.Precision.BF16X3, TOL_BF16X3)]
TC_TOL = dict(TC_FORMS)


@pytest.mark.parametrize("prec,tol", TC_FORMS, ids=lambda v: getattr(v, "name", str(v)))
@pytest.mark.parametrize("mode", list(S.FirMode))
@pytest.mark.parametrize("b,n,k", [(3, 1000, 63), (130, 3000, 700), (2, 40000, 4095), (1, 300, 1)])
def test_tensor_core_vs_fp64(cuda, prec, tol, mode, b, n, k):
    if mode == S.FirMode.VALID and n < k:
        pytest.skip("VALID needs n >= k")
    rng = np.random.default_rng(b + n + k + int(mode))
    x = rng.uniform(-1, 1, (b, n)).astype(np.float32)
    taps = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    ref = O.fir_mode_f64(x.astype(np.float64), taps.astype(np.float64), int(mode))
    y = S.fir_batched(_dev(x, cuda), _dev(taps, cuda), mode, prec).cpu().numpy()
    assert y.shape == ref.shape
    err = normwise_err(y, ref)
    assert err < tol, err


def test_tensor_core_cfg3_bandpass(cuda):
    # the long-tap configuration's filter and signal family, 130 channels
    rng = np.random.default_rng(0)
    n = 32768
    t = np.arange(n)
    x = np.zeros((130, n))
    for c in range(130):
        f = rng.uniform(0, 0.5, 32)
        ph = rng.uniform(0, 2 * np.pi, 32)
        x[c] = np.sum(np.sin(2 * np.pi * f[:, None] * t[None, :] + ph[:, None]), 0) / 32
        x[c] += rng.normal(0, 0.1, n)
    x = x.astype(np.float32)
    taps = ss.firwin(4095, [0.1, 0.3], window=("kaiser", 8.6), pass_zero=False).astype(np.float32)
    rows = [0, 1, 64, 127, 128, 129]
    ref = O.fir_mode_f64(x[rows].astype(np.float64), taps.astype(np.float64), int(S.FirMode.LFILTER))
    xd, td = _dev(x, cuda), _dev(taps, cuda)
    for prec in (S.Precision.BF16X3, S.Precision.BF16X6, S.Precision.FP16X3, S.Precision.AUTO):
        y = S.fir_batched(xd, td, S.FirMode.LFILTER, prec).cpu().numpy()
        assert normwise_err(y[rows], ref) < 1e-5, prec


def test_fp16x3_scaling(cuda):
    # FP16X3 scales every row (and the taps) by a power of two from its
    # largest finite magnitude: rows of 1e6 and 1e-20 in one batch, an
    # all-zero row, taps of 1e-4 scale; each row is held to 1e-5 of itself
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (6, 20000))
    x[1] *= 1e6
    x[2] *= 1e-20
    x[3] = 0.0
    x[4, ::7] *= 1e3  # a row whose largest samples sit on a sparse comb
    x = x.astype(np.float32)
    taps = (rng.standard_normal(1500) * 1e-4).astype(np.float32)
    ref = O.fir_mode_f64(x.astype(np.float64), taps.astype(np.float64), int(S.FirMode.LFILTER))
    y = S.fir_batched(_dev(x, cuda), _dev(taps, cuda), S.FirMode.LFILTER,
                      S.Precision.FP16X3).cpu().numpy()
    assert np.all(y[3] == 0.0)
    for r in (0, 1, 2, 4, 5):
        assert normwise_err(y[r], ref[r]) < TOL_FP32, r


def test_fp16x3_extreme_range(cuda):
    # rows at the ends of float's range: 1e36 (scaled down by 2^-113 .. so its
    # largest sample lands in [2^14, 2^15) -- a clamped shift would overflow
    # fp16) and 1e-36 (scaled up by about 2^134); taps of unit scale keep every
    # output a normal float
    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, (6, 12000))
    x[0] *= 1e36
    x[1] *= 1e-36
    x[2] *= 1e30
    x[3] *= 1e-30
    x[4, 100] = 3e38  # one sample near float's maximum in an otherwise small row
    x = x.astype(np.float32)
    taps = (rng.standard_normal(1500) / 40).astype(np.float32)
    ref = O.fir_mode_f64(x.astype(np.float64), taps.astype(np.float64), int(S.FirMode.LFILTER))
    y = S.fir_batched(_dev(x, cuda), _dev(taps, cuda), S.FirMode.LFILTER,
                      S.Precision.FP16X3).cpu().numpy()
    for r in (0, 1, 2, 3, 5):
        assert np.all(np.isfinite(y[r])), r
        assert normwise_err(y[r], ref[r]) < TOL_FP32, r
    # the 3e38 row: one scale per row, set by the spike, so the unit-size
    # samples fall below fp16's range -- the bound is normwise, relative to
    # the row's largest output, and holds
    assert np.all(np.isfinite(y[4]))
    assert normwise_err(y[4], ref[4]) < TOL_FP32


@pytest.mark.parametrize("prec", [S.Precision.FP16X3, S.Precision.BF16X6, S.Precision.FP32])
def test_tensor_core_dc_lowpass(cuda, prec):
    # a constant input through a low-pass filter with positive taps: every
    # partial sum grows the same way, so a rounding bias in the accumulation
    # would add up instead of cancelling
    x = np.ones((4, 30000), np.float32)
    x[1] = 0.75
    x[2, :] = np.linspace(0.5, 1.0, 30000, dtype=np.float32)
    x[3] = 3.0
    taps = ss.firwin(4095, 0.01).astype(np.float32)
    ref = O.fir_mode_f64(x.astype(np.float64), taps.astype(np.float64), int(S.FirMode.LFILTER))
    y = S.fir_batched(_dev(x, cuda), _dev(taps, cuda), S.FirMode.LFILTER, prec).cpu().numpy()
    assert normwise_err(y, ref) < TOL_FP32


@pytest.mark.parametrize("prec", [S.Precision.BF16X3, S.Precision.BF16X6, S.Precision.FP16X3])
@pytest.mark.parametrize("k", [2, 3, 16, 17, 64, 1025, 4000])
def test_tensor_core_unaligned_rows(cuda, prec, k):
    # x starting one float past a 16-byte boundary (scalar signal loads), an
    # odd output row stride (scalar stores), 260 channels (a partial third
    # channel group) and 2,500 samples (a partial output window); 4,000 taps
    # take the one-phase-per-tile shape (N = 256)
    import torch
    rng = np.random.default_rng(k)
    big = rng.uniform(-1, 1, (260, 2502)).astype(np.float32)
    taps = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    xd = _dev(big, cuda)[:, 1:2501]
    out = torch.zeros((260, 2503), device=cuda)[:, :2500]
    ref = O.fir_mode_f64(big[:, 1:2501].astype(np.float64), taps.astype(np.float64),
                         int(S.FirMode.LFILTER))
    S.fir_batched(xd, _dev(taps, cuda), S.FirMode.LFILTER, prec, out=out)
    assert normwise_err(out.cpu().numpy(), ref) < TC_TOL[prec]


@pytest.mark.parametrize("k", [1025, 4000])
def test_tensor_core_five_groups_and_graph(cuda, k):
    # 640 channels = 5 channel groups with one row at its own scale, rows of
    # the first and last groups against FP64; then the same call recorded in
    # a CUDA graph (the max pass, both splits and the persistent launch) and
    # replayed bit for bit
    import torch
    rng = np.random.default_rng(k)
    x = rng.uniform(-1, 1, (640, 6000)).astype(np.float32)
    x[300] *= 1e4  # a row with its own scale in the second chunk
    taps = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    rows = [0, 255, 256, 300, 639]
    ref = O.fir_mode_f64(x[rows].astype(np.float64), taps.astype(np.float64), int(S.FirMode.LFILTER))
    xd, td = _dev(x, cuda), _dev(taps, cuda)
    for prec in (S.Precision.FP16X3, S.Precision.BF16X3):
        y = S.fir_batched(xd, td, S.FirMode.LFILTER, prec).cpu().numpy()
        for i, r in enumerate(rows):
            assert normwise_err(y[r], ref[i]) < TC_TOL[prec], (prec, r)
    S.init(0)
    s = torch.cuda.Stream()
    eager = torch.zeros((640, 6000), device=cuda)
    out = torch.zeros_like(eager)
    with torch.cuda.stream(s):
        S.fir_batched(xd, td, S.FirMode.LFILTER, S.Precision.FP16X3, out=eager, stream=s)
        s.synchronize()
        with S.GraphCapture(s) as g:
            S.fir_batched(xd, td, S.FirMode.LFILTER, S.Precision.FP16X3, out=out, stream=s)
        out.fill_(float("nan"))
        g.launch()
        s.synchronize()
    assert torch.equal(out, eager)
    g.close()


def test_tensor_core_strided_and_repeat(cuda):
    import torch
    rng = np.random.default_rng(21)
    big = rng.uniform(-1, 1, (140, 5004)).astype(np.float32)
    taps = (rng.standard_normal(300) / 17).astype(np.float32)
    xd = _dev(big, cuda)[:, :5000]
    out = torch.zeros((140, 5100), device=cuda)[:, :5000]
    ref = O.fir_mode_f64(big[:, :5000].astype(np.float64), taps.astype(np.float64),
                         int(S.FirMode.REF_CORR))
    for _ in range(2):  # the second call reuses the stream-ordered scratch pool
        S.fir_batched(xd, _dev(taps, cuda), S.FirMode.REF_CORR, S.Precision.BF16X6, out=out)
        assert normwise_err(out.cpu().numpy(), ref) < TOL_FP32
