"""Second-order-section filtering on the GPU vs the oracle.

FP64_EXACT on f64 data is compared bit for bit with the restated reference
DF2T loop.  FP32 data with FP64 state must be within 1e-5 normwise of the FP64
oracle run on the same f32-rounded input.  The all-FP32 mode is reported, not
bounded tightly (poles within 2e-4 of the unit circle)."""
import numpy as np
import pytest
import scipy.signal as ss

import oracle as O
import scir_gb300 as S
from conftest import normwise_err

pytestmark = pytest.mark.gpu
TOL = 1e-5
SOS5 = ss.butter(8, [0.001, 0.002], btype="bandpass", output="sos")


def _dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


@pytest.mark.parametrize("case", ["low_pass", "high_pass", "band_pass", "band_stop"])
def test_strain_golden_bit_identical(cuda, golden_strain, case):
    sos = golden_strain[f"sos_{case}"]
    x = golden_strain["x"]
    y = S.sosfilt(sos, x)
    assert np.array_equal(y, O.sosfilt_f64(sos, x)[0])
    np.testing.assert_allclose(y, golden_strain[f"y_{case}"], atol=1e-12, rtol=0)


def test_signal_fixtures(cuda, golden_signal):
    f = golden_signal
    y = S.sosfilt(f["butter_sos"], f["sosfilt_input"])
    np.testing.assert_allclose(y, f["sosfilt_output"], atol=1e-6, rtol=1e-6)
    y = S.filtfilt(f["butter_sos"], f["sosfilt_input"])
    np.testing.assert_allclose(y, f["filtfilt_output"], atol=1e-6, rtol=1e-6)
    assert np.array_equal(y, O.filtfilt_ref_f64(f["butter_sos"], f["sosfilt_input"])[0])
    for name in ["cheby", "bessel", "butter_hp", "cheby_hp", "bessel_hp", "notch"]:
        y = S.sosfilt(f[f"{name}_sos"], f["sosfilt_input"])
        np.testing.assert_allclose(y, f[f"{name}_output"], atol=1e-12, rtol=1e-12)


@pytest.mark.parametrize("nsec", [1, 3, 8, 9, 16, 32])
def test_exact_f64_any_section_count(cuda, nsec):
    rng = np.random.default_rng(nsec)
    sos = np.zeros((nsec, 6))
    for i in range(nsec):  # stable random sections
        r, th = rng.uniform(0.3, 0.95), rng.uniform(0, np.pi)
        sos[i] = [rng.standard_normal(), rng.standard_normal(), rng.standard_normal(), 1.0,
                  -2 * r * np.cos(th), r * r]
    x = rng.standard_normal((70, 777))
    y = S.sosfilt_f64(sos, _dev(x, cuda)).cpu().numpy()
    assert np.array_equal(y, O.sosfilt_f64(sos, x))


def test_cfg5_fp32_data_fp64_state(cuda):
    rng = np.random.default_rng(0)
    x = rng.standard_normal((96, 131072)).astype(np.float32)
    ref = O.sosfilt_f64(SOS5, x.astype(np.float64))
    y = S.sosfilt_f32(SOS5, _dev(x, cuda), precision=S.SosPrecision.FP64).cpu().numpy()
    assert normwise_err(y, ref) < TOL
    ye = S.sosfilt_f32(SOS5, _dev(x, cuda), precision=S.SosPrecision.FP64_EXACT).cpu().numpy()
    assert normwise_err(ye, ref) < TOL
    y32 = S.sosfilt_f32(SOS5, _dev(x, cuda), precision=S.SosPrecision.FP32).cpu().numpy()
    e32 = normwise_err(y32, ref)
    assert np.isfinite(y32).all() and e32 > TOL  # all-FP32 cannot hold 1e-5 on these poles
    print(f"all-FP32 sosfilt normwise error {e32:.3e}")


def test_state_chaining(cuda):
    import torch
    rng = np.random.default_rng(1)
    x = rng.standard_normal((33, 5000))
    xd = _dev(x, cuda)
    y1, zf = S.sosfilt_f64(SOS5, xd[:, :2000].contiguous(), return_zf=True)
    y2 = S.sosfilt_f64(SOS5, xd[:, 2000:].contiguous(), zi=zf)
    full = torch.cat([y1, y2], 1).cpu().numpy()
    assert np.array_equal(full, O.sosfilt_f64(SOS5, x))
    zi = rng.standard_normal((33, 8, 2))
    y, zf = S.sosfilt_f64(SOS5, xd, zi=_dev(zi, cuda), return_zf=True)
    yr, zr = O.sosfilt_f64(SOS5, x, zi=zi, return_zf=True)
    assert np.array_equal(y.cpu().numpy(), yr)
    assert np.array_equal(zf.cpu().numpy(), zr)


@pytest.mark.parametrize("padlen", [None, 0, 200])
def test_sosfiltfilt_odd_vs_oracle(cuda, padlen):
    rng = np.random.default_rng(2)
    x = rng.standard_normal((40, 20000))
    ref = O.sosfiltfilt_f64(SOS5, x, padlen=padlen)
    y = S.sosfiltfilt_f64(SOS5, _dev(x, cuda), padlen=padlen).cpu().numpy()
    assert normwise_err(y, ref) < 1e-13
    y32 = S.sosfiltfilt_f32(SOS5, _dev(x.astype(np.float32), cuda), padlen=padlen).cpu().numpy()
    ref32 = O.sosfiltfilt_f64(SOS5, x.astype(np.float32).astype(np.float64), padlen=padlen)
    assert normwise_err(y32, ref32) < TOL


def test_sosfiltfilt_vs_scipy_and_in_place(cuda):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((5, 9000))
    xd = _dev(x, cuda)
    y = S.sosfiltfilt_f64(SOS5, xd).cpu().numpy()
    assert normwise_err(y, ss.sosfiltfilt(SOS5, x, axis=1)) < 1e-12
    S.sosfiltfilt_f64(SOS5, xd, out=xd)  # y aliases x
    assert normwise_err(xd.cpu().numpy(), y) == 0.0


def test_unpadded_is_reference_filtfilt(cuda):
    rng = np.random.default_rng(4)
    x = rng.standard_normal((7, 3000))
    y = S.sosfiltfilt_f64(SOS5, _dev(x, cuda), padtype=S.PadType.NONE).cpu().numpy()
    assert np.array_equal(y, O.filtfilt_ref_f64(SOS5, x))


def test_short_signal_rejected(cuda):
    x = _dev(np.ones((2, 51)), cuda)
    with pytest.raises(S.GpuError) as ei:
        S.sosfiltfilt_f64(SOS5, x)
    assert ei.value.kind == "ShapeMismatch"


# ---------------------------------------------------------------- coupled form
# FP32 state in coupled (modal) form with FP64-derived increments: <= 1e-5
# normwise vs the FP64 oracle on the near-unit-circle band-pass (cfg 5).
def test_cfg5_coupled_fp32(cuda):
    rng = np.random.default_rng(0)
    x = rng.standard_normal((96, 131072)).astype(np.float32)
    ref = O.sosfilt_f64(SOS5, x.astype(np.float64))
    y = S.sosfilt_f32(SOS5, _dev(x, cuda), precision=S.SosPrecision.FP32_COUPLED).cpu().numpy()
    assert normwise_err(y, ref) < TOL


@pytest.mark.parametrize("sos", [ss.butter(5, 0.2, output="sos"),            # a real-pole section
                                 ss.cheby1(6, 1, [0.1, 0.3], btype="bandpass", output="sos"),
                                 ss.butter(4, 0.3, btype="highpass", output="sos")])
def test_coupled_general_filters(cuda, sos):
    rng = np.random.default_rng(5)
    x = rng.standard_normal((40, 20000)).astype(np.float32)
    ref = O.sosfilt_f64(sos, x.astype(np.float64))
    y = S.sosfilt_f32(sos, _dev(x, cuda), precision=S.SosPrecision.FP32_COUPLED).cpu().numpy()
    assert normwise_err(y, ref) < TOL


def test_coupled_state_chaining_and_filtfilt(cuda):
    import torch
    rng = np.random.default_rng(6)
    x = rng.standard_normal((33, 30000)).astype(np.float32)
    xd = _dev(x, cuda)
    P = S.SosPrecision.FP32_COUPLED
    zi = rng.standard_normal((33, 8, 2)) * 0.01
    y1, zf = S.sosfilt_f32(SOS5, xd[:, :12000].contiguous(), zi=_dev(zi, cuda), return_zf=True,
                           precision=P)
    y2 = S.sosfilt_f32(SOS5, xd[:, 12000:].contiguous(), zi=zf, precision=P)
    full = torch.cat([y1, y2], 1).cpu().numpy()
    ref = O.sosfilt_f64(SOS5, x.astype(np.float64), zi=zi)
    assert normwise_err(full, ref) < TOL
    ref_zf = O.sosfilt_f64(SOS5, x[:, :12000].astype(np.float64), zi=zi, return_zf=True)[1]
    assert np.max(np.abs(zf.cpu().numpy() - ref_zf)) < 1e-4 * np.max(np.abs(ref_zf))
    yff = S.sosfiltfilt_f32(SOS5, xd, precision=P).cpu().numpy()
    assert normwise_err(yff, O.sosfiltfilt_f64(SOS5, x.astype(np.float64))) < TOL


# --------------------------------------------------- pipelined FP32 cascade
# The FP32 modes split the cascade over the warps of a CTA and move tiles of
# 32 samples through a shared-memory ring (full tiles by a fast path, edge
# tiles element by element); these lengths cover short signals, tile-boundary
# remainders, section counts that round up with identity sections and both
# directions of sosfiltfilt.  A misplaced sample shows as an O(1) error.
@pytest.mark.parametrize("n", [1, 2, 5, 7, 8, 31, 32, 33, 38, 39, 64, 100, 1000, 20003])
@pytest.mark.parametrize("order", [1, 4, 16, 18, 40])
def test_fp32_cascade_lengths(cuda, n, order):
    sos = ss.butter(order, 0.2, output="sos")
    rng = np.random.default_rng(n * 100 + order)
    x = rng.standard_normal((9, n)).astype(np.float32)
    x64 = x.astype(np.float64)
    zi = rng.standard_normal((9, sos.shape[0], 2)) * 0.1
    ref = O.sosfilt_f64(sos, x64)
    ref_zi = O.sosfilt_f64(sos, x64, zi=zi)
    for prec, tol in ((S.SosPrecision.FP32_COUPLED, 1e-5), (S.SosPrecision.FP32, 1e-4)):
        y = S.sosfilt_f32(sos, _dev(x, cuda), precision=prec).cpu().numpy()
        assert normwise_err(y, ref) < tol, (prec, "sosfilt")
        y = S.sosfilt_f32(sos, _dev(x, cuda), zi=_dev(zi, cuda), precision=prec).cpu().numpy()
        assert normwise_err(y, ref_zi) < tol, (prec, "sosfilt zi")
        padlen = None if n > 3 * (2 * sos.shape[0] + 1) else 0
        yff = S.sosfiltfilt_f32(sos, _dev(x, cuda), padlen=padlen, precision=prec).cpu().numpy()
        # a 20-section cascade run forward and backward in FP32 state: measured 1.2e-5 .. 3.9e-5
        tol_ff = tol * (5 if sos.shape[0] > 16 else 1)
        assert normwise_err(yff, O.sosfiltfilt_f64(sos, x64, padlen=padlen)) < tol_ff, (prec, "ff")
        ynp = S.sosfiltfilt_f32(sos, _dev(x, cuda), padtype=S.PadType.NONE, precision=prec).cpu().numpy()
        ref_np = O.filtfilt_ref_f64(sos, x64)
        if np.max(np.abs(ref_np)) > 1e-30:  # order 40 at n <= 2: ~1e-46, below FP32's range
            assert normwise_err(ynp, ref_np) < tol_ff, (prec, "unpadded")
        else:
            assert np.all(np.abs(ynp) < 1e-30), (prec, "unpadded, underflow")


# Two channels per lane (rows l and l + 32 of a 64-channel CTA): batches
# that fill both halves, leave the second half partly empty, and span many
# CTAs -- including a full-size-width case of 4,160 channels (65 CTAs).
@pytest.mark.parametrize("batch", [33, 64, 100, 4160])
def test_fp32_pipe_channel_halves(cuda, batch):
    import torch
    rng = np.random.default_rng(batch)
    n = 3000 if batch > 1000 else 7000
    x = rng.standard_normal((batch, n)).astype(np.float32)
    rows = sorted({0, 31, 32, 33, 63, batch // 2, batch - 33, batch - 32, batch - 1} &
                  set(range(batch)))
    x64 = x[rows].astype(np.float64)
    P = S.SosPrecision.FP32_COUPLED
    y = S.sosfilt_f32(SOS5, _dev(x, cuda), precision=P).cpu().numpy()
    assert normwise_err(y[rows], O.sosfilt_f64(SOS5, x64)) < TOL
    # every row against the row-by-row FP32 result of single-channel calls
    for r in rows[:4]:
        yr = S.sosfilt_f32(SOS5, _dev(x[r:r + 1], cuda), precision=P).cpu().numpy()
        assert np.array_equal(yr[0], y[r])
    xd = _dev(x, cuda)
    S.sosfiltfilt_f32(SOS5, xd, precision=P, out=xd)  # in place
    assert normwise_err(xd.cpu().numpy()[rows], O.sosfiltfilt_f64(SOS5, x64)) < TOL
    ydf = S.sosfilt_f32(SOS5, _dev(x, cuda), precision=S.SosPrecision.FP32).cpu().numpy()
    assert np.all(np.isfinite(ydf))
    del torch


# ----------------------------------------- block-parallel time scan (few, long channels)
# Up to 64 channels of long signals are cut into blocks filtered from zero
# state, the block states are chained by a scan with the cascade's L-step
# transition matrix, and every block is filtered again from its true state.
# FP32-state modes keep their 1e-5 bound; FP64 state takes the path with
# blocks of >= 65,536 samples and a stated bound of 1e-9; FP64_EXACT stays
# sequential (bit-identical to the reference order).
@pytest.mark.parametrize("batch,n", [(1, 1 << 20), (2, 3_000_017), (5, 700_001), (1, 1 << 24),
                                     (3, 200_000)])
def test_block_scan_fp32_coupled(cuda, batch, n):
    rng = np.random.default_rng(batch + n)
    x = rng.standard_normal((batch, n)).astype(np.float32)
    x64 = x.astype(np.float64)
    P = S.SosPrecision.FP32_COUPLED
    zi = rng.standard_normal((batch, 8, 2)) * 0.01
    y, zf = S.sosfilt_f32(SOS5, _dev(x, cuda), zi=_dev(zi, cuda), return_zf=True, precision=P)
    ref, ref_zf = O.sosfilt_f64(SOS5, x64, zi=zi, return_zf=True)
    assert normwise_err(y.cpu().numpy(), ref) < TOL
    assert np.max(np.abs(zf.cpu().numpy() - ref_zf)) < 1e-4 * np.max(np.abs(ref_zf))
    # chained: the second half continues from the first half's final state
    h = n // 2
    y1, z1 = S.sosfilt_f32(SOS5, _dev(x[:, :h], cuda), return_zf=True, precision=P)
    y2 = S.sosfilt_f32(SOS5, _dev(x[:, h:], cuda), zi=z1, precision=P)
    full = np.concatenate([y1.cpu().numpy(), y2.cpu().numpy()], 1)
    assert normwise_err(full, O.sosfilt_f64(SOS5, x64)) < TOL


def test_block_scan_fp64_state(cuda):
    rng = np.random.default_rng(11)
    x = rng.standard_normal((2, 9_000_000)).astype(np.float32)
    ref = O.sosfilt_f64(SOS5, x.astype(np.float64))
    y = S.sosfilt_f32(SOS5, _dev(x, cuda), precision=S.SosPrecision.FP64).cpu().numpy()
    assert normwise_err(y, ref) < 1e-6  # f32 outputs: their rounding dominates
    # f64 data, FP64 state: the scan's own bound
    xd = rng.standard_normal((1, 5_000_000))
    yd = S.sosfilt_f64(SOS5, _dev(xd, cuda), precision=S.SosPrecision.FP64).cpu().numpy()
    assert normwise_err(yd, O.sosfilt_f64(SOS5, xd)) < 1e-9


def test_block_scan_exact_and_in_place_stay_sequential(cuda):
    rng = np.random.default_rng(12)
    xd = rng.standard_normal((1, 2_000_000))
    y = S.sosfilt_f64(SOS5, _dev(xd, cuda), precision=S.SosPrecision.FP64_EXACT).cpu().numpy()
    assert np.array_equal(y, O.sosfilt_f64(SOS5, xd))  # the reference order, bit for bit
    x = rng.standard_normal((1, 1 << 20)).astype(np.float32)
    xg = _dev(x, cuda)
    S.sosfilt_f32(SOS5, xg, precision=S.SosPrecision.FP32_COUPLED, out=xg)  # in place
    assert normwise_err(xg.cpu().numpy(), O.sosfilt_f64(SOS5, x.astype(np.float64))) < TOL
