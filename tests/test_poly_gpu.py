"""Polyphase upfirdn / resample_poly on the GPU vs the oracle.

FP32 paths must be within 1e-5 normwise of the FP64 oracle on the same
f32-rounded inputs and taps; the reference-signature f64 resample_poly(2, 3)
is compared bit for bit with the restated reference loop."""
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


@pytest.mark.parametrize("up,down,kh,n", [(3, 2, 11, 777), (1, 4, 9, 500), (5, 1, 22, 301),
                                          (7, 3, 4, 1000), (160, 147, 3201, 5000), (2, 3, 31, 64),
                                          (1, 1, 5, 100), (4, 1, 64, 2000), (300, 7, 50, 300)])
def test_upfirdn_vs_oracle(cuda, up, down, kh, n):
    rng = np.random.default_rng(up * 1000 + down + kh)
    h = rng.standard_normal(kh).astype(np.float32)
    x = rng.standard_normal((3, n)).astype(np.float32)
    ref = O.upfirdn_f64(h.astype(np.float64), x.astype(np.float64), up, down)
    y = S.upfirdn(_dev(h, cuda), _dev(x, cuda), up, down).cpu().numpy()
    assert y.shape == ref.shape
    assert normwise_err(y, ref) < TOL_FP32


@pytest.mark.parametrize("up,down", [(160, 147), (3, 2), (2, 3), (1, 3), (5, 4), (4, 6)])
def test_resample_default_design_vs_oracle(cuda, up, down):
    rng = np.random.default_rng(up + down)
    x = rng.standard_normal((4, 20000)).astype(np.float32)
    h64 = S.resample_poly_default_taps(up, down, design=0)
    h32 = h64.astype(np.float32)
    ref = O.resample_poly_fast_f64(x.astype(np.float64), up, down, h32.astype(np.float64))
    y = S.resample_poly_f32(_dev(x, cuda), up, down).cpu().numpy()
    assert y.shape == ref.shape
    assert normwise_err(y, ref) < TOL_FP32
    # and against SciPy itself (FP64 design, FP64 data): the gap is the f32 rounding
    assert normwise_err(y, ss.resample_poly(x.astype(np.float64), up, down, axis=1)) < 1e-5


def test_resample_cfg2_full_size(cuda):
    # 256 channels x 1,048,576 N(0,1) samples, 160/147, SciPy default 3,201-tap Kaiser(5)
    import torch
    g = torch.Generator(device=cuda).manual_seed(0)
    x = torch.randn((256, 1048576), device=cuda, generator=g)
    y = S.resample_poly_f32(x, 160, 147)
    assert y.shape == (256, 1141308)
    rows = [0, 255]
    xs = x[rows].cpu().numpy().astype(np.float64)
    h = S.resample_poly_default_taps(160, 147).astype(np.float32).astype(np.float64)
    ref = O.resample_poly_fast_f64(xs, 160, 147, h)
    assert normwise_err(y[rows].cpu().numpy(), ref) < TOL_FP32
    del x, y
    torch.cuda.empty_cache()


def test_resample_explicit_taps_and_copy(cuda):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((2, 1000)).astype(np.float32)
    h = (rng.standard_normal(33) * 3).astype(np.float32)
    ref = O.resample_poly_fast_f64(x.astype(np.float64), 3, 2, h.astype(np.float64))
    y = S.resample_poly_f32(_dev(x, cuda), 3, 2, h=_dev(h, cuda)).cpu().numpy()
    assert normwise_err(y, ref) < TOL_FP32
    y = S.resample_poly_f32(_dev(x, cuda), 5, 5).cpu().numpy()
    assert np.array_equal(y, x)


def test_reference_resample_poly_2_3_bit_identical(cuda, golden_signal, golden_resample23):
    # crates/scir-signal/src/lib.rs:313-362 with its own 31-value table (the
    # literals extracted from the reference source), f64, through the
    # restated zero-stuff / full convolution / decimate loop
    x = golden_signal["sosfilt_input"]
    h = np.array([float(s) for s in golden_resample23["literals"]])
    ref = O.resample_poly_ref_f64(x, 2, 3, h)[0]
    y = S.resample_poly(x, 2, 3)
    assert np.array_equal(y, ref)
    # crates/scir-signal/src/lib.rs:655-668 tolerance against SciPy's fixture
    np.testing.assert_allclose(y, golden_signal["resample_poly_output"], atol=2e-2, rtol=1e-6)
    rng = np.random.default_rng(4)
    xb = rng.standard_normal((3, 5001))
    assert np.array_equal(S.resample_poly(xb, 2, 3), O.resample_poly_ref_f64(xb, 2, 3, h))
    # ragged lengths around the decimation period, and a long row
    for n in (1, 2, 3, 4, 5, 31, 32, 33, 100003):
        xr = rng.standard_normal((2, n))
        assert np.array_equal(S.resample_poly(xr, 2, 3), O.resample_poly_ref_f64(xr, 2, 3, h)), n
    with pytest.raises(S.GpuError):
        S.resample_poly(xb, 160, 147)


def test_resample_host_pipeline(cuda):
    rng = np.random.default_rng(5)
    x = rng.standard_normal((40, 300000)).astype(np.float32)
    y = S.resample_poly_host(x, 160, 147)
    h = S.resample_poly_default_taps(160, 147).astype(np.float32).astype(np.float64)
    ref = O.resample_poly_fast_f64(x[::13].astype(np.float64), 160, 147, h)
    assert normwise_err(y[::13], ref) < TOL_FP32


@pytest.mark.parametrize("pad", [0, 3])
def test_resample_padded_output_rows(cuda, pad):
    # rows padded to a multiple of 4 floats (16-byte aligned): outputs leave
    # shared memory by bulk copies, with a row end that is not a multiple of 4;
    # pad 3 gives an odd row stride and the per-lane store path
    import torch
    rng = np.random.default_rng(6)
    x = rng.standard_normal((5, 20000)).astype(np.float32)
    n_out = S.resample_poly_out_len(20000, 160, 147)
    assert n_out % 4 != 0
    width = (n_out + 3) // 4 * 4 + pad
    big = torch.full((5, width), 7.0, device=cuda)
    y = S.resample_poly_f32(_dev(x, cuda), 160, 147, out=big[:, :n_out])
    h = S.resample_poly_default_taps(160, 147).astype(np.float32).astype(np.float64)
    ref = O.resample_poly_fast_f64(x.astype(np.float64), 160, 147, h)
    assert normwise_err(y.cpu().numpy(), ref) < TOL_FP32
    assert bool((big[:, n_out:] == 7.0).all())  # nothing written past the row end


# ------------------------------------------------- tensor-core polyphase (BF16X3)
# split-bf16 products (x1c1 + x1c2 + x2c1) with FP32 accumulation: each
# operand keeps ~16 significant bits, so the stated bound of this form is
# 2e-5 normwise (measured 7e-6 .. 1.0e-5 on ~21-tap phases)
TOL_TC = 2e-5


@pytest.mark.parametrize("up,down", [(160, 147), (3, 2), (5, 4)])
@pytest.mark.parametrize("batch,n", [(3, 1000), (130, 20000), (256, 4100), (5, 4)])
def test_resample_tc_vs_oracle(cuda, up, down, batch, n):
    rng = np.random.default_rng(batch * 7 + n + up)
    x = rng.standard_normal((batch, n)).astype(np.float32)
    h32 = S.resample_poly_default_taps(up, down, design=0).astype(np.float32)
    ref = O.resample_poly_fast_f64(x.astype(np.float64), up, down, h32.astype(np.float64))
    y = S.resample_poly_f32(_dev(x, cuda), up, down, precision=S.Precision.BF16X3).cpu().numpy()
    assert y.shape == ref.shape
    err = normwise_err(y, ref)
    print(f"tensor-core resample {up}/{down} {batch}x{n}: normwise error {err:.2e}")
    assert err < TOL_TC


def test_upfirdn_tc_short_filter(cuda):
    rng = np.random.default_rng(5)
    h = rng.standard_normal(64).astype(np.float32)
    x = rng.standard_normal((129, 3000)).astype(np.float32)
    ref = O.upfirdn_f64(h.astype(np.float64), x.astype(np.float64), 4, 1)
    y = S.upfirdn(_dev(h, cuda), _dev(x, cuda), 4, 1, precision=S.Precision.BF16X3).cpu().numpy()
    assert y.shape == ref.shape
    assert normwise_err(y, ref) < TOL_TC


def test_resample_tc_padded_rows(cuda):
    import torch
    rng = np.random.default_rng(9)
    x = rng.standard_normal((140, 5000)).astype(np.float32)
    xp = torch.zeros((140, 5004), device=cuda)
    xp[:, :5000] = _dev(x, cuda)
    n_out = S.resample_poly_out_len(5000, 160, 147)
    ld = n_out + 12 + (-n_out) % 4  # a row pitch of whole 16-byte units
    out = torch.full((140, ld), 7.0, device=cuda)
    S.resample_poly_f32(xp[:, :5000], 160, 147, precision=S.Precision.BF16X3, out=out[:, :n_out])
    h32 = S.resample_poly_default_taps(160, 147).astype(np.float32).astype(np.float64)
    ref = O.resample_poly_fast_f64(x.astype(np.float64), 160, 147, h32)
    got = out.cpu().numpy()
    assert normwise_err(got[:, :n_out], ref) < TOL_TC
    assert np.all(got[:, n_out:] == 7.0)  # the row padding is not written


def test_resample_tc_refuses_unserved_shape(cuda):
    # 2/3 with the default 61-tap design: a 32-output segment spans more than
    # the 64-sample window, so the tensor-core path reports UNSUPPORTED rather
    # than running anything else
    x = np.zeros((4, 1000), np.float32)
    with pytest.raises(S.GpuError):
        S.resample_poly_f32(_dev(x, cuda), 2, 3, precision=S.Precision.BF16X3)
    # input rows without a 16-byte pitch cannot be read by the tensor map
    x = np.zeros((4, 1001), np.float32)
    with pytest.raises(S.GpuError):
        S.resample_poly_f32(_dev(x, cuda), 160, 147, precision=S.Precision.BF16X3)
    # FP16X3 is a form of the FIR entry points only
    x = np.zeros((4, 1024), np.float32)
    with pytest.raises(S.GpuError):
        S.resample_poly_f32(_dev(x, cuda), 160, 147, precision=S.Precision.FP16X3)


def test_resample_tc_cfg2_full_size(cuda):
    import torch
    g = torch.Generator(device=cuda).manual_seed(0)
    x = torch.randn((256, 1048576), device=cuda, generator=g)
    y = S.resample_poly_f32(x, 160, 147, precision=S.Precision.BF16X3)
    assert y.shape == (256, 1141308)
    rows = [0, 129, 255]
    xs = x[rows].cpu().numpy().astype(np.float64)
    h = S.resample_poly_default_taps(160, 147).astype(np.float32).astype(np.float64)
    ref = O.resample_poly_fast_f64(xs, 160, 147, h)
    err = normwise_err(y[rows].cpu().numpy(), ref)
    print(f"tensor-core resample cfg2: normwise error {err:.2e}")
    assert err < TOL_TC


# ------------------------------------- 160/147 default design over ragged lengths
# Lengths cover rows shorter than the filter, the 147-input period and its
# multiples around a work item, and a length that is not a multiple of 4; the
# default design and the same taps passed explicitly give the same result.
@pytest.mark.parametrize("n", [1, 2, 37, 1600, 4703, 4704, 4705, 9409, 150001])
@pytest.mark.parametrize("batch", [1, 3])
def test_resample_160_147_lengths(cuda, n, batch):
    rng = np.random.default_rng(n + batch)
    x = rng.standard_normal((batch, n)).astype(np.float32)
    h = S.resample_poly_default_taps(160, 147).astype(np.float32)
    ref = O.resample_poly_fast_f64(x.astype(np.float64), 160, 147, h.astype(np.float64))
    y = S.resample_poly_f32(_dev(x, cuda), 160, 147).cpu().numpy()
    assert y.shape == ref.shape
    assert normwise_err(y, ref) < TOL_FP32
    y2 = S.resample_poly_f32(_dev(x, cuda), 160, 147, h=_dev(h, cuda)).cpu().numpy()
    assert normwise_err(y, y2) < 1e-6
