"""DeviceArray elementwise ops and resize2d vs the reference's CPU semantics
(crates/scir-gpu/src/lib.rs:394-441, 629-725): bit-identical results."""
import ctypes

import numpy as np
import pytest

import oracle as O
import scir_gb300 as S
from scir_gb300._native import load


def test_oracle_resize_known_answers():
    data = np.arange(16, dtype=np.float32).reshape(4, 4)
    # lib.rs:1326-1335: same-size nearest resize is the identity
    assert np.array_equal(O.resize2d_f32(data, 4, 4, 0), data)
    # lib.rs:384-389 (doc example): 4x4 -> 2x2 nearest
    assert O.resize2d_f32(data, 2, 2, 0).shape == (2, 2)
    # lib.rs:1338-1356: a column ramp shrunk bilinearly stays in the source range
    ramp = np.tile(np.arange(4, dtype=np.float32), (4, 1))
    out = O.resize2d_f32(ramp, 2, 2, 1)
    assert out.shape == (2, 2) and np.all((out >= 0) & (out <= 3))


def test_resize_and_elementwise_validate_before_device():
    lib = load()
    buf = (ctypes.c_float * 4)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    assert lib.scir_resize2d_f32(p, 2, 2, p, 2, 2, 7, None) == S.ERR_INVALID_ARG
    assert lib.scir_resize2d_f32(p, 0, 2, p, 2, 2, 0, None) == S.ERR_SHAPE
    assert lib.scir_add_vec_f32(p, None, p, 4, None) == S.ERR_INVALID_ARG
    assert lib.scir_mul_scalar_f32(p, ctypes.c_float(2.0), p, -1, None) == S.ERR_INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 3, 4, 5, 1000, 1 << 20, (1 << 20) + 7])
def test_elementwise_bit_exact(cuda, n):
    import torch
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n + 1).astype(np.float32)
    b = rng.standard_normal(n + 1).astype(np.float32)
    ad, bd = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    for off in (0, 1):  # offset 1: not 16-byte aligned, the scalar path
        x, y = ad[off:off + n], bd[off:off + n]
        xa, ya = a[off:off + n], b[off:off + n]
        assert np.array_equal(S.add_vec(x, y).cpu().numpy(), xa + ya)
        assert np.array_equal(S.add_scalar(x, 0.3).cpu().numpy(), xa + np.float32(0.3))
        assert np.array_equal(S.mul_scalar(x, -1.7).cpu().numpy(), xa * np.float32(-1.7))
    with pytest.raises(S.GpuError) as ei:
        S.add_vec(ad[:n], bd[:max(n - 1, 1)] if n > 1 else bd[:2])
    assert ei.value.kind == "ShapeMismatch"


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(4, 4, 4, 4), (4, 4, 2, 2), (37, 53, 100, 71), (480, 640, 224, 224),
                                   (7, 5, 31, 2), (1, 9, 3, 27), (300, 200, 301, 199)])
@pytest.mark.parametrize("mode", [S.ResizeMode.NEAREST, S.ResizeMode.BILINEAR])
def test_resize2d_bit_exact(cuda, shape, mode):
    import torch
    sh, sw, oh, ow = shape
    rng = np.random.default_rng(sh * 1000 + sw)
    img = rng.standard_normal((sh, sw)).astype(np.float32)
    out = S.resize2d(torch.from_numpy(img).to(cuda), oh, ow, mode).cpu().numpy()
    assert np.array_equal(out, O.resize2d_f32(img, oh, ow, int(mode)))
