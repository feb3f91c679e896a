"""The tensor-core polyphase decomposition, checked on the CPU.

scir_gb300/csrc/poly_tc.cu computes upfirdn / resample_poly as one dense
product per 32-output segment: the window x[lo, lo + 64) with
lo = base(m0) - (Q - 1) rounded down to a multiple of 8, times a tap operand
B[n][k] = h[ph(m0 + n) + (base(m0 + n) - lo - k) * up] that depends only on the
segment's place in the tap pattern (s mod S, S = up / gcd(32 down, up)) and on
the window's misalignment mod 8.  This test restates that decomposition in
FP64 (no bf16 rounding) and compares it with the oracle, so an index error in
the scheme shows here independently of the GPU parity tests.  No GPU.
"""
import math

import numpy as np
import pytest

import oracle as O
import scir_gb300 as S

N_SEG, K_WIN = 32, 64


def _plan(kh, up, down, off):
    """The kernel's geometry, or None where it reports UNSUPPORTED."""
    Q = -(-kh // up)
    Sp = up // math.gcd(N_SEG * down, up)
    if Sp * 8 > 512:
        return None
    for sp in range(Sp):
        t0 = N_SEG * sp * down + off
        span = (t0 + (N_SEG - 1) * down) // up - t0 // up
        if span + Q + 7 > K_WIN:
            return None
    return Q, Sp


def _variants(h, up, down, off, Q, Sp):
    kh = h.size
    B = np.zeros((Sp * 8, N_SEG, K_WIN))
    for sp in range(Sp):
        t0 = N_SEG * sp * down + off
        base0 = t0 // up
        for r8 in range(8):
            for n in range(N_SEG):
                t = t0 + n * down
                base, ph = t // up, t % up
                for k in range(K_WIN):
                    q = (base - base0) + (Q - 1 + r8) - k
                    if 0 <= q < Q and ph + q * up < kh:
                        B[sp * 8 + r8, n, k] = h[ph + q * up]
    return B


def _segments(x, h, up, down, off, n_out):
    plan = _plan(h.size, up, down, off)
    assert plan is not None
    Q, Sp = plan
    B = _variants(h, up, down, off, Q, Sp)
    rows, n = x.shape
    y = np.zeros((rows, n_out))
    for s in range(-(-n_out // N_SEG)):
        m0 = N_SEG * s
        a0 = (m0 * down + off) // up - (Q - 1)
        r8 = a0 % 8
        lo = a0 - r8
        assert lo % 8 == 0
        win = np.zeros((rows, K_WIN))
        a, b = max(lo, 0), min(lo + K_WIN, n)
        if b > a:
            win[:, a - lo:b - lo] = x[:, a:b]
        seg = win @ B[(s % Sp) * 8 + r8].T
        m1 = min(m0 + N_SEG, n_out)
        y[:, m0:m1] = seg[:, :m1 - m0]
    return y


@pytest.mark.parametrize("up,down,kh,n", [(4, 1, 64, 3000), (3, 2, 11, 777), (5, 4, 41, 500),
                                          (160, 147, 3201, 2000), (7, 3, 30, 400)])
def test_upfirdn_segments_equal_oracle(up, down, kh, n):
    rng = np.random.default_rng(up * 97 + kh)
    h = rng.standard_normal(kh)
    x = rng.standard_normal((3, n))
    ref = O.upfirdn_f64(h, x, up, down)
    y = _segments(x, h, up, down, 0, ref.shape[1])
    np.testing.assert_allclose(y, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("up,down", [(160, 147), (3, 2), (5, 4)])
def test_resample_segments_equal_oracle(up, down):
    rng = np.random.default_rng(up + down)
    x = rng.standard_normal((2, 3000))
    h = S.resample_poly_default_taps(up, down)
    ref = O.resample_poly_fast_f64(x, up, down, h)
    y = _segments(x, h, up, down, (h.size - 1) // 2, ref.shape[1])
    np.testing.assert_allclose(y, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_unserved_shapes_match_the_kernel_plan():
    # 2/3 with the default 61-tap design spans more than the 64-sample window
    h = S.resample_poly_default_taps(2, 3)
    assert _plan(h.size, 2, 3, (h.size - 1) // 2) is None
    # 160/147 with its 3,201-tap design: 5 pattern positions x 8 misalignments
    assert _plan(3201, 160, 147, 1600) == (21, 5)
