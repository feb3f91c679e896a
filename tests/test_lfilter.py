"""General IIR lfilter(b, a) and lfilter_zi vs SciPy (the reference has no
general IIR filter; SciPy's lfilter is the oracle for these semantics)."""
import numpy as np
import pytest
import scipy.signal as ss

import scir_gb300 as S
from conftest import normwise_err

FILTERS = {
    "butter4_lp": ss.butter(4, 0.2),
    "cheby1_bp": ss.cheby1(5, 1, [0.2, 0.4], btype="bandpass"),
    "ellip_hp": ss.ellip(6, 0.5, 40, 0.3, btype="highpass"),
    "fir_as_iir": (ss.firwin(31, 0.25), [1.0]),
    "a0_not_one": ([2.0, 1.0, 0.5], [4.0, -1.0, 0.5]),
    "gain": ([3.0], [2.0]),
    "long_b": (np.r_[1.0, np.zeros(20), 0.5], [1.0, -0.9]),
}


@pytest.mark.parametrize("name", sorted(FILTERS))
def test_lfilter_zi_matches_scipy(name):
    b, a = FILTERS[name]
    np.testing.assert_allclose(S.lfilter_zi(b, a), ss.lfilter_zi(b, a), rtol=1e-12, atol=1e-14)


def test_lfilter_rejects_bad_coefficients():
    with pytest.raises(S.GpuError) as ei:
        S.lfilter_zi([1.0, 2.0], [0.0, 1.0])
    assert ei.value.status == S.ERR_INVALID_ARG
    with pytest.raises(S.GpuError) as ei:
        S.lfilter_zi(np.ones(40), [1.0])
    assert ei.value.status == S.ERR_UNSUPPORTED


def _dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


# FP64 with FMA on the GPU vs SciPy's separate multiply and add: the order-10
# Chebyshev band-pass in direct form amplifies the rounding difference to
# ~1.5e-12 normwise (state ~2.4e-10 relative); the bounds leave 100x room.
TOL64 = 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(FILTERS))
@pytest.mark.parametrize("n", [1, 31, 33, 5000])
def test_lfilter_vs_scipy(cuda, name, n):
    b, a = FILTERS[name]
    rng = np.random.default_rng(n)
    x = rng.standard_normal((37, n))
    ref = ss.lfilter(b, a, x, axis=1)
    y = S.lfilter(b, a, _dev(x, cuda)).cpu().numpy()
    assert normwise_err(y, ref) < TOL64
    y32 = S.lfilter(b, a, _dev(x.astype(np.float32), cuda)).cpu().numpy()
    ref32 = ss.lfilter(b, a, x.astype(np.float32).astype(np.float64), axis=1)
    assert normwise_err(y32, ref32) < 1e-6  # FP64 state; only the output is rounded to f32
    ns = max(len(np.atleast_1d(a)), len(np.atleast_1d(b))) - 1
    if ns:
        zi = rng.standard_normal((37, ns))
        refz, zfr = ss.lfilter(b, a, x, axis=1, zi=zi)
        yz, zf = S.lfilter(b, a, _dev(x, cuda), zi=_dev(zi, cuda), return_zf=True)
        assert normwise_err(yz.cpu().numpy(), refz) < TOL64
        np.testing.assert_allclose(zf.cpu().numpy(), zfr, rtol=1e-8, atol=1e-12)


@pytest.mark.gpu
def test_lfilter_state_chaining_and_in_place(cuda):
    b, a = FILTERS["cheby1_bp"]
    rng = np.random.default_rng(7)
    x = rng.standard_normal((64, 10000))
    xd = _dev(x, cuda)
    zi = np.outer(x[:, 0], ss.lfilter_zi(b, a))
    y1, zf = S.lfilter(b, a, xd[:, :4000].contiguous(), zi=_dev(zi, cuda), return_zf=True)
    y2 = S.lfilter(b, a, xd[:, 4000:].contiguous(), zi=zf)
    import torch
    full = torch.cat([y1, y2], 1).cpu().numpy()
    ref = ss.lfilter(b, a, x, axis=1, zi=zi)[0]
    assert normwise_err(full, ref) < TOL64
    S.lfilter(b, a, xd, out=xd)
    assert normwise_err(xd.cpu().numpy(), ss.lfilter(b, a, x, axis=1)) < TOL64
