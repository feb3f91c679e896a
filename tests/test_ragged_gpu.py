"""Ragged persistent FIR vs the oracle, and its CUDA-graph replay."""
import numpy as np
import pytest

import oracle as O
import scir_gb300 as S
from conftest import normwise_err

pytestmark = pytest.mark.gpu


def _ragged_set(seed, count, nmax, kmax):
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(1), np.log(nmax), count)).round().astype(np.int64)
    k = np.exp(rng.uniform(np.log(1), np.log(kmax), count)).round().astype(np.int64)
    x = rng.uniform(-1, 1, int(n.sum())).astype(np.float32)
    taps = rng.standard_normal(int(k.sum())).astype(np.float32)
    return n, k, x, taps


@pytest.mark.parametrize("mode", [S.FirMode.REF_CORR, S.FirMode.LFILTER, S.FirMode.FULL])
def test_ragged_fp32_vs_oracle(cuda, mode):
    import torch
    n, k, x, taps = _ragged_set(int(mode), 40, 30000, 3000)
    plan = S.RaggedPlan(n, k, mode, S.Precision.FP32)
    y = torch.full((plan.y_len,), float("nan"), device=cuda)
    plan.run(torch.from_numpy(x).to(cuda), torch.from_numpy(taps).to(cuda), y)
    y = y.cpu().numpy()
    for i in range(len(n)):
        xi = x[plan.x_off[i]:plan.x_off[i] + n[i]].astype(np.float64)
        ti = taps[plan.taps_off[i]:plan.taps_off[i] + k[i]].astype(np.float64)
        ref = O.fir_mode_f64(xi, ti, int(mode))[0]
        yi = y[plan.y_off[i]:plan.y_off[i] + plan.n_out[i]]
        assert normwise_err(yi, ref) < 1e-5, i


def test_ragged_exact_and_graph_replay(cuda):
    import torch
    n, k, x, taps = _ragged_set(7, 25, 20000, 700)
    plan = S.RaggedPlan(n, k, S.FirMode.REF_CORR, S.Precision.REF_EXACT)
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(taps).to(cuda)
    y = torch.zeros(plan.y_len, device=cuda)
    plan.run(xd, td, y)
    ref = np.concatenate([O.fir1d_batched_f32(x[plan.x_off[i]:plan.x_off[i] + n[i]],
                                              taps[plan.taps_off[i]:plan.taps_off[i] + k[i]])[0]
                          for i in range(len(n))])
    assert np.array_equal(y.cpu().numpy(), ref)
    # capture the launch (memset of the work counter + persistent kernel) and replay it
    y2 = torch.zeros_like(y)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            plan.run(xd, td, y2, stream=s)
    for _ in range(3):
        y2.zero_()
        g.replay()
    torch.cuda.synchronize()
    assert np.array_equal(y2.cpu().numpy(), ref)


def test_library_graph_capture_mixed_calls(cuda):
    """One graph recorded through the C ABI (scir_graph_capture_*) replays a
    batched FIR, a resample, an SOS cascade and a ragged launch."""
    import scipy.signal as ss
    import torch
    S.init(0)
    rng = np.random.default_rng(21)
    x = torch.from_numpy(rng.uniform(-1, 1, (16, 30000)).astype(np.float32)).to(cuda)
    t = torch.from_numpy(ss.firwin(127, 0.2).astype(np.float32)).to(cuda)
    sos = ss.butter(8, [0.01, 0.02], btype="bandpass", output="sos")
    n, k, xr, tr = _ragged_set(22, 12, 20000, 500)
    plan = S.RaggedPlan(n, k, S.FirMode.LFILTER, S.Precision.FP32)
    xrd, trd = torch.from_numpy(xr).to(cuda), torch.from_numpy(tr).to(cuda)
    s = torch.cuda.Stream()
    outs = {}

    def calls(tag):
        outs[tag] = [S.fir_batched(x, t, S.FirMode.LFILTER, S.Precision.FP32, out=outs[tag][0], stream=s),
                     S.resample_poly_f32(x, 160, 147, out=outs[tag][1], stream=s),
                     S.sosfilt_f32(sos, x, precision=S.SosPrecision.FP32_COUPLED, out=outs[tag][2],
                                   stream=s),
                     plan.run(xrd, trd, outs[tag][3], stream=s)]

    n_rs = S.resample_poly_out_len(30000, 160, 147)
    for tag in ("eager", "graph"):
        outs[tag] = [torch.zeros_like(x), torch.zeros((16, n_rs), device=cuda), torch.zeros_like(x),
                     torch.zeros(plan.y_len, device=cuda)]
    with torch.cuda.stream(s):
        calls("eager")  # first use creates taps, tensor maps and state outside the capture
        s.synchronize()
        with S.GraphCapture(s) as g:
            calls("graph")
        for a in outs["graph"]:
            a.fill_(float("nan"))
        for _ in range(2):
            g.launch()
        s.synchronize()
    for a, b in zip(outs["eager"], outs["graph"]):
        assert torch.equal(a, b)
    g.close()
    plan.close()


# ------------------------------- tensor-core bucket (AUTO = FP16X3, BF16X6, BF16X3)
# Signals with >= 512 taps and >= 16,384 outputs run the split-operand
# contraction as segment rows (up to 128 per signal) in their own persistent
# launch; the rest stay on the CUDA cores.  Both buckets are checked against
# the FP64 oracle, with odd output offsets (scalar stores) among them.
def _mixed_set(seed, count):
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(1000), np.log(400000), count)).round().astype(np.int64)
    k = np.exp(rng.uniform(np.log(16), np.log(2048), count)).round().astype(np.int64)
    n[:3] = [300000, 20000, 150001]
    k[:3] = [2048, 600, 4095]
    x = rng.uniform(-1, 1, int(n.sum())).astype(np.float32)
    taps = (rng.standard_normal(int(k.sum())) / np.sqrt(np.repeat(k, k))).astype(np.float32)
    return n, k, x, taps


@pytest.mark.parametrize("prec,tol", [(S.Precision.AUTO, 1e-5), (S.Precision.BF16X6, 1e-5),
                                      (S.Precision.BF16X3, 3e-5)])
@pytest.mark.parametrize("mode", [S.FirMode.LFILTER, S.FirMode.REF_CORR, S.FirMode.FULL,
                                  S.FirMode.VALID])
def test_ragged_tensor_core_bucket(cuda, prec, tol, mode):
    import torch
    n, k, x, taps = _mixed_set(int(mode) + 10, 24)
    n = np.maximum(n, k)  # VALID needs n >= k
    x = np.random.default_rng(3).uniform(-1, 1, int(n.sum())).astype(np.float32)
    # odd gaps between the outputs of consecutive signals
    n_out = np.array([S.fir_out_len(int(a), int(b), mode) for a, b in zip(n, k)])
    y_off = np.concatenate([[1], np.cumsum(n_out + 3)[:-1] + 1]).astype(np.int64)
    plan = S.RaggedPlan(n, k, mode, prec, y_off=y_off)
    tc_taps, tc_count = plan.tensor_cores()
    assert tc_taps == 512 and 3 <= tc_count < len(n)
    y = torch.full((int(y_off[-1] + n_out[-1] + 2),), float("nan"), device=cuda)
    plan.run(torch.from_numpy(x).to(cuda), torch.from_numpy(taps).to(cuda), y)
    y = y.cpu().numpy()
    for i in range(len(n)):
        xi = x[plan.x_off[i]:plan.x_off[i] + n[i]].astype(np.float64)
        ti = taps[plan.taps_off[i]:plan.taps_off[i] + k[i]].astype(np.float64)
        ref = O.fir_mode_f64(xi, ti, int(mode))[0]
        yi = y[y_off[i]:y_off[i] + n_out[i]]
        assert normwise_err(yi, ref) < tol, (i, int(n[i]), int(k[i]))
    plan.close()


def test_ragged_fp16x3_per_signal_scale(cuda):
    # every tensor-core signal has its own power-of-two scales (signal and
    # taps): magnitudes from 1e-15 to 1e6 side by side, one signal all zero
    import torch
    n, k, x, taps = _mixed_set(77, 12)
    scale = np.array([1e6, 1e-15, 0.0, 3e-3, 1.0, 1e4, 1.0, 2e-8, 1.0, 1.0, 5.0, 1.0])
    tscale = np.array([1.0, 1e3, 1.0, 1e-6, 1.0, 1.0, 1e-9, 1.0, 1.0, 7.0, 1.0, 1.0])
    plan = S.RaggedPlan(n, k, S.FirMode.LFILTER, S.Precision.FP16X3)
    for i in range(len(n)):
        x[plan.x_off[i]:plan.x_off[i] + n[i]] *= np.float32(scale[i])
        taps[plan.taps_off[i]:plan.taps_off[i] + k[i]] *= np.float32(tscale[i])
    assert plan.tensor_cores()[1] >= 3
    y = torch.full((plan.y_len,), float("nan"), device=cuda)
    plan.run(torch.from_numpy(x).to(cuda), torch.from_numpy(taps).to(cuda), y)
    y = y.cpu().numpy()
    for i in range(len(n)):
        xi = x[plan.x_off[i]:plan.x_off[i] + n[i]].astype(np.float64)
        ti = taps[plan.taps_off[i]:plan.taps_off[i] + k[i]].astype(np.float64)
        ref = O.fir_mode_f64(xi, ti, int(S.FirMode.LFILTER))[0]
        yi = y[plan.y_off[i]:plan.y_off[i] + n[i]]
        if scale[i] == 0.0:
            assert np.all(yi == 0.0)
        else:
            assert normwise_err(yi, ref) < 1e-5, (i, int(n[i]), int(k[i]))
    plan.close()


def test_ragged_tensor_core_graph_and_autotune(cuda):
    import torch
    n, k, x, taps = _mixed_set(31, 16)
    plan = S.RaggedPlan(n, k, S.FirMode.LFILTER, S.Precision.AUTO)
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(taps).to(cuda)
    y = torch.zeros(plan.y_len, device=cuda)
    plan.autotune(xd, td, y)
    plan.run(xd, td, y)
    ref = y.clone()
    y2 = torch.zeros_like(y)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            plan.run(xd, td, y2, stream=s)
    for _ in range(2):
        y2.fill_(float("nan"))
        g.replay()
    torch.cuda.synchronize()
    assert torch.equal(ref, y2)
    for i in range(len(n)):
        xi = x[plan.x_off[i]:plan.x_off[i] + n[i]].astype(np.float64)
        ti = taps[plan.taps_off[i]:plan.taps_off[i] + k[i]].astype(np.float64)
        ref_i = O.fir_mode_f64(xi, ti, int(S.FirMode.LFILTER))[0]
        assert normwise_err(y2[plan.y_off[i]:plan.y_off[i] + n[i]].cpu().numpy(), ref_i) < 1e-5
    plan.close()
