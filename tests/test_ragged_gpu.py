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
