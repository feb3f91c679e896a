"""Autotuner table persistence (CPU) and the tuned dispatch (GPU).

The table maps a problem shape on a device model to a kernel variant; the
tuned variant must give the same results as the default dispatch (bit for bit
in REF_EXACT mode)."""
import os

import numpy as np
import pytest
import scipy.signal as ss

import oracle as O
import scir_gb300 as S
from conftest import normwise_err

TABLE = """scir-autotune 1
fir NVIDIA_GB300_sm152 8 20000 300 20000 1 -299 1 2
fir NVIDIA_GB300_sm152 64 65536 63 65536 1 -62 -1 1
poly NVIDIA_GB300_sm152 4 20000 3201 160 147 1600 52
"""


def test_table_load_save_roundtrip(tmp_path):
    src = tmp_path / "in.txt"
    src.write_text(TABLE)
    S.autotune_clear()
    S.autotune_load(str(src))
    out = tmp_path / "out.txt"
    S.autotune_save(str(out))
    assert sorted(out.read_text().splitlines()) == sorted(TABLE.splitlines())
    S.autotune_clear()
    S.autotune_save(str(out))
    assert out.read_text() == "scir-autotune 1\n"


@pytest.mark.parametrize("text", ["not a table\n", "scir-autotune 2\n",
                                  "scir-autotune 1\nfir x 1 2 3\n",
                                  "scir-autotune 1\npoly m 1 2 3 4 5 6 99\n"])
def test_table_rejects_malformed(tmp_path, text):
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(S.GpuError):
        S.autotune_load(str(p))
    with pytest.raises(S.GpuError):
        S.autotune_load(str(tmp_path / "missing.txt"))


def _dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


@pytest.mark.gpu
def test_autotuned_fir_exact_and_auto(cuda, tmp_path):
    S.autotune_clear()
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, (8, 20000)).astype(np.float32)
    t = rng.standard_normal(300).astype(np.float32)
    choice, ms = S.autotune_fir(8, 20000, 300, S.FirMode.REF_CORR, S.Precision.REF_EXACT)
    assert choice in ("cuda-cores-v8", "cuda-cores-v16") and ms > 0
    y = S.fir_batched(_dev(x, cuda), _dev(t, cuda), S.FirMode.REF_CORR, S.Precision.REF_EXACT)
    assert np.array_equal(y.cpu().numpy(), O.fir1d_batched_f32(x, t))
    # AUTO may pick the tensor cores for a long filter; either way <= 1e-5
    xb = rng.uniform(-1, 1, (128, 16384)).astype(np.float32)
    tb = (ss.firwin(1025, 0.2) * 1.0).astype(np.float32)
    choice, ms = S.autotune_fir(128, 16384, 1025, S.FirMode.LFILTER, S.Precision.AUTO)
    assert choice in ("cuda-cores-v8", "cuda-cores-v16", "tensor-cores-fp16x3")
    y = S.fir_batched(_dev(xb, cuda), _dev(tb, cuda), S.FirMode.LFILTER, S.Precision.AUTO)
    ref = O.fir_mode_f64(xb[::31].astype(np.float64), tb.astype(np.float64), int(S.FirMode.LFILTER))
    assert normwise_err(y.cpu().numpy()[::31], ref) < 1e-5
    path = str(tmp_path / "t.txt")
    S.autotune_save(path)
    lines = open(path).read().splitlines()
    assert lines[0] == "scir-autotune 1" and len(lines) == 3
    S.autotune_clear()


@pytest.mark.gpu
def test_autotuned_resample(cuda):
    S.autotune_clear()
    choice, ms = S.autotune_resample_poly(4, 20000, 160, 147)
    assert choice.startswith("P=5 ") and ms > 0
    rng = np.random.default_rng(12)
    x = rng.standard_normal((4, 20000)).astype(np.float32)
    y = S.resample_poly_f32(_dev(x, cuda), 160, 147).cpu().numpy()
    h = S.resample_poly_default_taps(160, 147).astype(np.float32).astype(np.float64)
    assert normwise_err(y, O.resample_poly_fast_f64(x.astype(np.float64), 160, 147, h)) < 1e-5
    # a rate with several schedules (P from 1 to 5, one or two channels per item)
    choice, ms = S.autotune_resample_poly(4, 20000, 3, 2)
    assert choice.startswith("P=")
    y = S.resample_poly_f32(_dev(x, cuda), 3, 2).cpu().numpy()
    h = S.resample_poly_default_taps(3, 2).astype(np.float32).astype(np.float64)
    assert normwise_err(y, O.resample_poly_fast_f64(x.astype(np.float64), 3, 2, h)) < 1e-5
    S.autotune_clear()


@pytest.mark.gpu
def test_autotuned_ragged_plan(cuda):
    import torch
    rng = np.random.default_rng(13)
    n = np.exp(rng.uniform(np.log(100), np.log(40000), 30)).round().astype(np.int64)
    k = np.exp(rng.uniform(np.log(4), np.log(2000), 30)).round().astype(np.int64)
    x = rng.uniform(-1, 1, int(n.sum())).astype(np.float32)
    taps = rng.standard_normal(int(k.sum())).astype(np.float32)
    plan = S.RaggedPlan(n, k, S.FirMode.REF_CORR, S.Precision.REF_EXACT)
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(taps).to(cuda)
    y = torch.zeros(plan.y_len, device=cuda)
    thr, ms = plan.autotune(xd, td, y)
    assert thr in (32, 64, 128, 256, 512, 1 << 30) and ms > 0
    y.zero_()
    plan.run(xd, td, y)
    ref = np.concatenate([O.fir1d_batched_f32(x[plan.x_off[i]:plan.x_off[i] + n[i]],
                                              taps[plan.taps_off[i]:plan.taps_off[i] + k[i]])[0]
                          for i in range(len(n))])
    assert np.array_equal(y.cpu().numpy(), ref)
    plan.close()


@pytest.mark.gpu
@pytest.mark.parametrize("ct", [1, 2, 4])
def test_polyphase_schedules_via_table(cuda, tmp_path, ct):
    """Every channels-per-item schedule, forced through a loaded table, gives
    the oracle's result (6 channels: the last item of 4 holds 2 rows)."""
    S.autotune_clear()
    S.autotune_resample_poly(2, 1000, 160, 147)  # any tuned entry reveals the model tag
    path = tmp_path / "t.txt"
    S.autotune_save(str(path))
    model = path.read_text().splitlines()[1].split()[1]
    n = 20000
    path.write_text(f"scir-autotune 1\npoly {model} 6 {n} 3201 160 147 1600 {50 + ct}\n")
    S.autotune_clear()
    S.autotune_load(str(path))
    rng = np.random.default_rng(ct)
    x = rng.standard_normal((6, n)).astype(np.float32)
    y = S.resample_poly_f32(_dev(x, cuda), 160, 147).cpu().numpy()
    h = S.resample_poly_default_taps(160, 147).astype(np.float32).astype(np.float64)
    assert normwise_err(y, O.resample_poly_fast_f64(x.astype(np.float64), 160, 147, h)) < 1e-5
    S.autotune_clear()
