"""The benchmark's roofline arithmetic, on the CPU.

The roofline of the long-tap FIR counts the algorithmic work (one multiply-
add per tap and output, 2*B*n*k flops) against the bf16 peak, with the
tensor products the split form issues reported beside it; the ragged set's
floor is per signal the larger of its bytes at the HBM peak and its flops at
the peak of the unit that runs it, summed; the DRAM traffic comes from the
committed ncu summary.  No GPU and no library call is involved."""
import types

import numpy as np
import pytest

import bench


class _FakeTensorWorkload:
    name = "fir_long_4095"
    bound = "tensor"
    kernel = "fake"
    launches_per_step = 4
    roofline_launches = 1
    B, N, K = 1024, 262144, 4095

    def products(self, precision=None):
        return 3

    def alg_flops(self):
        return 2.0 * self.B * self.N * self.K

    def alg_bytes(self):
        return 8 * self.B * self.N


PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def test_tensor_roofline_counts_one_product():
    W = _FakeTensorWorkload()
    ms = 4.4
    r = bench.roofline(W, ms, PEAKS, lambda fp64: 76.4)
    alg = 2.0 * 1024 * 262144 * 4095 / (ms / 1e3) / 1e12
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert r["achieved"] == pytest.approx(alg)
    assert r["frac"] == pytest.approx(alg / 1900.0)
    assert r["products_issued"] == 3
    assert r["issued_frac"] == pytest.approx(3 * alg / 1900.0)
    # the committed step traffic of this workload
    assert r["traffic"] == pytest.approx(5675235328.0)


def test_hbm_roofline():
    W = _FakeTensorWorkload()
    W.bound = "hbm"
    r = bench.roofline(W, 1.0, PEAKS, lambda fp64: 76.4)
    assert r["achieved"] == pytest.approx(8 * 1024 * 262144 / 1e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6800.0)
    assert "products_issued" not in r


def test_ragged_floor_per_signal():
    # three signals: a short FIR on the CUDA cores (HBM-bound), a long one on
    # the CUDA cores (FMA-bound) and one in the tensor-core bucket
    n = np.array([100000, 100000, 100000])
    k = np.array([8, 150, 300])
    R = object.__new__(bench.Ragged)
    R.n, R.k = n, k
    R.precision = "AUTO"
    R.S = types.SimpleNamespace(Precision=types.SimpleNamespace(BF16X6="BF16X6"))
    R.plan = types.SimpleNamespace(tensor_cores=lambda: (192, 1), n_out=n.copy())
    fp32, bf16, hbm = 76.4, 1900.0, 6800.0
    got = R.floor_ms(fp32, bf16, hbm)
    by = 8.0 * n
    fl = 2.0 * n * k
    want = (max(by[0] / (hbm * 1e9), fl[0] / (fp32 * 1e12)) +
            max(by[1] / (hbm * 1e9), fl[1] / (fp32 * 1e12)) +
            max(by[2] / (hbm * 1e9), fl[2] / (bf16 * 1e12))) * 1e3
    assert got == pytest.approx(want)


def test_profile_traffic_lines_parse():
    assert bench.profile_traffic("fir_long_4095") == pytest.approx(5675235328.0)
    assert bench.profile_traffic("resample_poly_160_147") == pytest.approx(2046622720.0)
    assert bench.profile_traffic("no_such_workload") is None


class _FakeCpuWorkload:
    B = 64

    def __init__(self, full):
        self.full = full

    def cpu_row_len(self):
        return self.full

    def cpu_sample(self, O, rows, per):
        return rows * per, rows * per * 1e-9  # 1 ns per sample


def test_cpu_sample_never_exceeds_the_workload():
    # a workload whose full size takes far less than the target: one step is
    # the whole workload (64 full-length rows), not more rows of it
    rows, per = bench.calibrate_cpu(_FakeCpuWorkload(65536), None, 8, 10.0)
    assert (rows, per) == (64, 65536)
    # a long one: full-length rows, fewer than the workload holds
    rows, per = bench.calibrate_cpu(_FakeCpuWorkload(1 << 30), None, 8, 1.0)
    assert rows == 8 and per < (1 << 30)


def test_reference_arm_line():
    # the reference arm runs the restated reference loop on the host cores
    # and prints the benchmark's JSON line with impl = reference
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                          "--workload", "fir_short", "--steps", "2", "--warmup", "3"],
                         capture_output=True, text=True, timeout=300, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 3
    assert d["metric"] == "batched FIR Gsamples/s" and d["unit"] == "Gsamples/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"].startswith("64 channels x 65536 samples")
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["channels"] == 64
