#!/usr/bin/env python3
"""Throughput of the batched-filtering hot path on GB300.

Default workload (N=1): the long-tap batched FIR of 1,024 channels x 262,144
f32 samples with a 4,095-tap Kaiser(8.6) band-pass -- the configuration the
headline metric (batched FIR Gsamples/s, chosen split-operand tensor-core
form vs plain FP32 CUDA-core form at <= 1e-5 error) is quoted on; AUTO runs
the FP16X3 form there.  The same line carries the plain-FP32 timing and the
other tensor-core forms (BF16X6, BF16X3) of that workload and, under
"resample_poly_160_147", the polyphase resample of 256 x 1,048,576 samples
at 160/147 (HBM-bound).  Other configurations can be timed alone with
--workload (resample, fir_short, ragged, sosfilt, sosfiltfilt).

A step is one pass of the hot path over one batch of synthetic input,
resident in HBM.  W warm-up steps, then K timed steps between a barrier and
a device synchronize; the device time comes from CUDA events on the launch
stream, the max over ranks is reported by rank 0 as one JSON line.  Inputs
are larger than L2 (129 MB) for the default workload.  `e2e` re-times the
same work through the host-buffer C-ABI entry point (pinned host buffers,
host<->device copies inside the timed region).  `cpu_baseline` times the CPU
restatement of the reference's own algorithm on a bounded sample, on all
host cores and on one.

--impl reference times the reference's CPU implementation of the path (the
C restatement of its loops; no Rust toolchain is installed to build the Rust
reference) on the host cores, without loading this package.

--probe-peaks prints the measured FP32 and FP64 FMA throughput of the GPU
(the denominators of the CUDA-core-bound rooflines).

Multi-GPU: torchrun, one rank per GPU; every rank processes its own full batch
of channels (weak scaling, no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "bf16_tflops_sustained": float(d.get("bf16_tflops_sustained", d["bf16_tflops"])),
                "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "source": "fallback"}


def profile_traffic(workload: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (a line `traffic_bytes_per_launch: <n>` in profiles/<workload>*.md)."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for fn in sorted(os.listdir(pdir)):
        if fn.startswith(workload) and fn.endswith(".md"):
            with open(os.path.join(pdir, fn)) as f:
                for line in f:
                    if line.strip().startswith("traffic_bytes_per_launch:"):
                        try:
                            return float(line.split(":", 1)[1].split()[0])
                        except ValueError:
                            return None
    return None


# ----------------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.tmp = None

    def __enter__(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return self
        # nvidia-smi initialises slowly and can stall CUDA calls while it does;
        # start timing only once it is producing samples
        t0 = time.time()
        while time.time() - t0 < 15:
            try:
                if os.path.getsize(self.tmp.name) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.05)
        time.sleep(0.2)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.tmp is None:
            return None
        self.tmp.flush()
        self.tmp.seek(0)
        rows = [r.split(",") for r in self.tmp.read().strip().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [c.strip() for c in r]
            if len(r) < 7:
                continue
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except ValueError:
                continue
            for name, v in zip(names, r[3:7]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# ----------------------------------------------------------------------------- workloads

class Workload:
    name = ""
    metric = "batched FIR Gsamples/s"
    unit = "Gsamples/s"
    bound = "hbm"
    launches_per_step = 1
    flush_l2 = False      # working set below L2: flush before every timed step
    cpu_dtype = "f32"     # arithmetic of the restated reference loop

    def host_release(self):
        """Drops the pinned host buffers of the end-to-end leg."""
        for a in ("hx", "hy", "hyv", "hyf", "hx_np", "hy_np", "htaps"):
            if hasattr(self, a):
                delattr(self, a)

    def products(self, precision=None):
        return 1

    def samples_per_step(self) -> int:
        raise NotImplementedError

    def autotune(self):
        """Runs the library's autotuner for this workload's shape (outside the
        timed region); returns a short description of the choice or None."""
        return None


class Resample(Workload):
    name = "resample_poly_160_147"
    B, N, UP, DOWN = 256, 1048576, 160, 147
    cpu_dtype = "f64"

    def __init__(self, torch, dev, precision, channels=None):
        import scir_gb300 as S
        self.S, self.torch, self.dev = S, torch, dev
        self.precision = precision
        if channels:
            self.B = channels
        g = torch.Generator(device=dev).manual_seed(0)
        self.x = torch.randn((self.B, self.N), device=dev, generator=g)
        self.n_out = S.resample_poly_out_len(self.N, self.UP, self.DOWN)
        self.y = torch.empty((self.B, self.n_out), device=dev)
        self.kh = S.resample_poly_default_taps(self.UP, self.DOWN).size
        # BF16X3 runs the tensor-core polyphase (tap-operand build + the
        # contraction: two launches per step)
        tc = precision == S.Precision.BF16X3
        self.kernel = "poly_tc_kernel" if tc else "poly_stream_kernel"
        self.launches_per_step = 2 if tc else 1
        self.roofline_launches = 1

    @classmethod
    def config(cls):
        return {"workload": "resample_poly 160/147: 256 ch x 1,048,576 f32 N(0,1) samples, "
                            "SciPy default 3,201-tap Kaiser(5.0) design, zero-padded edges",
                "channels": cls.B, "samples_per_channel": cls.N, "up": cls.UP,
                "down": cls.DOWN, "taps": 3201, "outputs_per_channel": 1141308,
                "l2": "inputs larger than L2 (1.07 GB read, 1.17 GB written per step)"}

    def samples_per_step(self):
        return self.B * self.N

    def alg_bytes(self):
        return 4 * self.B * (self.N + self.n_out)

    def alg_flops(self):
        return 2.0 * self.B * self.n_out * (self.kh / self.UP)

    def step(self, stream, precision=None):
        self.S.resample_poly_f32(self.x, self.UP, self.DOWN, precision=self.precision if precision is None else precision,
                                 out=self.y, stream=stream)

    def autotune(self):
        choice, ms = self.S.autotune_resample_poly(self.B, self.N, self.UP, self.DOWN)
        return f"{choice} ({ms:.3f} ms)"

    def max_rel_err(self, precision=None):
        import scipy.signal as ss
        rows = [0, self.B - 1]
        self.step(None, precision)
        self.torch.cuda.synchronize()
        y = self.y[rows].cpu().numpy().astype(np.float64)
        ref = ss.resample_poly(self.x[rows].cpu().numpy().astype(np.float64), self.UP, self.DOWN,
                               axis=1)
        return float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))

    def host_setup(self):
        t = self.torch
        self.hx = t.empty((self.B, self.N), dtype=t.float32, pin_memory=True)
        self.hx.copy_(self.x)
        self.hy = t.empty((self.B, self.n_out), dtype=t.float32, pin_memory=True)
        self.hx_np, self.hy_np = self.hx.numpy(), self.hy.numpy()
        return 4 * self.B * self.N, 4 * self.B * self.n_out

    def host_step(self):
        self.S.resample_poly_host(self.hx_np, self.UP, self.DOWN, precision=self.precision,
                                  out=self.hy_np)

    # the reference's CPU algorithm (zero-stuff, full convolution, decimate,
    # crates/scir-signal/src/lib.rs:313-362) generalised to 160/147 with the
    # SciPy default design (the reference itself accepts only 2/3)
    @classmethod
    def cpu_taps(cls):
        import scipy.signal as ss
        mr = max(cls.UP, cls.DOWN)
        return ss.firwin(2 * 10 * mr + 1, 1.0 / mr, window=("kaiser", 5.0)) * cls.UP

    def cpu_sample(self, O, threads, per_channel):
        rng = np.random.default_rng(1)
        x = rng.standard_normal((threads, per_channel))
        h = self.cpu_taps()
        t0 = time.perf_counter()
        O.resample_poly_ref_f64(x, self.UP, self.DOWN, h)
        return threads * per_channel, time.perf_counter() - t0

    def cpu_row_len(self):
        return self.N

    def cpu_sample_desc(self, rows, per_channel):
        return (f"{rows} channels x {per_channel} samples per step through the restated "
                f"reference resample_poly (zero-stuff by 160, full 3,201-tap convolution, "
                f"decimate by 147), f64, channels spread over OpenMP threads")

    def scipy_sample(self, per_channel):
        import scipy.signal as ss
        x = np.random.default_rng(1).standard_normal((1, per_channel))
        t0 = time.perf_counter()
        ss.resample_poly(x, self.UP, self.DOWN, axis=1)
        return per_channel, time.perf_counter() - t0, "scipy.signal.resample_poly (polyphase, f64)"


class FirLong(Workload):
    """1,024 ch x 262,144 samples (sum of 32 random sinusoids + N(0, 0.1^2)),
    4,095-tap Kaiser(8.6) band-pass 0.1-0.3 x Nyquist, lfilter semantics."""
    name = "fir_long_4095"
    B, N, K = 1024, 262144, 4095
    bound = "tensor"

    def __init__(self, torch, dev, precision, channels=None):
        import scipy.signal as ss
        import scir_gb300 as S
        self.S, self.torch, self.dev = S, torch, dev
        self.precision = precision
        if channels:
            self.B = channels
        g = torch.Generator(device=dev).manual_seed(0)
        t = torch.arange(self.N, device=dev, dtype=torch.float32)
        self.x = torch.randn((self.B, self.N), device=dev, generator=g) * 0.1
        f = torch.rand((self.B, 32), device=dev, generator=g) * 0.5
        ph = torch.rand((self.B, 32), device=dev, generator=g) * (2 * np.pi)
        for i in range(32):
            # phase reduced in f64 so the f32 argument stays accurate
            arg = torch.remainder(f[:, i:i + 1].double() * t.double()[None, :], 1.0).float()
            self.x += torch.sin(2 * np.pi * arg + ph[:, i:i + 1]) / 32
        taps = ss.firwin(self.K, [0.1, 0.3], window=("kaiser", 8.6), pass_zero=False)
        self.taps = torch.from_numpy(taps.astype(np.float32)).to(dev)
        self.y = torch.empty((self.B, self.N), device=dev)
        if precision in (S.Precision.BF16X3, S.Precision.BF16X6, S.Precision.FP16X3,
                         S.Precision.AUTO):
            # (FP16X3: max pass +) operand split (signal, taps) + the
            # tensor-core launch; the roofline time is the whole step
            self.kernel = "fir_tc_kernel + max and split kernels (whole step)"
            self.launches_per_step = 3 if precision in (S.Precision.BF16X3,
                                                        S.Precision.BF16X6) else 4
            self.roofline_launches = 1
        else:
            self.kernel = "fir_simt_kernel"

    @classmethod
    def config(cls):
        return {"workload": "long-tap FIR: 1,024 ch x 262,144 f32 samples (32 random sinusoids + "
                            "N(0,0.1^2)), 4,095-tap Kaiser(8.6) band-pass 0.1-0.3 Nyquist, "
                            "lfilter semantics", "channels": cls.B,
                "samples_per_channel": cls.N, "taps": cls.K,
                "l2": "inputs larger than L2 (1.07 GB read, 1.07 GB written per step)"}

    def samples_per_step(self):
        return self.B * self.N

    def alg_bytes(self):
        return 8 * self.B * self.N

    def products(self, precision=None):
        p = self.precision if precision is None else precision
        # AUTO runs FP16X3 on this shape (the autotuner's record says so)
        return {self.S.Precision.BF16X3: 3, self.S.Precision.BF16X6: 6, self.S.Precision.FP16X3: 3,
                self.S.Precision.AUTO: 3}.get(p, 1)

    def alg_flops(self):
        # the algorithmic work: one multiply-add per tap and output (the split
        # forms issue products() times this on the tensor cores)
        return 2.0 * self.B * self.N * self.K

    def step(self, stream, precision=None):
        self.S.fir_batched(self.x, self.taps, self.S.FirMode.LFILTER,
                           self.precision if precision is None else precision, out=self.y,
                           stream=stream)

    def autotune(self):
        P = self.S.Precision
        if self.precision not in (P.FP32, P.REF_EXACT, P.AUTO):
            return None
        choice, ms = self.S.autotune_fir(self.B, self.N, self.K, self.S.FirMode.LFILTER,
                                         self.precision)
        return f"{choice} ({ms:.3f} ms)"

    def max_rel_err(self, precision=None):
        rows = [0, self.B - 1]
        self.step(None, precision)
        self.torch.cuda.synchronize()
        x = self.x[rows].cpu().numpy().astype(np.float64)
        h = self.taps.cpu().numpy().astype(np.float64)
        nf = 1 << int(np.ceil(np.log2(self.N + self.K)))
        ref = np.fft.irfft(np.fft.rfft(x, nf) * np.fft.rfft(h, nf), nf)[:, :self.N]
        y = self.y[rows].cpu().numpy().astype(np.float64)
        return float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))

    def host_setup(self):
        t = self.torch
        self.hx = t.empty((self.B, self.N), dtype=t.float32, pin_memory=True)
        self.hx.copy_(self.x)
        self.hy = t.empty((self.B, self.N), dtype=t.float32, pin_memory=True)
        self.htaps = self.taps.cpu().numpy()
        return 4 * self.B * self.N, 4 * self.B * self.N

    def host_step(self):
        self.S.fir_batched_host(self.hx.numpy(), self.htaps, self.S.FirMode.LFILTER,
                                self.precision, out=self.hy.numpy())

    # the reference's CPU loop (crates/scir-gpu/src/lib.rs:1134-1152), f32, on
    # rows of the configuration's signal with its band-pass taps
    @classmethod
    def cpu_inputs(cls, rows, per_channel):
        import scipy.signal as ss
        rng = np.random.default_rng(1)
        t = np.arange(per_channel)
        x = rng.standard_normal((rows, per_channel)) * 0.1
        for r in range(rows):
            f, ph = rng.uniform(0, 0.5, 32), rng.uniform(0, 2 * np.pi, 32)
            x[r] += np.sin(2 * np.pi * np.outer(f, t) + ph[:, None]).sum(0) / 32
        taps = ss.firwin(cls.K, [0.1, 0.3], window=("kaiser", 8.6), pass_zero=False)
        return x.astype(np.float32), taps.astype(np.float32)

    def cpu_sample(self, O, threads, per_channel):
        x, taps = self.cpu_inputs(threads, per_channel)
        t0 = time.perf_counter()
        O.fir1d_batched_f32(x, taps)
        return threads * per_channel, time.perf_counter() - t0

    def cpu_row_len(self):
        return self.N

    def cpu_sample_desc(self, rows, per_channel):
        return (f"{rows} channels x {per_channel} samples per step through the restated "
                f"reference fir1d_batched_f32 loop (4,095 taps, f32, sequential per channel), "
                f"channels spread over OpenMP threads")

    def scipy_sample(self, per_channel):
        import scipy.signal as ss
        x, taps = self.cpu_inputs(1, per_channel)
        t0 = time.perf_counter()
        ss.lfilter(taps.astype(np.float64), 1.0, x[0].astype(np.float64))
        return per_channel, time.perf_counter() - t0, "scipy.signal.lfilter (direct form, f64)"


class FirShort(Workload):
    """64 ch x 65,536 U[-1,1) samples, 63-tap Hamming low-pass (0.2 x Nyquist);
    one step = the 'valid' and the 'full' lfilter pass (2 launches)."""
    name = "fir_short_63"
    B, N, K = 64, 65536, 63
    launches_per_step = 2
    flush_l2 = True

    def __init__(self, torch, dev, precision, channels=None):
        import scipy.signal as ss
        import scir_gb300 as S
        self.S, self.torch, self.dev = S, torch, dev
        self.precision = precision
        if channels:
            self.B = channels
        g = torch.Generator(device=dev).manual_seed(0)
        self.x = torch.rand((self.B, self.N), device=dev, generator=g) * 2 - 1
        self.taps = torch.from_numpy(ss.firwin(self.K, 0.2, window="hamming").astype(np.float32)).to(dev)
        self.yv = torch.empty((self.B, self.N - self.K + 1), device=dev)
        self.yf = torch.empty((self.B, self.N + self.K - 1), device=dev)
        self.kernel = "fir_simt_kernel"

    @classmethod
    def config(cls):
        return {"workload": "short-tap FIR: 64 ch x 65,536 f32 U[-1,1) samples, 63-tap Hamming "
                            "low-pass 0.2 Nyquist, 'valid' + 'full' lfilter passes per step",
                "channels": cls.B, "samples_per_channel": cls.N, "taps": cls.K,
                "l2": "working set (33.5 MB) below L2: a 256 MB write flushes L2 before every "
                      "timed step"}

    def samples_per_step(self):
        return 2 * self.B * self.N

    def alg_bytes(self):
        return 4 * self.B * (2 * self.N + (self.N - self.K + 1) + (self.N + self.K - 1))

    def alg_flops(self):
        return 2.0 * self.K * self.B * (2 * self.N)

    def autotune(self):
        P, M = self.S.Precision, self.S.FirMode
        if self.precision not in (P.FP32, P.REF_EXACT, P.AUTO):
            return None
        out = []
        for mode in (M.VALID, M.FULL):
            choice, ms = self.S.autotune_fir(self.B, self.N, self.K, mode, self.precision)
            out.append(f"{mode.name.lower()}: {choice} ({ms:.3f} ms)")
        return "; ".join(out)

    def step(self, stream, precision=None):
        p = self.precision if precision is None else precision
        self.S.fir_batched(self.x, self.taps, self.S.FirMode.VALID, p, out=self.yv, stream=stream)
        self.S.fir_batched(self.x, self.taps, self.S.FirMode.FULL, p, out=self.yf, stream=stream)

    def max_rel_err(self, precision=None):
        rows = [0, self.B - 1]
        self.step(None, precision)
        self.torch.cuda.synchronize()
        x = self.x[rows].cpu().numpy().astype(np.float64)
        h = self.taps.cpu().numpy().astype(np.float64)
        ref = np.array([np.convolve(r, h, "full") for r in x])
        y = self.yf[rows].cpu().numpy()
        return float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))

    def host_setup(self):
        t = self.torch
        self.hx = t.empty((self.B, self.N), dtype=t.float32, pin_memory=True)
        self.hx.copy_(self.x)
        self.hyv = t.empty(tuple(self.yv.shape), dtype=t.float32, pin_memory=True)
        self.hyf = t.empty(tuple(self.yf.shape), dtype=t.float32, pin_memory=True)
        self.htaps = self.taps.cpu().numpy()
        return 2 * 4 * self.B * self.N, 4 * (self.yv.numel() + self.yf.numel())

    def host_step(self):
        self.S.fir_batched_host(self.hx.numpy(), self.htaps, self.S.FirMode.VALID, self.precision,
                                out=self.hyv.numpy())
        self.S.fir_batched_host(self.hx.numpy(), self.htaps, self.S.FirMode.FULL, self.precision,
                                out=self.hyf.numpy())

    def cpu_sample(self, O, threads, per_channel):
        rng = np.random.default_rng(1)
        x = rng.uniform(-1, 1, (threads, per_channel)).astype(np.float32)
        taps = np.ones(self.K, np.float32) / self.K
        t0 = time.perf_counter()
        O.fir1d_batched_f32(x, taps)
        return threads * per_channel, time.perf_counter() - t0

    def cpu_row_len(self):
        return self.N

    def cpu_sample_desc(self, rows, per_channel):
        return (f"{rows} channels x {per_channel} samples per step through the restated "
                f"reference fir1d_batched_f32 loop (63 taps, f32), channels spread over OpenMP "
                f"threads")

    def scipy_sample(self, per_channel):
        import scipy.signal as ss
        x = np.random.default_rng(1).uniform(-1, 1, per_channel)
        t0 = time.perf_counter()
        ss.lfilter(ss.firwin(self.K, 0.2, window="hamming"), 1.0, x)
        return per_channel, time.perf_counter() - t0, "scipy.signal.lfilter (direct form, f64)"


class Ragged(Workload):
    """4,096 signals, lengths log-uniform in [1,024, 4,194,304], taps log-uniform
    in [16, 2,048] (Hamming sinc, cutoff U[0.05, 0.45]), U[-1,1) samples; one
    persistent launch (lfilter semantics)."""
    name = "fir_ragged_4096"
    COUNT = 4096
    bound = "mixed"

    def __init__(self, torch, dev, precision, channels=None):
        import scipy.signal as ss
        import scir_gb300 as S
        self.S, self.torch, self.dev = S, torch, dev
        # AUTO: signals with long filters on the tensor cores (split-bf16, <= 1e-5),
        # the rest in FP32 on the CUDA cores
        self.precision = precision
        count = channels or self.COUNT
        self.n, self.k, cut = self.draw(count)
        taps = np.concatenate([ss.firwin(int(k), c, window="hamming") for k, c in zip(self.k, cut)])
        self.taps = torch.from_numpy(taps.astype(np.float32)).to(dev)
        g = torch.Generator(device=dev).manual_seed(0)
        self.x = torch.rand(int(self.n.sum()), device=dev, generator=g) * 2 - 1
        self.plan = S.RaggedPlan(self.n, self.k, S.FirMode.LFILTER, self.precision)
        self.y = torch.empty(self.plan.y_len, device=dev)
        self.kernel = ("ragged_kernel + fir_tc_kernel (tensor-core bucket), replayed from a "
                       "CUDA graph")
        self.graph = None

    @staticmethod
    def draw(count):
        """Signal lengths, tap counts and cutoffs of the ragged set (seeded)."""
        rng = np.random.default_rng(1)
        n = np.exp(rng.uniform(np.log(1024), np.log(4194304), count)).round().astype(np.int64)
        k = np.exp(rng.uniform(np.log(16), np.log(2048), count)).round().astype(np.int64)
        return n, k, rng.uniform(0.05, 0.45, count)

    @classmethod
    def config(cls):
        return {"workload": "ragged FIR: 4,096 signals, lengths log-uniform [1,024, 4,194,304], "
                            "taps log-uniform [16, 2,048] Hamming sinc (cutoff U[0.05,0.45]), "
                            "U[-1,1) f32, one persistent launch", "signals": cls.COUNT}

    def samples_per_step(self):
        return int(self.n.sum())

    def alg_bytes(self):
        return 8 * int(self.n.sum())

    def alg_flops(self):
        return 2.0 * self.plan.macs

    def floor_ms(self, fp32_tflops, bf16_tflops, hbm_gbs):
        """Time floor of the plan: per signal the larger of its bytes (input
        and output once) at the HBM peak and its multiply-adds at the peak of
        the unit that runs it (FP32 FMA, or the tensor cores' bf16 rate for
        one product), summed over the signals."""
        thr, _ = self.plan.tensor_cores()
        n_out = self.plan.n_out.astype(np.float64)
        tc = (self.k >= thr) & (n_out >= 16384) if thr else np.zeros(len(self.k), bool)
        fl = 2.0 * n_out * self.k
        peak = np.where(tc, bf16_tflops, fp32_tflops) * 1e12
        by = 4.0 * (self.n.astype(np.float64) + n_out)
        return 1e3 * float(np.maximum(fl / peak, by / (hbm_gbs * 1e9)).sum())

    def prepare(self):
        """Records the plan's launch (work-counter reset + persistent kernel)
        into a CUDA graph once; every step replays it.  Runs after the
        autotuner, which rebuilds the plan's tile table."""
        self.S.init(self.dev.index or 0)
        # split kernels + tensor-core launch (when the plan has that bucket) + the
        # CUDA-core launch; the roofline covers the whole step
        self.launches_per_step = 4 if self.plan.tensor_cores()[1] else 1
        self.roofline_launches = 1
        self.plan.run(self.x, self.taps, self.y)
        self.torch.cuda.synchronize()
        cs = self.torch.cuda.Stream(self.dev)
        self.graph = self.S.GraphCapture(cs)
        with self.graph:
            self.plan.run(self.x, self.taps, self.y, stream=cs)
        self.torch.cuda.synchronize()

    def step(self, stream, precision=None):
        if precision is not None and precision != self.precision:
            self.other_plan(precision).run(self.x, self.taps, self.y, stream=stream)
        elif self.graph is not None:
            self.graph.launch(stream)
        else:
            self.plan.run(self.x, self.taps, self.y, stream=stream)

    def other_plan(self, precision):
        """A plan of the same signals at another precision (FP32: no
        tensor-core bucket), autotuned once on first use."""
        plans = self.__dict__.setdefault("plans", {})
        if precision not in plans:
            plan = self.S.RaggedPlan(self.n, self.k, self.S.FirMode.LFILTER, precision)
            plan.autotune(self.x, self.taps, self.y)
            plans[precision] = plan
        return plans[precision]

    def autotune(self):
        thr, ms = self.plan.autotune(self.x, self.taps, self.y)
        tc, cnt = self.plan.tensor_cores()
        return (f"16 outputs per thread from {thr} taps; tensor cores from "
                f"{tc if tc and tc < (1 << 30) else 'never'} taps ({cnt} signals) ({ms:.3f} ms)")

    def per_signal_ms(self, stream):
        """The same work as one scir_fir_batched_f32 launch per signal."""
        t = self.torch
        xo, to = self.plan.x_off, self.plan.taps_off
        e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(len(self.n)):
            xi = self.x[xo[i]:xo[i] + self.n[i]].view(1, -1)
            ti = self.taps[to[i]:to[i] + self.k[i]]
            yi = self.y[self.plan.y_off[i]:self.plan.y_off[i] + self.n[i]].view(1, -1)
            self.S.fir_batched(xi, ti, self.S.FirMode.LFILTER, self.precision, out=yi,
                               stream=stream)
        e1.record(stream)
        t.cuda.synchronize()
        return e0.elapsed_time(e1)

    def max_rel_err(self, precision=None):
        import scipy.signal as ss
        self.step(None, precision)
        self.torch.cuda.synchronize()
        errs = []
        for i in np.argsort(self.n)[:: max(1, len(self.n) // 6)][:6]:
            xi = self.x[self.plan.x_off[i]:self.plan.x_off[i] + self.n[i]].cpu().numpy().astype(np.float64)
            ti = self.taps[self.plan.taps_off[i]:self.plan.taps_off[i] + self.k[i]].cpu().numpy()
            ref = ss.lfilter(ti.astype(np.float64), 1, xi)
            yi = self.y[self.plan.y_off[i]:self.plan.y_off[i] + self.n[i]].cpu().numpy()
            errs.append(np.max(np.abs(yi - ref)) / np.max(np.abs(ref)))
        return float(max(errs))

    def host_setup(self):
        return 0, 0

    def host_step(self):
        self.step(None)

    def cpu_sample(self, O, threads, per_channel):
        rng = np.random.default_rng(1)
        x = rng.uniform(-1, 1, (threads, per_channel)).astype(np.float32)
        taps = np.ones(self.median_k(), np.float32)
        t0 = time.perf_counter()
        O.fir1d_batched_f32(x, taps)
        return threads * per_channel, time.perf_counter() - t0

    def median_k(self):
        return int(np.median(self.draw(self.COUNT)[1]))

    def cpu_row_len(self):
        return 1 << 19  # about the mean signal length (504 k)

    def cpu_sample_desc(self, rows, per_channel):
        return (f"{rows} signals x {per_channel} samples per step through the restated "
                f"reference fir1d_batched_f32 loop at the median tap count ({self.median_k()})")

    def scipy_sample(self, per_channel):
        import scipy.signal as ss
        x = np.random.default_rng(1).uniform(-1, 1, per_channel)
        t0 = time.perf_counter()
        ss.lfilter(ss.firwin(self.median_k(), 0.25, window="hamming"), 1.0, x)
        return per_channel, time.perf_counter() - t0, "scipy.signal.lfilter at the median tap count"


class Sos(Workload):
    """16,384 ch x 131,072 N(0,1) f32 samples, butter(8, [0.001, 0.002]) band-pass
    as 8 sections; sosfilt (or sosfiltfilt with odd padding and zi)."""
    name = "sosfilt_16384"
    B, N = 16384, 131072
    cpu_dtype = "f64"
    bound = "hbm"
    filtfilt = False

    def __init__(self, torch, dev, precision, channels=None):
        import scipy.signal as ss
        import scir_gb300 as S
        self.S, self.torch, self.dev = S, torch, dev
        # f32 data: AUTO is the coupled-form FP32 state (<= 1e-5 vs FP64 on this
        # filter); SOS precision names select a mode directly
        if isinstance(precision, S.SosPrecision):
            self.sprec = precision
        else:
            self.sprec = {S.Precision.AUTO: S.SosPrecision.FP32_COUPLED,
                          S.Precision.FP32: S.SosPrecision.FP32,
                          S.Precision.REF_EXACT: S.SosPrecision.FP64_EXACT}.get(
                              precision, S.SosPrecision.FP64)
        self.precision = precision
        if channels:
            self.B = channels
        self.sos = self.cpu_sos()
        g = torch.Generator(device=dev).manual_seed(0)
        self.x = torch.randn((self.B, self.N), device=dev, generator=g)
        self.y = torch.empty_like(self.x)
        # FP32 and coupled FP32 state run the warp-pipelined sos_pipe_kernel (both
        # passes in one launch for filtfilt); FP64 state the per-channel kernels
        fp32 = self.sprec in (S.SosPrecision.FP32, S.SosPrecision.FP32_COUPLED)
        self.kernel = ("sos_pipe_kernel" if fp32 else
                       "sosfiltfilt_kernel" if self.filtfilt else "sosfilt_kernel")
        self.bound = "hbm" if self.sprec in (S.SosPrecision.FP32,
                                             S.SosPrecision.FP32_COUPLED) else "fp64"

    def alg_flops(self):
        # 9 flops per section per sample per pass (5 multiplies, 4 adds)
        return 9.0 * 8 * self.B * self.N * (2 if self.filtfilt else 1)

    @classmethod
    def config(cls):
        return {"workload": ("sosfiltfilt" if cls.filtfilt else "sosfilt") +
                            ": 16,384 ch x 131,072 f32 N(0,1) samples, butter(8, [0.001, 0.002]) "
                            "band-pass, 8 sections" + (", odd padding 51 + sosfilt_zi"
                                                       if cls.filtfilt else ""),
                "channels": cls.B, "samples_per_channel": cls.N, "sections": 8}

    def samples_per_step(self):
        return self.B * self.N

    def alg_bytes(self):
        return (16 if self.filtfilt else 8) * self.B * self.N

    def step(self, stream, precision=None):
        p = self.sprec if precision is None else {self.S.Precision.FP32: self.S.SosPrecision.FP32}.get(
            precision, self.sprec)
        if self.filtfilt:
            self.S.sosfiltfilt_f32(self.sos, self.x, precision=p, out=self.y, stream=stream)
        else:
            self.S.sosfilt_f32(self.sos, self.x, precision=p, out=self.y, stream=stream)

    def max_rel_err(self, precision=None):
        import scipy.signal as ss
        rows = [0, self.B - 1]
        self.step(None, precision)
        self.torch.cuda.synchronize()
        x = self.x[rows].cpu().numpy().astype(np.float64)
        ref = ss.sosfiltfilt(self.sos, x, axis=1) if self.filtfilt else ss.sosfilt(self.sos, x, axis=1)
        y = self.y[rows].cpu().numpy()
        return float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))

    def host_setup(self):
        return 0, 0

    def host_step(self):
        self.step(None)

    @staticmethod
    def cpu_sos():
        import scipy.signal as ss
        return ss.butter(8, [0.001, 0.002], btype="bandpass", output="sos")

    def cpu_sample(self, O, threads, per_channel):
        rng = np.random.default_rng(1)
        x = rng.standard_normal((threads, per_channel))
        sos = self.cpu_sos()
        t0 = time.perf_counter()
        if self.filtfilt:
            O.filtfilt_ref_f64(sos, x)
        else:
            O.sosfilt_f64(sos, x)
        return threads * per_channel, time.perf_counter() - t0

    def scipy_sample(self, per_channel):
        import scipy.signal as ss
        x = np.random.default_rng(1).standard_normal(per_channel)
        sos = self.cpu_sos()
        t0 = time.perf_counter()
        if self.filtfilt:
            ss.sosfiltfilt(sos, x)
        else:
            ss.sosfilt(sos, x)
        return per_channel, time.perf_counter() - t0, (
            "scipy.signal." + ("sosfiltfilt (odd pad, zi)" if self.filtfilt else "sosfilt") + ", f64")

    def cpu_row_len(self):
        return self.N

    def cpu_sample_desc(self, rows, per_channel):
        return (f"{rows} channels x {per_channel} samples per step through the restated "
                f"reference DF2T {'filtfilt' if self.filtfilt else 'sosfilt'} (f64)")


class SosFiltFilt(Sos):
    name = "sosfiltfilt_16384"
    filtfilt = True


WORKLOADS = {"resample": Resample, "fir_long": FirLong, "fir_short": FirShort,
             "ragged": Ragged, "sosfilt": Sos, "sosfiltfilt": SosFiltFilt}


# ----------------------------------------------------------------------------- runners

def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def smi_index(local_rank: int) -> int:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        parts = [p.strip() for p in vis.split(",") if p.strip()]
        if local_rank < len(parts) and parts[local_rank].isdigit():
            return int(parts[local_rank])
    return local_rank


def calibrate_cpu(W, O, threads, target_s):
    """A bounded sample of the workload that takes about target_s on
    `threads` host threads: (rows, samples per row).  Rows grow to the
    configuration's own length first, then more rows (a multiple of the
    thread count) are taken, up to the configuration's own channel or signal
    count: a step never holds more than the workload."""
    full = W.cpu_row_len()
    cap = getattr(W, "B", None) or getattr(W, "COUNT", None)
    rows, per = threads, 64
    while True:
        n, dt = W.cpu_sample(O, rows, per)
        if dt >= 0.25 or per >= full:
            break
        per = min(full, per * 4)
    scale = target_s / max(dt, 1e-6)
    if per < full and scale > 1:
        per2 = min(full, int(per * scale))
        scale /= per2 / per
        per = per2
    if per >= full:
        rows = max(threads, int(round(rows * scale / threads)) * threads)
        if cap:
            rows = min(rows, cap)
    else:
        per = max(16, int(per * scale))
    return rows, per


def cpu_rates(W, O, threads, target_s, reps):
    """Rate of the restated reference loop on `threads` host threads, over
    `reps` bounded samples of ~target_s each: (Gsamples/s, sample text,
    seconds per sample)."""
    O.set_threads(threads)
    rows, per = calibrate_cpu(W, O, threads, target_s)
    tot_n, tot_t = 0, 0.0
    for _ in range(reps):
        n, dt = W.cpu_sample(O, rows, per)
        tot_n += n
        tot_t += dt
    return (tot_n / tot_t / 1e9, W.cpu_sample_desc(rows, per) + f", {threads} host thread(s)",
            tot_t / reps)


def scipy_rate(W, target_s=2.0):
    """SciPy's FP64 implementation of the same operation on one host core, a
    secondary CPU reference."""
    per = 4096
    while True:
        n, dt, what = W.scipy_sample(per)
        if dt >= 0.25 or per >= 1 << 24:
            break
        per *= 4
    per = max(1024, int(per * target_s / max(dt, 1e-6)))
    n, dt, what = W.scipy_sample(per)
    return {"value": n / dt / 1e9, "unit": W.unit, "cores": 1,
            "sample": f"1 channel x {per} samples through {what}"}


def run_reference(args):
    """The reference arm: the C restatement of the reference's CPU loop for
    the workload (oracle/), timed on the host cores.  This package is never
    imported here, so no kernel library of this repository is loaded."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle as O
    import torch  # noqa: F401  (same interpreter as the GPU arm)

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    W = WORKLOADS[args.workload].__new__(WORKLOADS[args.workload])
    per_step_s = max(0.5, min(3.0, 90.0 / max(1, args.steps + args.warmup)))
    rows, per = calibrate_cpu(W, O, threads, per_step_s)
    for _ in range(args.warmup):
        W.cpu_sample(O, rows, per)
    total_n, total_t = 0, 0.0
    for _ in range(args.steps):
        n, dt = W.cpu_sample(O, rows, per)
        total_n += n
        total_t += dt
    value = total_n / total_t / 1e9
    one, one_desc, _ = cpu_rates(W, O, 1, 3.0, 1)
    cfg = WORKLOADS[args.workload].config()
    line = {"impl": "reference", "metric": W.metric, "value": value, "unit": W.unit,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * total_t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": W.cpu_dtype, "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {"value": value, "unit": W.unit, "cores": threads, "kind": "port",
                             "sample": W.cpu_sample_desc(rows, per) + f", {threads} host threads"},
            "single_core": {"value": one, "unit": W.unit, "cores": 1, "sample": one_desc},
            "scipy": scipy_rate(W),
            "e2e": {"value": value, "unit": W.unit, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference is Rust and no Rust toolchain is installed on this host; "
                    "this arm times the C restatement of its CPU loop (oracle/scir_oracle.c) "
                    "on a bounded sample of the configuration per step, on all host threads; "
                    "single_core is the same loop on one thread (the reference is "
                    "single-threaded); scipy is SciPy's FP64 implementation on one core"}
    print(json.dumps(line), flush=True)
    return 0


def max_over_ranks(torch, value, dev, world):
    """The largest of the ranks' values, on every rank (the slowest rank sets
    the job's time); `value` itself with one rank."""
    t = torch.tensor([float(value)], device=dev, dtype=torch.float64)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def time_steps(torch, W, stream, steps, precision=None, flush=None):
    """Per-step milliseconds of `steps` steps, CUDA events on the launch stream."""
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        if flush is not None:
            flush.fill_(float(i))  # 256 MB write evicts L2 (129 MB) between steps
        ev0[i].record(stream)
        W.step(stream, precision)
        ev1[i].record(stream)
    torch.cuda.synchronize()
    return [ev0[i].elapsed_time(ev1[i]) for i in range(steps)]


def roofline(W, kern_ms, peaks, fma):
    """Roofline of the dominant kernel: the algorithmic work of one launch
    over its mean duration, against the binding peak."""
    rl = getattr(W, "roofline_launches", W.launches_per_step)
    if W.bound == "mixed":
        floor = W.floor_ms(fma(False), peaks["bf16_tflops"], peaks["hbm_gbs"])
        return {"bound": "mixed", "achieved": floor, "peak": kern_ms, "unit": "ms (floor vs measured)",
                "frac": floor / kern_ms, "traffic": profile_traffic(W.name), "kernel": W.kernel,
                "kernel_ms": kern_ms,
                "peak_source": "per-signal floor max(bytes / HBM, flops / unit peak) summed: FP32 "
                               "FMA peak measured live by scir_probe_fma_peak, HBM and bf16 " +
                               peaks["source"]}
    if W.bound == "hbm":
        achieved = W.alg_bytes() / rl / (kern_ms / 1e3) / 1e9
        peak, unit, src = peaks["hbm_gbs"], "GB/s", peaks["source"]
    elif W.bound == "tensor" and W.products() > 1:
        achieved = W.alg_flops() / rl / (kern_ms / 1e3) / 1e12
        peak, unit, src = peaks["bf16_tflops"], "TFLOP/s", peaks["source"]
    else:
        fp64 = W.bound == "fp64"
        achieved = W.alg_flops() / rl / (kern_ms / 1e3) / 1e12
        peak, unit = fma(fp64), "TFLOP/s"
        src = "measured live by scir_probe_fma_peak (" + ("FP64 DFMA" if fp64 else "FP32 FFMA") + ")"
    out = {"bound": W.bound, "achieved": achieved, "peak": peak, "unit": unit,
           "frac": achieved / peak, "traffic": profile_traffic(W.name), "kernel": W.kernel,
           "kernel_ms": kern_ms, "peak_source": src}
    if W.bound == "tensor" and W.products() > 1:
        # the split form issues products() tensor products per algorithmic one
        out["products_issued"] = W.products()
        out["issued_frac"] = achieved * W.products() / peak
    return out


def resample_record(torch, S, dev, stream, steps, peaks, fma):
    """The polyphase resample configuration (256 x 1,048,576, 160/147) as a
    sub-record of the default line: device rate, HBM roofline, error, and the
    tensor-core (BF16X3) form beside the chosen one."""
    W = Resample(torch, dev, S.Precision.AUTO)
    tuned = W.autotune()
    for _ in range(3):
        W.step(stream)
    per = time_steps(torch, W, stream, steps)
    ms = statistics.mean(per)
    rec = {"workload": Resample.config()["workload"], "precision": "AUTO", "autotune": tuned,
           "value": W.samples_per_step() / (ms / 1e3) / 1e9, "unit": W.unit, "ms_per_step": ms,
           "roofline": roofline(W, ms, peaks, fma), "max_rel_err_vs_fp64": W.max_rel_err(),
           "gpu_launches": W.launches_per_step * steps}
    for _ in range(3):
        W.step(stream, S.Precision.BF16X3)
    tc = statistics.mean(time_steps(torch, W, stream, steps, S.Precision.BF16X3))
    rec["bf16x3"] = {"ms_per_step": tc, "value": W.samples_per_step() / (tc / 1e3) / 1e9,
                     "max_rel_err_vs_fp64": W.max_rel_err(S.Precision.BF16X3),
                     "kernel": "poly_tc_kernel (tensor cores) + tap-operand build"}
    del W
    torch.cuda.empty_cache()
    return rec


def run_ours(args):
    import torch
    import torch.distributed as dist

    import scir_gb300 as S

    rank, world, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    peaks = load_peaks()
    fma_cache = {}

    def fma(fp64):
        if fp64 not in fma_cache:
            fma_cache[fp64] = S.probe_fma_peak(fp64)
        return fma_cache[fp64]

    if args.precision in S.Precision.__members__:
        prec = S.Precision[args.precision]
    elif args.workload in ("sosfilt", "sosfiltfilt") and args.precision in S.SosPrecision.__members__:
        prec = S.SosPrecision[args.precision]
    else:
        raise SystemExit(f"unknown precision {args.precision} for {args.workload}")
    W = WORKLOADS[args.workload](torch, dev, prec, args.channels)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            dist.barrier(device_ids=[local])

    tuned = None if args.no_autotune else W.autotune()
    if hasattr(W, "prepare"):
        W.prepare()
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev) if W.flush_l2 else None
    with ClockSampler(smi_index(local)) as clk:
        # the warm-up runs after the sampler's start-up wait, so the timed
        # steps follow busy steps rather than a ~0.3 s idle gap (at short
        # steps the first ones after an idle gap ran ~5 % slow)
        for _ in range(max(3, args.warmup)):
            W.step(stream)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        per_step = time_steps(torch, W, stream, args.steps, flush=flush)
    barrier()
    total_ms = max_over_ranks(torch, sum(per_step), dev, world)
    ms_step = total_ms / args.steps
    value = world * W.samples_per_step() * args.steps / (total_ms / 1e3) / 1e9

    # plain FP32 on the same inputs, for the chosen-vs-plain comparison
    plain = None
    if prec != S.Precision.FP32:
        for _ in range(3):
            W.step(stream, S.Precision.FP32)
        pms = statistics.mean(time_steps(torch, W, stream, args.steps, S.Precision.FP32,
                                         flush=flush))
        plain = {"value": W.samples_per_step() / (pms / 1e3) / 1e9, "unit": W.unit,
                 "ms_per_step": pms, "max_rel_err_vs_fp64": W.max_rel_err(S.Precision.FP32),
                 "chosen_speedup": pms / ms_step}
    err = W.max_rel_err()
    # the other tensor-core forms beside the chosen one (long-tap FIR)
    forms = None
    if isinstance(W, FirLong) and prec not in (S.Precision.FP32, S.Precision.REF_EXACT):
        forms = {}
        for f in (S.Precision.FP16X3, S.Precision.BF16X6, S.Precision.BF16X3):
            if f == prec:
                continue
            for _ in range(3):
                W.step(stream, f)
            xms = statistics.mean(time_steps(torch, W, stream, args.steps, f, flush=flush))
            forms[f.name] = {"ms_per_step": xms,
                             "value": W.samples_per_step() / (xms / 1e3) / 1e9,
                             "max_rel_err_vs_fp64": W.max_rel_err(f),
                             "vs_plain_fp32": (plain["ms_per_step"] / xms) if plain else None}

    # end to end through the host-buffer C-ABI call
    h2d, d2h = W.host_setup()
    for _ in range(max(1, args.warmup)):  # staging buffers, pinned pages, tuning: untimed
        W.host_step()
    torch.cuda.synchronize()
    # the pinned-copy rate of this host right now (the link is shared with the
    # other GPU of the superchip): the floor the host-buffer step can reach
    floor = None
    if h2d or d2h:
        cc = copy_ceiling(torch, mib=256, chunks=(4,))
        floor_s = max(h2d / (cc["h2d_4_streams_gbs"] * 1e9), d2h / (cc["d2h_4_streams_gbs"] * 1e9),
                      (h2d + d2h) / (cc["both_4_streams_gbs"] * 1e9))
        floor = {"value": W.samples_per_step() / floor_s / 1e9,
                 "h2d_gbs": cc["h2d_4_streams_gbs"], "d2h_gbs": cc["d2h_4_streams_gbs"],
                 "both_gbs": cc["both_4_streams_gbs"]}
    barrier()
    step_s = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t1 = time.perf_counter()
        W.host_step()
        step_s.append(time.perf_counter() - t1)  # host_step returns after its copies
    torch.cuda.synchronize()
    e2e_total_s = max_over_ranks(torch, time.perf_counter() - t0, dev, world)
    # the rate at the median step (a burst of host traffic from the other GPU
    # of the superchip slows single steps: the slowest and the total-time rate
    # are reported beside it)
    med_s = max_over_ranks(torch, statistics.median(step_s), dev, world)
    e2e_value = world * W.samples_per_step() / med_s / 1e9
    e2e = {"value": e2e_value, "unit": W.unit, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h,
           "value_total_time": world * W.samples_per_step() * args.steps / e2e_total_s / 1e9,
           "ms_per_step_median": 1e3 * statistics.median(step_s),
           "ms_per_step_min": 1e3 * min(step_s),
           "ms_per_step_max": 1e3 * max(step_s),
           "copy_floor": floor,
           "of_copy_floor": e2e_value / (world * floor["value"]) if floor else None} \
        if (h2d or d2h) else None

    kern_ms = statistics.mean(per_step) / getattr(W, "roofline_launches", W.launches_per_step)
    roof = roofline(W, kern_ms, peaks, fma)
    per_signal = None
    if hasattr(W, "per_signal_ms"):
        W.per_signal_ms(stream)  # warm
        per_signal = {"ms_per_step": W.per_signal_ms(stream),
                      "note": "the same signals, one scir_fir_batched_f32 launch each"}
    W.host_release()

    extra = None
    if args.workload == DEFAULT_WORKLOAD and not args.no_extra and args.channels is None:
        extra = resample_record(torch, S, dev, stream, args.steps, peaks, fma)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        import oracle as O
        threads = os.cpu_count() or 1
        v, desc, _ = cpu_rates(W, O, threads, 3.0, 3)
        v1, desc1, _ = cpu_rates(W, O, 1, 3.0, 1)
        cpu = {"value": v, "unit": W.unit, "cores": threads, "kind": "port", "sample": desc,
               "single_core": {"value": v1, "cores": 1, "sample": desc1}}
    clocks = clk.summary()
    if world > 1:
        dist.destroy_process_group()
    if rank != 0:
        return 0
    line = {
        "metric": W.metric, "value": value, "unit": W.unit, "n_gpus": world,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded torch generators on the device)",
        "config": run_config(W, prec, world),
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": W.launches_per_step * args.steps,
        "autotune": tuned,
        "max_rel_err_vs_fp64": err,
        "plain_fp32": plain,
        "tensor_core_forms": forms,
        "per_signal_launches": per_signal,
        "clocks": clocks,
    }
    if extra is not None:
        line["resample_poly_160_147"] = extra
    print(json.dumps(line), flush=True)
    return 0


def copy_ceiling(torch, mib=1024, chunks=(1, 4)):
    """Pinned host <-> device copy bandwidth in GB/s: one direction at a
    time and both at once, the buffer split into `chunks` copies on as many
    streams (the host-buffer entry points overlap copies in both directions
    with the kernels, so these bound their end-to-end rate)."""
    n = mib << 18  # floats
    h_in = torch.empty(n, dtype=torch.float32, pin_memory=True)
    h_out = torch.empty(n, dtype=torch.float32, pin_memory=True)
    d_in = torch.empty(n, dtype=torch.float32, device="cuda")
    d_out = torch.empty(n, dtype=torch.float32, device="cuda")
    h_in.fill_(1.0)
    out = {}
    for c in chunks:
        streams = [torch.cuda.Stream() for _ in range(c)]
        step = n // c

        def run(h2d, d2h):
            for i, st in enumerate(streams):
                with torch.cuda.stream(st):
                    sl = slice(i * step, (i + 1) * step)
                    if h2d:
                        d_in[sl].copy_(h_in[sl], non_blocking=True)
                    if d2h:
                        h_out[sl].copy_(d_out[sl], non_blocking=True)

        for name, h2d, d2h in (("h2d", True, False), ("d2h", False, True), ("both", True, True)):
            run(h2d, d2h)
            torch.cuda.synchronize()
            moved = 4 * n * ((1 if h2d else 0) + (1 if d2h else 0))
            rates = []
            for _ in range(5):  # trials of three copies each: median and best
                t0 = time.perf_counter()
                for _ in range(3):
                    run(h2d, d2h)
                torch.cuda.synchronize()
                rates.append(moved * 3 / (time.perf_counter() - t0) / 1e9)
            out[f"{name}_{c}_streams_gbs"] = statistics.median(rates)
            out[f"{name}_{c}_streams_best_gbs"] = max(rates)
    return out


def run_probe():
    import torch

    import scir_gb300 as S
    torch.cuda.set_device(0)
    line = {"probe": "FMA throughput of the CUDA cores (scir_probe_fma_peak) and pinned "
                     "host<->device copy bandwidth (1 GiB each way)",
            "fp32_tflops": [S.probe_fma_peak(False) for _ in range(3)],
            "fp64_tflops": [S.probe_fma_peak(True) for _ in range(3)],
            "copies": copy_ceiling(torch),
            "device": torch.cuda.get_device_name(0)}
    print(json.dumps(line), flush=True)
    return 0


def run_config(W, prec, world):
    """The workload's configuration as run: the class describes its default
    size, and --channels overrides the channel count."""
    cfg = dict(W.config(), channels=getattr(W, "B", None), precision=prec.name,
               parallelism=f"replicas x{world}")
    default = getattr(type(W), "B", None)
    if cfg["channels"] is not None and default is not None and cfg["channels"] != default:
        cfg["workload"] += f" (run with {cfg['channels']} channels instead of {default})"
    return cfg


DEFAULT_WORKLOAD = "fir_long"


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--precision", default="AUTO")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the resample sub-record of the default workload")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the library autotuner (default dispatch heuristics)")
    ap.add_argument("--channels", type=int, default=None,
                    help="override the channel count (profiling runs on a smaller case)")
    ap.add_argument("--probe-peaks", action="store_true",
                    help="print the measured FP32/FP64 FMA throughput and exit")
    args = ap.parse_args()
    if args.probe_peaks:
        return run_probe()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
