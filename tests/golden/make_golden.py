#!/usr/bin/env python3
"""Regenerate the golden fixtures under tests/golden/ from the reference tree.

Run in a container where the reference checkout is present:

    python tests/golden/make_golden.py /path/to/scir-reference

It writes two files:

* ``signal_fixtures.npz`` -- the output of the reference's own fixture
  generator ``scripts/gen_signal_fixtures.py`` (SciPy designs of butter /
  cheby1 / bessel / notch SOS, their ``sosfilt`` responses, the no-pad
  forward-backward response and ``resample_poly(x, 2, 3)`` on
  ``linspace(0, 1, 32)``), executed unchanged in a scratch directory.
* ``strain_df2t.npz`` -- the strain-gauge input of
  ``crates/scir-iir-filters/test_data`` and the four SciPy butter(5)
  responses that ``crates/scir-iir-filters/src/filter.rs:287-428`` checks the
  DF2T loop against at 1e-12, cut to the first ``N_KEEP`` samples (the
  filters are causal, so a prefix of the expected output is the expected
  output of the prefix), plus the SOS matrices SciPy designs for those four
  cases (``butter(5, ..., fs=81, output='sos')``).

The test suite only reads the .npz files; it never needs the reference tree.
"""
from __future__ import annotations

import os
import runpy
import sys
import tempfile

import numpy as np
import scipy.signal as ss

N_KEEP = 8192
HERE = os.path.dirname(os.path.abspath(__file__))


def _load_two_column(path: str) -> np.ndarray:
    vals = []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 2:
                vals.append(float(parts[1]))
    return np.asarray(vals, np.float64)


def main(ref_root: str) -> None:
    # 1. the reference's fixture generator, unchanged, in a scratch cwd
    script = os.path.join(ref_root, "scripts", "gen_signal_fixtures.py")
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            runpy.run_path(script, run_name="__main__")
        finally:
            os.chdir(cwd)
        fx = os.path.join(tmp, "fixtures")
        arrays = {os.path.splitext(f)[0]: np.load(os.path.join(fx, f))
                  for f in sorted(os.listdir(fx)) if f.endswith(".npy")}
    np.savez_compressed(os.path.join(HERE, "signal_fixtures.npz"), **arrays)

    # 2. strain-gauge DF2T vectors
    td = os.path.join(ref_root, "crates", "scir-iir-filters", "test_data")
    x = _load_two_column(os.path.join(td, "bridge-strain-0-left-s-0-short.txt"))
    out = {"x": x[:N_KEEP], "n_full": np.int64(x.size)}
    cases = {
        "low_pass": dict(N=5, Wn=12.0, btype="lowpass"),
        "high_pass": dict(N=5, Wn=1.0, btype="highpass"),
        "band_pass": dict(N=5, Wn=[1.0, 10.0], btype="bandpass"),
        "band_stop": dict(N=5, Wn=[4.0, 5.0], btype="bandstop"),
    }
    for name, kw in cases.items():
        y = _load_two_column(os.path.join(td, f"test_filter_butter_{name}_expected.txt"))
        out[f"y_{name}"] = y[:N_KEEP]
        out[f"sos_{name}"] = ss.butter(kw["N"], kw["Wn"], btype=kw["btype"], fs=81.0, output="sos")
    np.savez_compressed(os.path.join(HERE, "strain_df2t.npz"), **out)
    print("wrote", sorted(arrays), "and strain_df2t.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout>")
    main(sys.argv[1])
