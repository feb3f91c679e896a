"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and call the library through its C
ABI; everything else runs on a CPU-only host.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


@pytest.fixture(scope="session")
def golden_signal():
    return dict(np.load(os.path.join(GOLDEN, "signal_fixtures.npz")))


@pytest.fixture(scope="session")
def golden_strain():
    return dict(np.load(os.path.join(GOLDEN, "strain_df2t.npz")))


@pytest.fixture(scope="session")
def golden_resample23():
    """The reference's baked resample_poly(2, 3) table as literal text and
    IEEE-754 bits (tests/golden/make_resample_golden.py)."""
    import json
    with open(os.path.join(GOLDEN, "resample23_table.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def cuda():
    """The CUDA device; a GPU test fails (never skips) when it is missing."""
    import torch
    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    import scir_gb300
    scir_gb300.load()
    assert scir_gb300.device_errors() == 0
    yield torch.device("cuda:0")
    # no kernel of the session may have given up a bounded device-side wait
    assert scir_gb300.device_errors() == 0


def normwise_err(y, ref):
    """max|y - ref| / max|ref| (0 for an all-zero reference)."""
    y = np.asarray(y, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.max(np.abs(ref)) if ref.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(y))) if y.size else 0.0
    return float(np.max(np.abs(y - ref)) / scale)
