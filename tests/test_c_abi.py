"""The header compiles as C (gcc -std=c99 -Wall -Werror) and a C program
linked against the library gets the host-only results a Python caller gets:
the ABI version, the FIR output length, the host chunk plan, firwin and the
Butterworth band-pass of the 16,384-channel SOS workload (vs SciPy), and a
status plus message for a bad call.  No device is touched."""
import os
import shutil
import subprocess

import numpy as np
import pytest
import scipy.signal as ss

import scir_gb300 as S
from scir_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def c_output(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    _native.load()  # builds the library if needed
    lib = _native.lib_path()
    exe = str(tmp_path_factory.mktemp("c_abi") / "host_calls")
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi", "host_calls.c"), lib,
           "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return {line.split()[0]: line.split()[1:] for line in r.stdout.splitlines()}


def test_c_caller_basics(c_output):
    assert c_output["abi"] == ["1"]
    assert c_output["ok"] == ["ok"]
    assert c_output["valid_len"] == [str(65536 - 63 + 1)]
    assert c_output["plan"] == ["0", "9", "64"] + ["128"] * 7 + ["64"]
    assert c_output["bad"] == [str(S.ERR_INVALID_ARG), "message"]


def test_c_caller_designs_match_scipy(c_output):
    fw = c_output["firwin"]
    assert fw[0] == "0"
    np.testing.assert_allclose(np.array(fw[1:], float), ss.firwin(63, 0.2, window="hamming"),
                               rtol=0, atol=1e-15)
    bw = c_output["butter"]
    assert bw[0] == "0" and bw[1] == "8"
    sos = np.array(bw[2:], float).reshape(8, 6)
    ref = ss.butter(8, [0.001, 0.002], btype="bandpass", output="sos")
    # same system: compare frequency responses (section order and scaling may differ)
    w = np.linspace(0, np.pi * 0.01, 400)
    _, h1 = ss.sosfreqz(sos, worN=w)
    _, h2 = ss.sosfreqz(ref, worN=w)
    np.testing.assert_allclose(h1, h2, rtol=1e-7, atol=1e-9)
