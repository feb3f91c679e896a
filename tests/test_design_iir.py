"""Host-side IIR design: iirfilter (Butterworth, Chebyshev I, Bessel with the
three normalisations) and zpk2sos with the three pairings.

Known answers are the reference's own tests (crates/scir-iir-filters/src/
sos.rs:467-775, which hold Octave / MATLAB / SciPy values; filter_design.rs
butter_internal tests, extracted into tests/golden/design_zpk.json) and the
SOS designs in the reference's fixture file; the sweeps compare with
scipy.signal, whose iirfilter / zpk2sos the reference follows.  No GPU.
"""
import json
import os

import numpy as np
import pytest

import scir_gb300 as sg

ss = pytest.importorskip("scipy.signal")

# (zeros, poles, gain, {pairing: expected sos}, tol) from sos.rs:467-755
_D = np.pi / 180.0


def _jackson(thetas_z, thetas_p, mags, extra_z=()):
    z = [np.exp(1j * t * _D) for t in thetas_z]
    z = z + [v.conjugate() for v in z] + list(extra_z)
    p = [m * np.exp(1j * t * _D) for t, m in zip(thetas_p, mags)]
    p = p + [v.conjugate() for v in p]
    return z, p


_JZ1, _JP1 = _jackson([22.5, 45.0, 77.5], [22.5, 45.0, 77.5], [0.8, 0.6, 0.9])
_JZ2, _JP2 = _jackson([85.0, 10.0], [22.5, 45.0, 77.5], [0.8, 0.6, 0.9], [1.0, -1.0])
_BOTH = ("nearest", "keep_odd")

KNOWN = [
    # sos.rs:473 test_basic_1
    ([-1, -1], [0.57149 + 0.29360j, 0.57149 - 0.29360j], 1.0,
     {k: [[1, 2, 1, 1, -1.14298, 0.41280]] for k in _BOTH}, 1e-4),
    # :489 test_basic_2
    ([1j, -1j], [0.9, -0.9, 0.7j, -0.7j], 1.0,
     {k: [[1, 0, 1, 1, 0, 0.49], [1, 0, 0, 1, 0, -0.81]] for k in _BOTH}, 1e-4),
    # :508 test_basic_3
    ([], [0.8, -0.5 + 0.25j, -0.5 - 0.25j], 1.0,
     {k: [[1, 0, 0, 1, 1, 0.3125], [1, 0, 0, 1, -0.8, 0]] for k in _BOTH}, 1e-4),
    # :527 test_basic_4
    ([1, 1, 0.9j, -0.9j], [0.99 + 0.01j, 0.99 - 0.01j, 0.1 + 0.9j, 0.1 - 0.9j], 1.0,
     {k: [[1, 0, 0.81, 1, -0.2, 0.82], [1, -2, 1, 1, -1.98, 0.9802]] for k in _BOTH}, 1e-4),
    # :546 test_basic_5 (nearest and keep_odd differ)
    ([0.9 + 0.1j, 0.9 - 0.1j, -0.9], [0.75 + 0.25j, 0.75 - 0.25j, 0.9], 1.0,
     {"nearest": [[1, 0.9, 0, 1, -1.5, 0.625], [1, -1.8, 0.82, 1, -0.9, 0]],
      "keep_odd": [[1, -1.8, 0.82, 1, -1.5, 0.625], [1, 0.9, 0, 1, -0.9, 0]]}, 1e-4),
    # :580 test_basic_6
    ([-0.3090 + 0.9511j, -0.3090 - 0.9511j, 0.8090 + 0.5878j, 0.8090 - 0.5878j, -1.0],
     [-0.3026 + 0.9312j, -0.3026 - 0.9312j, 0.7922 + 0.5755j, 0.7922 - 0.5755j, -0.9791], 1.0,
     {k: [[1, 1, 0, 1, 0.97915, 0], [1, 0.61803, 1, 1, 0.60515, 0.95873],
          [1, -1.61803, 1, 1, -1.58430, 0.95873]] for k in _BOTH}, 1e-4),
    # :613 test_basic_7
    ([-1 - 1.4142j, -1 + 1.4142j, -0.625 - 1.0533j, -0.625 + 1.0533j],
     [-0.2 - 0.6782j, -0.2 + 0.6782j, -0.1 - 0.5385j, -0.1 + 0.5385j], 4.0,
     {k: [[4, 8, 12, 1, 0.2, 0.3], [1, 1.25, 1.5, 1, 0.4, 0.5]] for k in _BOTH}, 1e-3),
    # :640 test_basic_8
    ([], [0.2, -0.5 + 0.25j, -0.5 - 0.25j], 1.0,
     {k: [[1, 0, 0, 1, -0.2, 0], [1, 0, 0, 1, 1, 0.3125]] for k in _BOTH}, 1e-4),
    # :663 test_jackson_1
    (_JZ1, _JP1, 1.0,
     {k: [[1, -1.41421, 1, 1, -0.84853, 0.36], [1, -1.84776, 1, 1, -1.47821, 0.64],
          [1, -0.43288, 1, 1, -0.38959, 0.81]] for k in _BOTH}, 1e-4),
    # :699 test_jackson_2
    (_JZ2, _JP2, 1.0,
     {k: [[1, 0, -1, 1, -0.84853, 0.36], [1, -1.96962, 1, 1, -1.47821, 0.64],
          [1, -0.17431, 1, 1, -0.38959, 0.81]] for k in _BOTH}, 1e-4),
    # :739 test_pairing (all three pairings)
    ([-1, -0.5 - 0.5j, -0.5 + 0.5j], [0.75, 0.8 + 0.1j, 0.8 - 0.1j], 1.0,
     {"nearest": [[1, 1, 0.5, 1, -0.75, 0], [1, 1, 0, 1, -1.6, 0.65]],
      "keep_odd": [[1, 1, 0, 1, -0.75, 0], [1, 1, 0.5, 1, -1.6, 0.65]],
      "minimal": [[0, 1, 1, 0, 1, -0.75], [1, 1, 0.5, 1, -1.6, 0.65]]}, 1e-4),
]

_PAIR = {"nearest": sg.SosPairing.NEAREST, "keep_odd": sg.SosPairing.KEEP_ODD,
         "minimal": sg.SosPairing.MINIMAL}


@pytest.mark.parametrize("case", range(len(KNOWN)))
def test_zpk2sos_reference_known_answers(case):
    z, p, k, expected, tol = KNOWN[case]
    for pairing, sos in expected.items():
        got = sg.zpk2sos(z, p, k, _PAIR[pairing])
        np.testing.assert_allclose(got, np.asarray(sos, float), atol=tol, rtol=0,
                                   err_msg=f"pairing {pairing}")
        # and SciPy's own zpk2sos on the same input
        ref = ss.zpk2sos(np.asarray(z, complex), np.asarray(p, complex), k, pairing=pairing)
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14)


def test_butter_reference_known_answer():
    """sos.rs:757-775: butter(5, [12], 'low', fs=81, output='sos')."""
    sos = sg.butter(5, 12.0, "low", fs=81.0)
    expected = [[0.00659168, 0.01318336, 0.00659168, 1.0, -0.33136391, 0.0],
                [1.0, 2.0, 1.0, 1.0, -0.72429772, 0.21290681],
                [1.0, 1.0, 0.0, 1.0, -0.95708485, 0.60273144]]
    np.testing.assert_allclose(sos, expected, atol=1e-4, rtol=0)
    np.testing.assert_allclose(sos, ss.butter(5, 12.0, "low", fs=81.0, output="sos"),
                               rtol=1e-13, atol=1e-16)


_BANDS = [("low", 0.3), ("high", 0.2), ("bandpass", [0.1, 0.4]), ("bandstop", [0.2, 0.6])]


@pytest.mark.parametrize("btype,wn", _BANDS)
@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5, 8, 13, 32])
def test_butter_cheby1_match_scipy(order, btype, wn):
    for fs in (None, 48000.0):
        w = wn if fs is None else np.asarray(wn) * fs / 2
        got = sg.butter(order, w, btype, fs=fs)
        ref = ss.butter(order, w, btype, fs=fs, output="sos")
        np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-13)
        for rp in (0.1, 1.0, 3.0):
            got = sg.cheby1(order, rp, w, btype, fs=fs)
            ref = ss.cheby1(order, rp, w, btype, fs=fs, output="sos")
            np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-13)


@pytest.mark.parametrize("norm", ["phase", "delay", "mag"])
@pytest.mark.parametrize("order", list(range(0, 26)))
def test_bessel_matches_scipy(order, norm):
    # Bessel poles come from a root solve (Aberth + double-double Newton);
    # "mag" also solves for the -3 dB frequency, so it gets a looser bound.
    rtol = 1e-12 if norm != "mag" else 1e-10
    for btype, wn in _BANDS:
        got = sg.bessel(order, wn, btype, norm=norm)
        ref = ss.bessel(order, wn, btype, norm=norm, output="sos")
        np.testing.assert_allclose(got, ref, rtol=rtol, atol=1e-13)


@pytest.mark.parametrize("family,extra", [("butter", {}), ("cheby1", {"rp": 0.5}),
                                          ("bessel", {}), ("bessel", {"norm": "mag"})])
@pytest.mark.parametrize("btype,wn", _BANDS)
def test_zpk_output_matches_scipy(family, extra, btype, wn):
    order = 7
    fn = {"butter": sg.butter, "cheby1": sg.cheby1, "bessel": sg.bessel}[family]
    sfn = {"butter": ss.butter, "cheby1": ss.cheby1, "bessel": ss.bessel}[family]
    if family == "cheby1":
        z, p, k = fn(order, extra["rp"], wn, btype, output="zpk")
        zr, pr, kr = sfn(order, extra["rp"], wn, btype, output="zpk")
    else:
        z, p, k = fn(order, wn, btype, output="zpk", **extra)
        zr, pr, kr = sfn(order, wn, btype, output="zpk", **extra)

    def key(v):
        return np.asarray(sorted(np.round(v, 9), key=lambda c: (c.real, c.imag)))

    assert z.size == np.asarray(zr).size and p.size == np.asarray(pr).size
    np.testing.assert_allclose(np.sort_complex(key(z)), np.sort_complex(key(zr)), atol=1e-8)
    np.testing.assert_allclose(np.sort_complex(key(p)), np.sort_complex(key(pr)), atol=1e-8)
    assert k == pytest.approx(kr, rel=1e-10)


def test_zpk2sos_random_systems_match_scipy():
    rng = np.random.default_rng(11)
    for trial in range(300):
        nzc, nzr = rng.integers(0, 4), rng.integers(0, 4)
        npc, npr = rng.integers(0, 4), rng.integers(0, 4)
        zc = rng.uniform(0.2, 1.2, nzc) * np.exp(1j * rng.uniform(0.05, np.pi - 0.05, nzc))
        pc = rng.uniform(0.1, 0.98, npc) * np.exp(1j * rng.uniform(0.05, np.pi - 0.05, npc))
        z = np.concatenate([zc, zc.conj(), rng.uniform(-1.2, 1.2, nzr)])
        p = np.concatenate([pc, pc.conj(), rng.uniform(-0.98, 0.98, npr)])
        rng.shuffle(z)
        rng.shuffle(p)
        k = float(rng.uniform(0.1, 3.0))
        for pairing in ("nearest", "keep_odd", "minimal"):
            if pairing == "minimal" and z.size > p.size:
                with pytest.raises(sg.GpuError):
                    sg.zpk2sos(z, p, k, _PAIR[pairing])
                continue
            if p.size + z.size == 0:
                continue
            try:
                ref = ss.zpk2sos(z, p, k, pairing=pairing)
            except (ValueError, IndexError):
                # systems SciPy cannot pair (e.g. a last real pole with only
                # complex zeros left) are refused here too
                with pytest.raises(sg.GpuError):
                    sg.zpk2sos(z, p, k, _PAIR[pairing])
                continue
            got = sg.zpk2sos(z, p, k, _PAIR[pairing])
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-13,
                                       err_msg=f"trial {trial} {pairing}")


def test_zpk2sos_empty_system():
    np.testing.assert_array_equal(sg.zpk2sos([], [], 2.5), [[2.5, 0, 0, 1, 0, 0]])


@pytest.mark.parametrize("call", [
    lambda: sg.butter(4, 0.0),                         # Wn must be > 0
    lambda: sg.butter(4, 1.0),                         # Wn must be < 1 (Nyquist)
    lambda: sg.butter(4, 30.0, fs=50.0),               # above fs / 2
    lambda: sg.butter(4, [0.4, 0.2], "bandpass"),      # edges must increase
    lambda: sg.cheby1(4, 0.0, 0.3),                    # rp must be > 0
    lambda: sg.bessel(26, 0.3),                        # above the Bessel range
    lambda: sg.butter(-1, 0.3),                        # negative order
    lambda: sg.zpk2sos([0.5 + 0.5j], [0.1], 1.0),      # unpaired complex zero
])
def test_design_errors(call):
    with pytest.raises(sg.GpuError):
        call()


def test_sos_capacity_reported():
    lib = sg.load()
    import ctypes
    wn = np.array([0.2, 0.3])
    nsec = ctypes.c_int(-1)
    assert lib.scir_iirfilter_sos(6, 0, 2, sg._ptr(wn), 0.0, -1.0, None, 0, ctypes.byref(nsec)) == 0
    assert nsec.value == 6
    buf = np.zeros((5, 6))
    assert lib.scir_iirfilter_sos(6, 0, 2, sg._ptr(wn), 0.0, -1.0, sg._ptr(buf), 5,
                                  ctypes.byref(nsec)) == sg.ERR_SHAPE
    assert not buf.any()


# ------------------------------------------------ pinned by the reference's design tests
_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_DESIGN = json.load(open(os.path.join(_GOLDEN, "design_zpk.json")))
_BT = {"LowPass": "low", "HighPass": "high", "BandPass": "bandpass", "BandStop": "bandstop"}


def _sorted_c(v):
    v = np.asarray(v, complex)
    return v[np.lexsort((np.round(v.real, 9), np.round(v.imag, 9)))]


@pytest.mark.parametrize("case", _DESIGN, ids=[c["name"] for c in _DESIGN])
def test_butter_zpk_reference_known_answers(case):
    """crates/scir-iir-filters/src/filter_design.rs butter_internal(N, ..., None) tests."""
    z, p, k = sg.butter(case["order"], case["wn"], _BT[case["btype"]], output="zpk")
    ze = np.array([complex(a, b) for a, b in case["z"]])
    pe = np.array([complex(a, b) for a, b in case["p"]])
    assert z.size == ze.size and p.size == pe.size
    tol = case["tol"]
    np.testing.assert_allclose(_sorted_c(z), _sorted_c(ze), atol=tol, rtol=0)
    np.testing.assert_allclose(_sorted_c(p), _sorted_c(pe), atol=tol, rtol=0)
    assert abs(k - case["k"]) <= tol * max(1.0, abs(case["k"]))


@pytest.mark.parametrize("order", range(25))
def test_butter_highpass_zeros_at_dc(order):
    """filter_design.rs test_butter__basic_digital_z_plane: HighPass(0.01), N < 25."""
    z, p, _ = sg.butter(order, 0.01, "high", output="zpk")
    assert z.size == order and np.all(z == 1.0)
    assert np.all(np.abs(p) <= 1.0)


_FIXTURE_DESIGNS = {
    # tests/golden/signal_fixtures.npz keys -> the design the reference's
    # scripts/gen_signal_fixtures.py made them with (Wn normalised, no fs)
    "butter_sos": lambda: sg.butter(4, 0.2),
    "cheby_sos": lambda: sg.cheby1(4, 1.0, 0.2),
    "bessel_sos": lambda: sg.bessel(4, 0.2),
    "bessel_lp_delay_sos": lambda: sg.bessel(4, 0.2, norm="delay"),
    "bessel_lp_mag_sos": lambda: sg.bessel(4, 0.2, norm="mag"),
    "butter_hp_sos": lambda: sg.butter(4, 0.3, "high"),
    "cheby_hp_sos": lambda: sg.cheby1(4, 1.0, 0.3, "high"),
    "bessel_hp_sos": lambda: sg.bessel(4, 0.3, "high", norm="phase"),
}


@pytest.mark.parametrize("key", sorted(_FIXTURE_DESIGNS))
def test_design_matches_reference_fixtures(key):
    fx = np.load(os.path.join(_GOLDEN, "signal_fixtures.npz"))
    np.testing.assert_allclose(_FIXTURE_DESIGNS[key](), fx[key], rtol=1e-11, atol=1e-14)


# ------------------------------------------------------------------ firwin
_FIRWIN_BANDS = [(0.2, True), ([0.1, 0.3], False), ([0.1, 0.3], True), (0.4, False),
                 ([0.1, 0.2, 0.5, 0.7], True), ([0.1, 0.2, 0.5, 0.7], False)]
_WINDOWS = ["hamming", ("kaiser", 8.6), ("kaiser", 5.0), "hann", "blackman", "boxcar"]


@pytest.mark.parametrize("numtaps", [1, 2, 3, 31, 64, 101, 4095])
@pytest.mark.parametrize("cutoff,pass_zero", _FIRWIN_BANDS)
def test_firwin_matches_scipy(numtaps, cutoff, pass_zero):
    import warnings
    for window in _WINDOWS:
        for scale in (True, False):
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                try:
                    ref = ss.firwin(numtaps, cutoff, window=window, pass_zero=pass_zero, scale=scale)
                except ValueError:
                    ref = None
            if ref is None or not np.isfinite(ref).all():
                # SciPy refuses (a Nyquist band with even taps) or divides by
                # a zero response; the library refuses both
                with pytest.raises(sg.GpuError):
                    sg.firwin(numtaps, cutoff, window=window, pass_zero=pass_zero, scale=scale)
                continue
            got = sg.firwin(numtaps, cutoff, window=window, pass_zero=pass_zero, scale=scale)
            np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max(),
                                       err_msg=f"{window} scale={scale}")


def test_firwin_benchmark_designs():
    # the designs of the short-tap, long-tap and resample configurations
    np.testing.assert_allclose(sg.firwin(63, 0.2, window="hamming"),
                               ss.firwin(63, 0.2, window="hamming"), rtol=0, atol=1e-16)
    np.testing.assert_allclose(
        sg.firwin(4095, [0.1, 0.3], window=("kaiser", 8.6), pass_zero=False),
        ss.firwin(4095, [0.1, 0.3], window=("kaiser", 8.6), pass_zero=False), rtol=0, atol=1e-15)
    np.testing.assert_allclose(sg.firwin(3201, 1.0 / 160, window=("kaiser", 5.0)) * 160,
                               sg.resample_poly_default_taps(160, 147), rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(
        sg.firwin(101, [100.0, 300.0], window="blackman", pass_zero="bandpass", fs=2000.0),
        ss.firwin(101, [100.0, 300.0], window="blackman", pass_zero="bandpass", fs=2000.0),
        rtol=0, atol=1e-15)


@pytest.mark.parametrize("call", [
    lambda: sg.firwin(0, 0.2),                         # no taps
    lambda: sg.firwin(31, 1.0),                        # at Nyquist
    lambda: sg.firwin(31, [0.3, 0.2], pass_zero=False),  # decreasing
    lambda: sg.firwin(32, 0.2, pass_zero=False),       # high-pass with even taps
    lambda: sg.firwin(31, 0.2, window="tukey"),        # window not offered
])
def test_firwin_errors(call):
    with pytest.raises(sg.GpuError):
        call()
