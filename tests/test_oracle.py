"""The oracle itself, on the CPU: pinned to the project's tools/reference.py through the golden
vectors, to its fixture files through their SHA-256, and to brute-force definitions, the way the
project checks its own reference (tests/test_reference.py)."""
from __future__ import annotations

import hashlib
import importlib.util
import json

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import rf_oracle as orc
from rfx import signals

_spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
make_golden = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(make_golden)

# float64 against float64: rounding-order differences only (the project uses 1e-9).
RTOL = 1e-9
ATOL = 1e-9


def random_complex(seed: int, n: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


# --- inputs: the fixture files are reproduced byte for byte --------------------------------

SHAS = json.loads((GOLDEN / "fixture_sha256.json").read_text())


@pytest.mark.parametrize("name", ["tone", "tone_odd", "short", "zeros"])
def test_fixture_signal_bytes_match_the_project(name: str) -> None:
    x = signals.fixture_signal(name)
    assert hashlib.sha256(x.astype("<c8").tobytes()).hexdigest() == SHAS[f"{name}.cf32"]


@pytest.mark.parametrize("name", ["lowpass", "lowpass_long", "channelizer_proto", "identity"])
def test_fixture_taps_bytes_match_the_project(name: str) -> None:
    h = signals.fixture_taps(name)
    assert hashlib.sha256(h.astype("<f4").tobytes()).hexdigest() == SHAS[f"{name}.f32"]


def test_sigmf_fixture_bytes_match_the_project() -> None:
    iq = signals.tone_ci16()
    assert iq.dtype == np.dtype("<i2") and iq.size == 2 * 10007
    assert hashlib.sha256(iq.tobytes()).hexdigest() == SHAS["tone_ci16.sigmf-data"]
    # Half of full scale: no component clips (tests/test_fixtures.py:85-92).
    assert 0.45 * 32767 < np.max(np.abs(iq)) <= 0.5 * 32767 + 1


def test_decode_converts_as_the_sigmf_reader() -> None:
    # ci16: v / 32768, exact in float32; the extremes included.
    c16 = np.array([-32768, 32767, 0, -1, 1, 12345], dtype="<i2")
    z = orc.decode(c16, "ci16")
    assert z.dtype == np.complex64
    np.testing.assert_array_equal(z.real, c16[0::2].astype(np.float64) / 32768)
    np.testing.assert_array_equal(z.imag, c16[1::2].astype(np.float64) / 32768)
    # ci8: every value, v / 128.
    c8 = np.arange(-128, 128, dtype=np.int8)
    z = orc.decode(c8, "ci8")
    np.testing.assert_array_equal(z.real, c8[0::2].astype(np.float64) / 128)
    np.testing.assert_array_equal(z.imag, c8[1::2].astype(np.float64) / 128)
    # cf32 as is; the SigMF fixture through decode is the fixture signal.
    assert np.array_equal(orc.decode(signals.tone_ci16(), "ci16"),
                          signals.fixture_signal("tone_ci16"))
    with pytest.raises(ValueError):
        orc.decode(c16[:3], "ci16")


# --- golden vectors from tools/reference.py ------------------------------------------------

def case_inputs(case: dict) -> tuple[np.ndarray, np.ndarray]:
    if "signal" in case:
        return (signals.fixture_signal(case["signal"]).astype(np.complex128),
                signals.fixture_taps(case["taps"]).astype(np.float64))
    if "workload" in case:
        make = {"fir1025": signals.long_fir, "pfb64": signals.channelizer64,
                "pfb1024": signals.channelizer1024}[case["workload"]]
        w = make(case["n"])
        return w.x.astype(np.complex128), w.taps.astype(np.float64)
    if case["op"] == "fir":
        x = random_complex(case["x_seed"], case["n"])
        h = np.random.default_rng(case["h_seed"]).standard_normal(case["k"])
    else:
        rng = np.random.default_rng(case["seed"])
        x = rng.standard_normal(case["n"]) + 1j * rng.standard_normal(case["n"])
        h = rng.standard_normal(case["k"])
    return (signals.to_cf32(x).astype(np.complex128),
            h.astype(np.float32).astype(np.float64))


def check_against_golden(golden, name: str, y: np.ndarray) -> None:
    y = np.asarray(y, dtype=np.complex128).ravel()
    assert y.size == golden.cases[name]["size"]
    scale = max(1.0, float(np.max(np.abs(golden.val(name)))))
    np.testing.assert_allclose(y[golden.idx(name)], golden.val(name), rtol=RTOL,
                               atol=ATOL * scale)
    sums = make_golden.checksums(y)
    np.testing.assert_allclose(sums, golden.sums(name), rtol=1e-9,
                               atol=1e-9 * float(np.abs(golden.sums(name)[1])) ** 0.5)


def golden_names(op: str) -> list[str]:
    data = np.load(GOLDEN / "reference_outputs.npz")
    return [c["name"] for c in json.loads(str(data["__cases__"])) if c["op"] == op]


@pytest.mark.parametrize("name", golden_names("fir"))
def test_numpy_fir_matches_golden(golden, name: str) -> None:
    x, h = case_inputs(golden.cases[name])
    check_against_golden(golden, name, orc.fir(x, h))


@pytest.mark.parametrize("name", golden_names("fir"))
def test_c_fir_matches_golden(golden, name: str) -> None:
    x, h = case_inputs(golden.cases[name])
    check_against_golden(golden, name, orc.fir_fast(x, h, threads=4))


@pytest.mark.parametrize("name", golden_names("channelize"))
def test_numpy_channelize_matches_golden(golden, name: str) -> None:
    c = golden.cases[name]
    x, h = case_inputs(c)
    check_against_golden(golden, name, orc.channelize(x, h, c["channels"]))


@pytest.mark.parametrize("name", golden_names("channelize"))
def test_c_channelize_matches_golden(golden, name: str) -> None:
    c = golden.cases[name]
    x, h = case_inputs(c)
    check_against_golden(golden, name, orc.channelize_fast(x, h, c["channels"], threads=4))


# --- brute-force definitions (as tests/test_reference.py:38-44, :198-205) ------------------

def fir_brute(x: np.ndarray, taps: np.ndarray) -> np.ndarray:
    y = np.zeros(len(x), dtype=np.complex128)
    for n in range(len(x)):
        for k in range(len(taps)):
            if n - k >= 0:
                y[n] += taps[k] * x[n - k]
    return y


def channelize_brute(x: np.ndarray, h: np.ndarray, m: int) -> np.ndarray:
    frames = -(-len(x) // m)
    z = np.zeros((frames, m), dtype=np.complex128)
    for t in range(frames):
        for k in range(m):
            z[t, k] = sum(h[l] * x[t * m - l] * np.exp(2j * np.pi * k * l / m)
                          for l in range(len(h)) if t * m - l >= 0)
    return z


@pytest.mark.parametrize("n,k", [(50, 7), (50, 1), (5, 12), (1, 1), (40, 33)])
def test_fir_matches_brute_force(n: int, k: int) -> None:
    x = signals.to_cf32(random_complex(3, n)).astype(np.complex128)
    h = np.random.default_rng(4).standard_normal(k).astype(np.float32).astype(np.float64)
    ref = fir_brute(x, h)
    np.testing.assert_allclose(orc.fir(x, h), ref, rtol=RTOL, atol=ATOL)
    np.testing.assert_allclose(orc.fir_fast(x, h, threads=3), ref, rtol=RTOL, atol=ATOL)


@pytest.mark.parametrize("n,k,m", [(100, 37, 4), (64, 16, 16), (7, 63, 4), (33, 1, 1),
                                   (50, 24, 8), (45, 20, 6)])
def test_channelize_matches_brute_force(n: int, k: int, m: int) -> None:
    rng = np.random.default_rng(n + k + m)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(complex)
    h = rng.standard_normal(k).astype(np.float32).astype(np.float64)
    ref = channelize_brute(x, h, m)
    np.testing.assert_allclose(orc.channelize(x, h, m), ref, atol=1e-10)
    np.testing.assert_allclose(orc.channelize_fast(x, h, m, threads=2), ref, atol=1e-10)


def test_one_channel_channelizer_is_the_fir() -> None:
    x = signals.fixture_signal("tone_odd")
    h = signals.fixture_taps("lowpass")
    np.testing.assert_allclose(orc.channelize_fast(x, h, 1).ravel(), orc.fir_fast(x, h),
                               atol=1e-10)


# --- known answers (tests/test_reference.py:124-154, tests/test_pipeline.py:386-398) -------

@pytest.mark.parametrize("taps_name", ["lowpass", "lowpass_long"])
def test_lowpass_keeps_passband_and_removes_stopband(taps_name: str) -> None:
    y = orc.fir_fast(signals.fixture_signal("tone"), signals.fixture_taps(taps_name))
    mag = np.abs(np.fft.fft(y[2048:3072]))
    np.testing.assert_allclose(mag[40], 1024.0, rtol=0.02, atol=0)
    assert mag[-300 % 1024] < 512.0 / 100.0


def test_identity_and_zeros_are_exact() -> None:
    x = signals.fixture_signal("tone")
    assert np.array_equal(orc.fir_fast(x, signals.fixture_taps("identity")),
                          x.astype(np.complex128))
    assert np.array_equal(orc.fir_f32_seq(x, signals.fixture_taps("identity")), x)
    z = signals.fixture_signal("zeros")
    for name in ["lowpass", "lowpass_long", "identity"]:
        assert not np.any(orc.fir_fast(z, signals.fixture_taps(name)))
        assert not np.any(orc.fir_f32_seq(z, signals.fixture_taps(name)))


def test_channelizer_puts_a_tone_in_its_channel() -> None:
    n = np.arange(16 * 512)
    x = signals.to_cf32(np.exp(2j * np.pi * 3 * n / 16))
    z = orc.channelize_fast(x, signals.fixture_taps("channelizer_proto"), 16)[16:]
    power = np.mean(np.abs(z) ** 2, axis=0)
    assert np.argmax(power) == 3
    assert power[3] > 1000 * np.max(np.delete(power, 3))
    np.testing.assert_allclose(np.abs(z[:, 3]), 1.0, atol=0.02)


# --- the float32 restatements --------------------------------------------------------------

def test_f32_sequential_fir_is_float32_close_and_thread_independent() -> None:
    x = signals.fixture_signal("tone_odd")
    h = signals.fixture_taps("lowpass_long")
    y1 = orc.fir_f32_seq(x, h, threads=1)
    y7 = orc.fir_f32_seq(x, h, threads=7)
    assert np.array_equal(y1.view(np.uint32), y7.view(np.uint32))
    np.testing.assert_allclose(y1, orc.fir_fast(x, h), rtol=1e-5, atol=1e-5)


def test_f32_sequential_fir_uses_fused_multiply_add() -> None:
    # Two taps: y[1] = fma(h1, x0, fma(h0, x1, 0)) with h0 x1 = -(1 + 2^-11) and
    # h1 x0 = (1 + 2^-12)^2 = 1 + 2^-11 + 2^-24. Fused, the 2^-24 survives; a rounded product
    # followed by an add would give exactly 0.
    x = np.array([1.0 + 2.0 ** -12, -(1.0 + 2.0 ** -11)], dtype=np.float32).astype(np.complex64)
    h = np.array([1.0, 1.0 + 2.0 ** -12], dtype=np.float32)
    y = orc.fir_f32_seq(x, h, threads=1)
    assert y[1].real == np.float32(2.0 ** -24)


def test_branch_f32_matches_float64_branches() -> None:
    x = signals.fixture_signal("tone")
    h = signals.fixture_taps("lowpass_long")
    u = orc.channelize_branch_f32_seq(x, h, 64)
    z_from_u = np.fft.ifft(u.astype(np.complex128), axis=1) * 64
    np.testing.assert_allclose(z_from_u, orc.channelize_fast(x, h, 64), rtol=1e-5, atol=1e-4)


def test_normwise_error_definition() -> None:
    ref = np.array([1.0, -4.0, 2.0j])
    y = ref + np.array([0.0, 1e-6, 0.0])
    assert orc.normwise_error(y, ref) == pytest.approx(0.25e-6)
    assert orc.normwise_error(np.zeros(3), np.zeros(3)) == 0.0


def test_convolve_baseline_equals_the_direct_form() -> None:
    # The CPU baseline's method (np.convolve, the project's tools/reference.py fir) gives the
    # oracle's values.
    rng = np.random.default_rng(7)
    x = (rng.standard_normal(3000) + 1j * rng.standard_normal(3000)).astype(np.complex64)
    h = rng.standard_normal(257).astype(np.float32)
    np.testing.assert_allclose(orc.fir_convolve(x, h), orc.fir(x, h), rtol=1e-12, atol=1e-12)
    assert orc.fir_convolve(x[:0], h).size == 0
