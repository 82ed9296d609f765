"""FIR of integer I/Q input (SigMF ci16_le, ci8) converted in the kernels' load stage.

The project reads such recordings by converting every component on the host (ci16: v / 32768,
ci8: v / 128; src/io.cpp:110-148) and then filtering the cf32 samples. rfx_fir_launch_format
uploads the stored components and converts them on the device instead. Both conversions are
exact in float32, so the results must be BIT-IDENTICAL to rfx_fir_launch over the converted
samples for every implementation: checked here over sizes around every tile and block boundary
and tap counts around every unroll and chunk boundary, and against the oracle (plain: its
float32 restatement bit for bit; tensor core: the 2e-6 normwise bound against float64).
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import rfx
from oracle import rf_oracle as orc

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")
TC_NORMWISE = 2e-6
COMPONENT = {"ci16": np.dtype("<i2"), "ci8": np.dtype(np.int8)}


def stored(fmt: str, n: int, seed: int) -> np.ndarray:
    """2 n random components over the format's whole range (its most negative value too)."""
    info = np.iinfo(COMPONENT[fmt])
    rng = np.random.default_rng(seed)
    c = rng.integers(info.min, info.max, size=2 * n, endpoint=True).astype(COMPONENT[fmt])
    if n > 0:
        c[0] = info.min
        c[-1] = info.max
    return c


def taps_of(k: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a).view(np.uint32)


def both(fmt: str, c: np.ndarray, h: np.ndarray, impl: str) -> tuple[np.ndarray, np.ndarray]:
    """(FIR converted on the device, FIR of the samples converted on the host) by `impl`."""
    dh = dev(h)
    y_fmt = rfx.fir_format(dev(c), dh, fmt, impl=impl)
    y_ref = rfx.fir(dev(orc.decode(c, fmt)), dh, impl=impl)
    torch.cuda.synchronize()
    return y_fmt.cpu().numpy(), y_ref.cpu().numpy()


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


@pytest.mark.parametrize("fmt", ["ci16", "ci8"])
@pytest.mark.parametrize("n", [1, 5, 127, 128, 129, 2303, 2304, 2305, 4611, 20000])
@pytest.mark.parametrize("k", [1, 2, 9, 63, 64, 65, 1025])
def test_plain_is_bit_exact(fmt: str, n: int, k: int) -> None:
    c = stored(fmt, n, seed=n + 7 * k)
    h = taps_of(k, seed=k)
    y, y_ref = both(fmt, c, h, "plain")
    assert np.array_equal(bits(y), bits(y_ref))
    assert np.array_equal(bits(y), bits(orc.fir_f32_seq(orc.decode(c, fmt), h, threads=8)))


@pytest.mark.parametrize("fmt", ["ci16", "ci8"])
@pytest.mark.parametrize("n", [100, 128, 129, 12287, 12288, 12289, 40000, 100003])
@pytest.mark.parametrize("k", [2, 63, 129, 1025, 2049])
def test_tensor_core_matches_cf32_bits(fmt: str, n: int, k: int) -> None:
    c = stored(fmt, n, seed=3 * n + k)
    h = taps_of(k, seed=k + 1)
    y, y_ref = both(fmt, c, h, "tc_split")
    # The cf32 run takes the single-CTA form too (the built-in tuning), so the bits agree.
    assert np.array_equal(bits(y), bits(y_ref))
    assert orc.normwise_error(y, orc.fir_fast(orc.decode(c, fmt), h, threads=8)) <= TC_NORMWISE


@pytest.mark.parametrize("fmt", ["ci16", "ci8"])
@pytest.mark.parametrize("impl", ["plain", "tc_split", "auto"])
def test_long_capture_matches_cf32_bits(fmt: str, impl: str) -> None:
    # Full-size property: 4 Mi samples, 1025 taps, identical bits to the cf32 path.
    n = (1 << 22) + 77
    c = stored(fmt, n, seed=11)
    h = taps_of(1025, seed=12)
    y, y_ref = both(fmt, c, h, impl)
    assert np.array_equal(bits(y), bits(y_ref))
    assert np.isfinite(y).all() and np.abs(y).max() > 0


def test_sigmf_fixture_through_every_impl() -> None:
    from rfx import signals

    c = signals.tone_ci16()
    x = signals.fixture_signal("tone_ci16")
    for taps in ["lowpass", "lowpass_long", "identity"]:
        h = signals.fixture_taps(taps)
        ref = orc.fir(x.astype(np.complex128), h.astype(np.float64))
        for impl in ["plain", "tc_split", "auto"]:
            y, y_ref = both("ci16", c, h, impl)
            assert np.array_equal(bits(y), bits(y_ref)), (taps, impl)
            np.testing.assert_allclose(y, ref, rtol=1e-5, atol=1e-5)
    # Identity taps return the converted samples exactly.
    y, _ = both("ci16", c, signals.fixture_taps("identity"), "plain")
    assert np.array_equal(bits(y), bits(x))


def test_misaligned_input_is_refused_before_launch() -> None:
    c = dev(stored("ci16", 1000, seed=1))
    h = dev(taps_of(7, seed=2))
    y = torch.empty(998, dtype=torch.complex64, device=DEV)
    with pytest.raises(rfx.RfxError) as err:
        rfx.fir_launch_format("plain", "ci16", c[2:], h, y, num_samples=998)
    assert err.value.status == 3


def test_host_format_entry_uploads_the_stored_bytes() -> None:
    import ctypes

    c = stored("ci8", 50000, seed=5)
    h = taps_of(63, seed=6)
    y = np.empty(50000, dtype=np.complex64)
    b = rfx.Bench(warmup=1, runs=3)
    status = rfx.load().rfx_fir_host_format(rfx.parse_fir_impl("auto"), 2, c.ctypes.data,
                                            50000, h.ctypes.data, 63, 256, y.ctypes.data,
                                            ctypes.byref(b))
    assert status == 0, rfx.load().rfx_last_error()
    y_ref, _ = rfx.fir_host("auto", orc.decode(c, "ci8"), h)
    assert np.array_equal(bits(y), bits(y_ref))
    assert b.h2d_ms_mean > 0 and b.kernel_ms_mean > 0
