"""Magnitude and the fused channelize |> magnitude, on the GPU through the C ABI.

The project's magnitude (src/magnitude.cu:17-25) is |x| = sqrt(re^2 + im^2) per sample, tested
against tools/reference.py at rtol = atol = 1e-6 (tests/test_pipeline.py:88-110); zeros give
exactly zero. The fused form takes the magnitude of the channelizer's outputs in the
tensor-core kernel's epilogue, from the same floats the complex output would hold, with the
same rounding steps as the standalone kernel: its bits must equal magnitude(channelize(x)).
The plain form runs the two kernels back to back: the same bits by construction.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import rfx
from oracle import rf_oracle as orc
from rfx import signals

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")
MAGNITUDE_RTOL = 1e-6
MAGNITUDE_ATOL = 1e-6
CHANNELIZE_RTOL = 1e-5   # tests/test_pipeline.py:363-364
CHANNELIZE_ATOL = 1e-4
TC_NORMWISE = 2e-6


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def bits(a) -> np.ndarray:
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else a
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


@pytest.mark.parametrize("name", ["tone", "tone_odd", "short", "tone_ci16"])
def test_magnitude_matches_reference(name: str) -> None:
    x = signals.fixture_signal(name)
    mag = rfx.magnitude(dev(x)).cpu().numpy()
    np.testing.assert_allclose(mag, orc.magnitude(x), rtol=MAGNITUDE_RTOL, atol=MAGNITUDE_ATOL)


@pytest.mark.parametrize("n", [1, 2, 3, 255, 256, 257, 100003, (1 << 22) + 1])
def test_magnitude_sizes_and_extremes(n: int) -> None:
    rng = np.random.default_rng(n)
    x = signals.to_cf32(rng.standard_normal(n) * 1e3 + 1j * rng.standard_normal(n) * 1e-3)
    x[0] = 0
    if n > 2:
        x[1] = np.complex64(3e38 + 0j)           # near the float32 limit: no overflow in re^2?
        x[2] = np.complex64(1e-30 + 1e-30j)      # tiny: squares underflow to subnormal/zero
    mag = rfx.magnitude(dev(x)).cpu().numpy()
    ref = orc.magnitude(x)
    finite = np.isfinite(mag)
    # re^2 overflows float32 for |re| > 1.8e19, as in the project's kernel: inf there.
    big = np.abs(x.real.astype(np.float64)) > 1.8e19
    assert np.all(np.isinf(mag[big])) and np.all(finite[~big])
    np.testing.assert_allclose(mag[~big & (ref > 1e-18)], ref[~big & (ref > 1e-18)],
                               rtol=MAGNITUDE_RTOL, atol=0)
    assert mag[0] == 0.0


def test_magnitude_of_zeros_is_exactly_zero() -> None:
    mag = rfx.magnitude(dev(signals.fixture_signal("zeros"))).cpu().numpy()
    assert not np.any(mag)


def test_magnitude_host_entry() -> None:
    x = signals.fixture_signal("tone_odd")
    mag, b = rfx.magnitude_host(x, warmup=1, runs=3)
    assert np.array_equal(bits(mag), bits(rfx.magnitude(dev(x))))
    assert b.kernel_ms_mean > 0


@pytest.mark.parametrize("impl", ["tc_split", "plain"])
@pytest.mark.parametrize("n,k", [(64, 1024), (65, 1024), (10007, 1024), (8192, 16),
                                 (8193, 129), (300000, 1024), (40000, 2048)])
def test_fused_magnitude_is_magnitude_of_channelize(impl: str, n: int, k: int) -> None:
    rng = np.random.default_rng(n + k)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    dx, dh = dev(x), dev(h)
    z = rfx.channelize(dx, dh, 64, impl=impl)
    unfused = rfx.magnitude(z)
    fused = rfx.channelize_magnitude(dx, dh, 64, impl=impl)
    torch.cuda.synchronize()
    assert fused.shape == (rfx.frames(n, 64), 64)
    assert np.array_equal(bits(fused), bits(unfused))
    ref = orc.magnitude(orc.channelize_fast(x, h, 64, threads=8))
    got = fused.cpu().numpy()
    if impl == "plain":
        np.testing.assert_allclose(got, ref, rtol=CHANNELIZE_RTOL, atol=CHANNELIZE_ATOL)
    else:
        assert np.max(np.abs(got - ref)) <= TC_NORMWISE * np.max(np.abs(ref))


@pytest.mark.parametrize("channels", [1, 4, 16, 1024])
def test_plain_fused_magnitude_any_channel_count(channels: int) -> None:
    x = signals.fixture_signal("tone")
    h = signals.fixture_taps("channelizer_proto")
    dx, dh = dev(x), dev(h)
    fused = rfx.channelize_magnitude(dx, dh, channels, impl="plain")
    unfused = rfx.magnitude(rfx.channelize(dx, dh, channels, impl="plain"))
    torch.cuda.synchronize()
    assert np.array_equal(bits(fused), bits(unfused))


def test_fused_magnitude_host_entry_and_plan_reuse() -> None:
    w = signals.channelizer64(1 << 18)
    mag, b = rfx.channelize_magnitude_host("tc_split", w.x, w.taps, 64, warmup=1, runs=2)
    dx, dh = dev(w.x), dev(w.taps)
    assert np.array_equal(bits(mag), bits(rfx.channelize_magnitude(dx, dh, 64, "tc_split")))
    # One plain plan: the first magnitude call allocates its scratch; complex calls still work.
    with rfx.ChanPlan(64, w.x.size, "plain") as plan:
        out_m = torch.empty((rfx.frames(w.x.size, 64), 64), dtype=torch.float32, device=DEV)
        out_z = torch.empty((rfx.frames(w.x.size, 64), 64), dtype=torch.complex64, device=DEV)
        for _ in range(2):
            plan.launch_magnitude(dx, dh, out_m)
            plan.launch(dx, dh, out_z)
        torch.cuda.synchronize()
        assert np.array_equal(bits(out_m), bits(rfx.magnitude(out_z)))
    assert b.kernel_ms_mean > 0
