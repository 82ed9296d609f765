"""Channelizer on the GPU through the C ABI, against the oracle.

Mirrors the project's channelizer tests (tests/test_pipeline.py:360-405): its five fixture cases
at rtol 1e-5 / atol 1e-4, the channel-3 tone, and a bad channel count; plus the channel counts
the benchmark workloads use (64 and 1024) and ragged lengths.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import rfx
from oracle import rf_oracle as orc
from rfx import signals

pytestmark = pytest.mark.gpu

CHANNELIZE_RTOL = 1e-5
CHANNELIZE_ATOL = 1e-4
DEV = torch.device("cuda:0")


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def run(x: np.ndarray, h: np.ndarray, m: int, impl="plain") -> np.ndarray:
    z = rfx.channelize(dev(x), dev(h), m, impl=impl)
    torch.cuda.synchronize()
    return z.cpu().numpy()


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


@pytest.mark.parametrize("name,taps,channels", [
    ("tone", "channelizer_proto", 16),
    ("tone_odd", "channelizer_proto", 16),   # partial last frame
    ("tone", "lowpass_long", 64),            # taps not a multiple of M
    ("short", "lowpass", 4),                 # input shorter than the filter
    ("tone_odd", "identity", 1),             # one channel, one tap: the input itself
])
def test_channelize_matches_reference(name: str, taps: str, channels: int) -> None:
    x, h = signals.fixture_signal(name), signals.fixture_taps(taps)
    z = run(x, h, channels)
    ref = orc.channelize_fast(x, h, channels)
    assert z.shape == ref.shape
    np.testing.assert_allclose(z, ref, rtol=CHANNELIZE_RTOL, atol=CHANNELIZE_ATOL)


def test_channelize_puts_a_tone_in_its_channel() -> None:
    n = np.arange(16 * 512)
    x = signals.to_cf32(np.exp(2j * np.pi * 3 * n / 16))
    z = run(x, signals.fixture_taps("channelizer_proto"), 16)[16:]
    power = np.mean(np.abs(z) ** 2, axis=0)
    assert np.argmax(power) == 3
    assert power[3] > 1000 * np.max(np.delete(power, 3))
    np.testing.assert_allclose(np.abs(z[:, 3]), 1.0, atol=0.02)


@pytest.mark.parametrize("n,k,m", [(100, 37, 4), (64, 16, 16), (7, 63, 4), (33, 1, 1),
                                   (50, 24, 8), (70001, 1024, 64), (1 << 16, 4096, 1024),
                                   (5 * 1024 + 3, 32768, 1024), (12345, 100, 12)])
def test_channelize_random_cases(n: int, k: int, m: int) -> None:
    rng = np.random.default_rng(n + k + m)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    z = run(x, h, m)
    ref = orc.channelize_fast(x, h, m)
    assert orc.normwise_error(z, ref) < 1e-5


def test_pfb64_workload_prefix() -> None:
    w = signals.channelizer64(1 << 20)
    z = run(w.x, w.taps, 64)
    assert orc.normwise_error(z, orc.channelize_fast(w.x, w.taps, 64)) < 1e-5


def test_host_buffer_path() -> None:
    x, h = signals.fixture_signal("tone"), signals.fixture_taps("channelizer_proto")
    z, bench = rfx.channelize_host("plain", x, h, 16, warmup=1, runs=3)
    np.testing.assert_allclose(z, orc.channelize_fast(x, h, 16), rtol=CHANNELIZE_RTOL,
                               atol=CHANNELIZE_ATOL)
    assert bench.kernel_ms_mean > 0


def test_plan_frame_count_is_checked() -> None:
    x = dev(signals.fixture_signal("tone_odd"))
    h = dev(signals.fixture_taps("channelizer_proto"))
    out = torch.empty(1024 * 16, dtype=torch.complex64, device=DEV)
    with rfx.ChanPlan(16, 4096) as plan:
        with pytest.raises(rfx.RfxError) as e:
            plan.launch(x, h, out)
        assert e.value.status == 1


def test_bad_channel_count_is_an_error() -> None:
    with pytest.raises(rfx.RfxError):
        rfx.ChanPlan(0, 100)


@pytest.mark.parametrize("n,k,m", [(100, 37, 4), (64, 16, 16), (7, 63, 4), (33, 1, 1),
                                   (50, 24, 8), (70001, 1024, 64), (1 << 16, 4096, 1024),
                                   (5 * 1024 + 3, 32768, 1024), (12345, 100, 12),
                                   (3000, 640, 160), (1 << 18, 1024, 64), (999, 2000, 3),
                                   # the shared-memory form (64 channels and up): partial branch
                                   # blocks, partial frame blocks, inputs shorter than the taps,
                                   # taps not a multiple of the channels, one tap per branch
                                   (5000, 333, 100), (20011, 6400, 200), (130, 4096, 64),
                                   (64 * 65 + 1, 64 * 40 + 7, 64), (70000, 128, 128),
                                   (4097, 65, 65), (1 << 16, 32768, 1024), (200, 64, 64),
                                   # the register-ring form (8, 16, 24 or 32 taps in every
                                   # branch): many segments per branch at each ring depth,
                                   # several segments per block (fewer than 128 channels),
                                   # partial branch blocks, partial last steps, inputs within
                                   # the tested first steps
                                   (1 << 20, 24 * 64, 64), (300007, 8 * 48, 48),
                                   (1 << 21, 1600, 100), (1 << 22, 32768, 1024),
                                   (1 << 20, 32 * 256, 256), (777777, 24 * 33, 33),
                                   (130, 8 * 16, 16), (5003, 16 * 64, 64),
                                   # tap counts just off the ring form take the other kernel
                                   (1 << 20, 16 * 256 - 3, 256), (777777, 20 * 33, 33)])
def test_branch_sums_are_bit_exact(n: int, k: int, m: int) -> None:
    # rfx_channelize_branches against the reference's float32 branch arithmetic, bit for bit.
    rng = np.random.default_rng(7 * n + k + m)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    u = rfx.channelize_branches(dev(x), dev(h), m)
    torch.cuda.synchronize()
    want = orc.channelize_branch_f32_seq(x, h, m)
    assert np.array_equal(u.cpu().numpy().view(np.uint32), want.view(np.uint32))


# Long ragged inputs for the register-ring branch kernel's shapes (8, 16 and 32 taps per
# branch): the channels within the project's tolerance, the branch sums bit for bit.
@pytest.mark.parametrize("m,p", [(64, 16), (1024, 32), (256, 8)])
def test_plain_long_ragged_input_matches_oracle(m: int, p: int) -> None:
    n = (1 << 21) * 2 + (1 << 20) + 3 * m + 5      # ends in a partial frame
    rng = np.random.default_rng(m)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(m * p) / np.sqrt(m * p)).astype(np.float32)
    z = run(x, h, m)
    np.testing.assert_allclose(z, orc.channelize_fast(x, h, m), rtol=CHANNELIZE_RTOL,
                               atol=CHANNELIZE_ATOL)
    u = rfx.channelize_branches(dev(x), dev(h), m)
    torch.cuda.synchronize()
    want = orc.channelize_branch_f32_seq(x, h, m)
    assert np.array_equal(u.cpu().numpy().reshape(-1).view(np.uint32),
                          want.reshape(-1).view(np.uint32))


def test_plain_long_input_magnitude_and_ci16() -> None:
    m, p = 64, 16
    n = (1 << 21) * 3 + 1000
    rng = np.random.default_rng(9)
    comps = rng.integers(-32768, 32767, size=2 * n, dtype=np.int16)
    h = (rng.standard_normal(m * p) / np.sqrt(m * p)).astype(np.float32)
    x = orc.decode(comps, "ci16")
    ref = orc.channelize_fast(x, h, m)
    z = rfx.channelize_format(dev(comps), dev(h), m, "ci16", impl="plain")
    mag = rfx.channelize_format(dev(comps), dev(h), m, "ci16", impl="plain", magnitude=True)
    zm = rfx.channelize_magnitude(dev(x), dev(h), m, impl="plain")
    torch.cuda.synchronize()
    np.testing.assert_allclose(z.cpu().numpy(), ref, rtol=CHANNELIZE_RTOL, atol=CHANNELIZE_ATOL)
    np.testing.assert_allclose(mag.cpu().numpy(), np.abs(ref), rtol=CHANNELIZE_RTOL,
                               atol=CHANNELIZE_ATOL)
    np.testing.assert_allclose(zm.cpu().numpy(), np.abs(ref), rtol=CHANNELIZE_RTOL,
                               atol=CHANNELIZE_ATOL)
