"""Tensor-core channelizer for 1024 channels (tc_split: FP32 branch sums, then the DFT factored
32 x 32 on tcgen05) through the C ABI, against the float64 oracle: normwise relative error
<= 2e-6 (CHAN_TC_NORMWISE), the workload's accuracy target, on ragged lengths, filters from one
tap to more than 32 per branch, the wideband workload's signal, a tone, silence, and its input
formats."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import rfx
from oracle import rf_oracle as orc
from rfx import signals

pytestmark = pytest.mark.gpu

CHAN_TC_NORMWISE = 2e-6
M = 1024
DEV = torch.device("cuda:0")


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def run(x: np.ndarray, h: np.ndarray) -> np.ndarray:
    z = rfx.channelize(dev(x), dev(h), M, impl="tc_split")
    torch.cuda.synchronize()
    return z.cpu().numpy()


def bits(t: torch.Tensor) -> np.ndarray:
    return t.cpu().numpy().view(np.uint32)


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


@pytest.mark.parametrize("n,k", [(1024, 32768), (1025, 32768), (5 * 1024 + 3, 32768),
                                 (40 * 1024, 1024), (1 << 16, 1), (70001, 30000),
                                 (1 << 20, 16384), (1 << 20, 2048 + 5), (123457, 32768),
                                 (1 << 22, 32768)])
def test_wide_random_cases(n: int, k: int) -> None:
    rng = np.random.default_rng(n + 3 * k)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    z = run(x, h)
    ref = orc.channelize_fast(x, h, M)
    assert z.shape == ref.shape
    assert orc.normwise_error(z, ref) <= CHAN_TC_NORMWISE


def test_wide_workload_signal() -> None:
    # The wideband workload's generator (16 tones over 60 dB + noise, Kaiser prototype).
    w = signals.channelizer1024(1 << 22)
    z = run(w.x, w.taps)
    ref = orc.channelize_fast(w.x, w.taps, M)
    assert orc.normwise_error(z, ref) <= CHAN_TC_NORMWISE
    assert orc.per_channel_error(z, ref).shape == (M,)


def test_wide_tone_lands_in_its_channel() -> None:
    n = np.arange(M * 256)
    x = signals.to_cf32(np.exp(2j * np.pi * 37 * n / M))
    h = signals.channelizer1024(M).taps
    z = run(x, h)[64:]
    power = np.mean(np.abs(z) ** 2, axis=0)
    assert np.argmax(power) == 37
    assert power[37] > 1000 * np.max(np.delete(power, 37))


def test_wide_zeros_are_exact() -> None:
    z = run(np.zeros(M * 100, np.complex64), signals.channelizer1024(M).taps)
    assert not np.any(z)


def test_wide_magnitude_is_the_modulus_of_its_output() -> None:
    w = signals.channelizer1024(1 << 20)
    x, h = dev(w.x), dev(w.taps)
    z = rfx.channelize(x, h, M, impl="tc_split")
    mag = rfx.channelize_magnitude(x, h, M, impl="tc_split")
    torch.cuda.synchronize()
    assert np.array_equal(bits(mag), bits(rfx.magnitude(z)))


@pytest.mark.parametrize("fmt", ["ci16", "ci8"])
@pytest.mark.parametrize("n", [3000, 1 << 20])
def test_wide_integer_input_matches_the_converted_input(fmt: str, n: int) -> None:
    rng = np.random.default_rng(n)
    lim = 32768 if fmt == "ci16" else 128
    c = rng.integers(-lim, lim, size=2 * n).astype(np.int16 if fmt == "ci16" else np.int8)
    h = signals.channelizer1024(M).taps
    got = rfx.channelize_format(dev(c), dev(h), M, fmt, impl="tc_split")
    want = rfx.channelize(dev(orc.decode(c, fmt)), dev(h), M, impl="tc_split")
    torch.cuda.synchronize()
    assert np.array_equal(bits(got), bits(want))


@pytest.mark.parametrize("k", [32 * M + 1, 40000])
def test_wide_filters_longer_than_32_taps_per_branch(k: int) -> None:
    # The branch sums then come from the two-block kernel; the DFT is the same.
    n = 50000
    rng = np.random.default_rng(k)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    z = run(x, h)
    assert orc.normwise_error(z, orc.channelize_fast(x, h, M)) <= CHAN_TC_NORMWISE


def test_wide_dft_of_the_bit_exact_branch_sums() -> None:
    # The form's branch sums are the plain form's (bit for bit), so its DFT alone is within
    # the bound of the float64 DFT of those float32 sums.
    w = signals.channelizer1024(1 << 20)
    z = run(w.x, w.taps)
    u = orc.channelize_branch_f32_seq(w.x, w.taps, M).astype(np.complex128)
    ref = np.fft.ifft(u, axis=1) * M
    assert orc.normwise_error(z, ref) <= CHAN_TC_NORMWISE


def test_wide_host_path() -> None:
    # rfx_channelize_host (host buffers in and out, the project's channelize_cuda contract).
    w = signals.channelizer1024(1 << 18)
    z, bench = rfx.channelize_host("tc_split", w.x, w.taps, M, warmup=1, runs=2)
    assert orc.normwise_error(z, orc.channelize_fast(w.x, w.taps, M)) <= CHAN_TC_NORMWISE
    assert bench.kernel_ms_mean > 0
