"""Tensor-core channelizer (tc_split, 64 channels) on the GPU through the C ABI, against the
float64 oracle: normwise relative error <= 2e-6 (CHAN_TC_NORMWISE), the workload's accuracy
target, plus the project's channelizer tolerance (rtol 1e-5, atol 1e-4,
tests/test_pipeline.py:363-364) on its 64-channel fixture case."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import rfx
from oracle import rf_oracle as orc
from rfx import signals

pytestmark = pytest.mark.gpu

CHAN_TC_NORMWISE = 2e-6
DEV = torch.device("cuda:0")


def run(x: np.ndarray, h: np.ndarray, m: int = 64) -> np.ndarray:
    z = rfx.channelize(torch.from_numpy(np.ascontiguousarray(x)).to(DEV),
                       torch.from_numpy(np.ascontiguousarray(h)).to(DEV), m, impl="tc_split")
    torch.cuda.synchronize()
    return z.cpu().numpy()


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


def test_tc_fixture_case_tone_lowpass_long() -> None:
    # tests/test_pipeline.py:370: taps (1025) not a multiple of M, 17 taps per branch.
    x, h = signals.fixture_signal("tone"), signals.fixture_taps("lowpass_long")
    z = run(x, h)
    ref = orc.channelize_fast(x, h, 64)
    np.testing.assert_allclose(z, ref, rtol=1e-5, atol=1e-4)
    assert orc.normwise_error(z, ref) <= CHAN_TC_NORMWISE


@pytest.mark.parametrize("n,k", [(64, 1024), (65, 1024), (100, 37), (8192, 1024),
                                 (8192 * 3 + 65, 1024), (70001, 1000), (200000, 64),
                                 (50000, 1), (10007, 2048), (1 << 20, 1024)])
def test_tc_random_cases(n: int, k: int) -> None:
    rng = np.random.default_rng(n + k)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    z = run(x, h)
    ref = orc.channelize_fast(x, h, 64)
    assert z.shape == ref.shape
    assert orc.normwise_error(z, ref) <= CHAN_TC_NORMWISE


def test_tc_pfb64_workload() -> None:
    w = signals.channelizer64(1 << 22)
    z = run(w.x, w.taps)
    ref = orc.channelize_fast(w.x, w.taps, 64)
    assert orc.normwise_error(z, ref) <= CHAN_TC_NORMWISE
    err = orc.per_channel_error(z, ref)
    assert err.shape == (64,)


def test_tc_tone_lands_in_its_channel() -> None:
    n = np.arange(64 * 2048)
    x = signals.to_cf32(np.exp(2j * np.pi * 5 * n / 64))
    h = signals.channelizer64(64).taps
    z = run(x, h)[32:]
    power = np.mean(np.abs(z) ** 2, axis=0)
    assert np.argmax(power) == 5
    assert power[5] > 1000 * np.max(np.delete(power, 5))


def test_tc_zeros_are_exact() -> None:
    z = run(np.zeros(8192 * 2, np.complex64), signals.channelizer64(64).taps)
    assert not np.any(z)


def test_tc_plan_rejects_other_channel_counts() -> None:
    with pytest.raises(rfx.RfxError) as e:
        rfx.ChanPlan(16, 1000, impl="tc_split")
    assert e.value.status == 2


def test_tc_host_path() -> None:
    w = signals.channelizer64(1 << 18)
    z, bench = rfx.channelize_host("tc_split", w.x, w.taps, 64, warmup=1, runs=2)
    assert orc.normwise_error(z, orc.channelize_fast(w.x, w.taps, 64)) <= CHAN_TC_NORMWISE
    assert bench.kernel_ms_mean > 0
