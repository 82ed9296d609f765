"""The channelizer over integer I/Q recordings (SigMF ci16_le, ci8) converted where the kernels
read the samples (rfx_channelize_launch_format).

The project converts such recordings on the host (src/io.cpp:110-148: v / 32768, v / 128, exact
in float32) before channelizing. The tensor-core kernel's TMA windows here carry the stored
components and its branch-sum loads convert them; the plain kernel converts on its global loads.
Both give the converted samples' floats, so every output must be BIT-IDENTICAL to channelizing
the host-converted samples with the same implementation — complex outputs and the fused
magnitude alike.
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
INT = {"ci16": np.dtype("<i2"), "ci8": np.dtype(np.int8)}


def stored(fmt: str, n: int, seed: int) -> np.ndarray:
    info = np.iinfo(INT[fmt])
    rng = np.random.default_rng(seed)
    return rng.integers(info.min, info.max, size=2 * n, endpoint=True).astype(INT[fmt])


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def bits(t) -> np.ndarray:
    return np.ascontiguousarray(t.cpu().numpy()).view(np.uint32)


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


@pytest.mark.parametrize("fmt", ["ci16", "ci8"])
@pytest.mark.parametrize("impl", ["tc_split", "plain"])
@pytest.mark.parametrize("n,k", [(64, 1024), (65, 1024), (10007, 1024), (8192, 16),
                                 (40000, 2048), (300001, 1024), (8193, 129)])
@pytest.mark.parametrize("magnitude", [False, True])
def test_64_channels_match_the_converted_input(fmt: str, impl: str, n: int, k: int,
                                               magnitude: bool) -> None:
    c = stored(fmt, n, seed=n + k)
    h = (np.random.default_rng(k).standard_normal(k) / np.sqrt(k)).astype(np.float32)
    dh = dev(h)
    got = rfx.channelize_format(dev(c), dh, 64, fmt, impl=impl, magnitude=magnitude)
    x = dev(orc.decode(c, fmt))
    want = (rfx.channelize_magnitude(x, dh, 64, impl=impl) if magnitude
            else rfx.channelize(x, dh, 64, impl=impl))
    torch.cuda.synchronize()
    assert got.shape == want.shape
    assert np.array_equal(bits(got), bits(want))


@pytest.mark.parametrize("fmt", ["ci16", "ci8"])
@pytest.mark.parametrize("n,k,m", [(100, 37, 4), (7, 63, 4), (12345, 100, 12), (5000, 333, 100),
                                   (1 << 16, 32768, 1024), (999, 2000, 3),
                                   (1 << 18, 1024, 64), (1 << 20, 32768, 1024)])
def test_plain_branch_sums_of_any_channel_count(fmt: str, n: int, k: int, m: int) -> None:
    c = stored(fmt, n, seed=3 * n + m)
    h = (np.random.default_rng(m).standard_normal(k) / np.sqrt(k)).astype(np.float32)
    dh = dev(h)
    got = rfx.channelize_format(dev(c), dh, m, fmt, impl="plain")
    want = rfx.channelize(dev(orc.decode(c, fmt)), dh, m, impl="plain")
    torch.cuda.synchronize()
    assert np.array_equal(bits(got), bits(want))
    # and against the reference's float32 branch arithmetic, through the FFT-free branch path
    u = rfx.channelize_branches(dev(orc.decode(c, fmt)), dh, m)
    torch.cuda.synchronize()
    assert np.array_equal(bits(u), orc.channelize_branch_f32_seq(orc.decode(c, fmt), h, m)
                          .view(np.uint32))


def test_sigmf_fixture_and_host_entry() -> None:
    c = signals.tone_ci16()
    x = signals.fixture_signal("tone_ci16")
    h = signals.fixture_taps("lowpass_long")
    import ctypes

    f = rfx.frames(x.size, 64)
    out = np.empty(f * 64, dtype=np.complex64)
    b = rfx.Bench(warmup=1, runs=2)
    st = rfx.load().rfx_channelize_host_format(rfx.parse_chan_impl("tc_split"), 1, 0,
                                               c.ctypes.data, x.size, h.ctypes.data, h.size, 64,
                                               out.ctypes.data, ctypes.byref(b))
    assert st == 0, rfx.load().rfx_last_error()
    want = rfx.channelize(dev(x), dev(h), 64, impl="tc_split")
    assert np.array_equal(out.view(np.uint32), bits(want).ravel())
    ref = orc.channelize_fast(x, h, 64)
    assert orc.normwise_error(out.reshape(f, 64), ref) <= 2e-6


def test_bad_format_and_output_are_refused() -> None:
    x = dev(stored("ci16", 1000, 1))
    h = dev(np.ones(64, np.float32))
    out = torch.empty((rfx.frames(1000, 64), 64), dtype=torch.complex64, device=DEV)
    with rfx.ChanPlan(64, 1000, "tc_split") as plan:
        for fmt, output in ((3, 0), (1, 2)):
            st = rfx.load().rfx_channelize_launch_format(plan.handle, fmt, output, x.data_ptr(),
                                                         h.data_ptr(), out.data_ptr(), 1000, 64,
                                                         None)
            assert st == 1
