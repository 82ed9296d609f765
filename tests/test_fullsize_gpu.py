"""Parity at the five benchmark workloads' full sizes, over the whole output.

Each workload is generated as the bench generates it (rfx.signals, fixed seeds) and run through
the C ABI; the complete output is compared with the oracle:

* fir1025 (2^24 samples, 1025 Kaiser taps, 8 tones over 60 dB + noise): tc_split and auto,
  normwise error <= 2e-6 against float64 over the whole output and within every 2^16-output
  segment (so a wrong stretch far into the capture cannot hide behind the global maximum);
* fir63 (2^24 samples, 63 taps): plain bit-exact against the float32 restatement of the
  project's FIR kernels (one fma per tap in tap order, tests/test_pipeline.py:116-135 holds
  them to 1e-5); tc_split and auto (the resident-window tensor-core form) <= 2e-6 normwise
  over the whole output and every 2^16-output segment;
* pfb64 (2^24 samples, 64 channels, 1024 taps): tc_split <= 2e-6 normwise, and per channel
  (against each channel's own level) within 2.5x of the FP32 cuFFT form; plain: branch sums
  bit-exact against the float32 restatement and the channels within the project's channelizer
  tolerance (rtol 1e-5, atol 1e-4, tests/test_pipeline.py:363-364);
* pfb1024 (2^26 samples, 1024 channels, 32768 taps): the same bars; the per-channel error of
  each form is printed (pytest -s shows it);
* batch256 (256 captures of 2^12 .. 2^22 samples, own taps each), run as one batch plan (one
  launch): every capture completely, auto and tc_split; captures the plan runs on the plain
  tile function are bit-exact.

The oracle is the C restatement (oracle/rf_oracle.c) on every host core.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import rfx
from oracle import rf_oracle as orc
from rfx import signals

pytestmark = pytest.mark.gpu

TC_NORMWISE = 2e-6
CHAN_RTOL = 1e-5
CHAN_ATOL = 1e-4
DEV = torch.device("cuda:0")
SEGMENT = 1 << 16


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


def worst_segment(y: np.ndarray, ref: np.ndarray, seg: int = SEGMENT) -> float:
    """Largest normwise error of any `seg`-sample stretch, each against its own level."""
    n = ref.size // seg * seg
    d = np.abs(y[:n].astype(np.complex128) - ref[:n]).reshape(-1, seg).max(axis=1)
    s = np.abs(ref[:n]).reshape(-1, seg).max(axis=1)
    worst = float(np.max(d / s))
    if n < ref.size:
        worst = max(worst, orc.normwise_error(y[n:], ref[n:]))
    return worst


def fir_on_gpu(w, impl: str) -> np.ndarray:
    xd = torch.from_numpy(w.x).to(DEV)
    hd = torch.from_numpy(w.taps).to(DEV)
    y = rfx.fir(xd, hd, impl=impl)
    torch.cuda.synchronize()
    out = y.cpu().numpy()
    del xd, y
    return out


# --- fir1025 -----------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def fir1025():
    w = signals.long_fir(1 << 24)
    return w, orc.fir_fast(w.x, w.taps)


@pytest.mark.parametrize("impl", ["tc_split", "auto"])
def test_fir1025_full_output(fir1025, impl: str) -> None:
    w, ref = fir1025
    y = fir_on_gpu(w, impl)
    assert y.shape == ref.shape
    assert orc.normwise_error(y, ref) <= TC_NORMWISE
    assert worst_segment(y, ref) <= TC_NORMWISE


# --- fir63 -------------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def fir63():
    w = signals.plain_fir(1 << 24)
    return w, orc.fir_f32_seq(w.x, w.taps)


def test_fir63_full_output_bit_exact(fir63) -> None:
    w, ref32 = fir63
    y = fir_on_gpu(w, "plain")
    assert np.array_equal(y.view(np.uint32), ref32.view(np.uint32))


@pytest.mark.parametrize("impl", ["tc_split", "auto"])
def test_fir63_tensor_core_full_output(fir63, impl: str) -> None:
    w, _ = fir63
    assert rfx.fir_impl_used(impl, w.taps.size, w.x.size) == "tc_split"
    y = fir_on_gpu(w, impl)
    ref = orc.fir_fast(w.x, w.taps)
    assert orc.normwise_error(y, ref) <= TC_NORMWISE
    assert worst_segment(y, ref) <= TC_NORMWISE


# --- channelizers -----------------------------------------------------------------------------

def chan_on_gpu(w, impl: str) -> np.ndarray:
    xd = torch.from_numpy(w.x).to(DEV)
    hd = torch.from_numpy(w.taps).to(DEV)
    z = rfx.channelize(xd, hd, w.channels, impl=impl)
    torch.cuda.synchronize()
    out = z.cpu().numpy()
    del xd, z
    return out


def branches_on_gpu(w) -> np.ndarray:
    xd = torch.from_numpy(w.x).to(DEV)
    hd = torch.from_numpy(w.taps).to(DEV)
    u = rfx.channelize_branches(xd, hd, w.channels)
    torch.cuda.synchronize()
    out = u.cpu().numpy()
    del xd, u
    return out


@pytest.fixture(scope="module")
def pfb64():
    w = signals.channelizer64(1 << 24)
    return w, orc.channelize_fast(w.x, w.taps, w.channels)


@pytest.fixture(scope="module")
def pfb1024():
    w = signals.channelizer1024(1 << 26)
    return w, orc.channelize_fast(w.x, w.taps, w.channels)


def check_channelizer(name: str, w, ref: np.ndarray) -> None:
    """Both forms on the whole output. The tensor-core form meets the workload's bar (2e-6
    normwise); per channel (each against its own level, channels in the stopband included) its
    error is listed and held within 2.5x of the FP32 cuFFT form's, which itself exceeds 2e-6
    in the quietest channels: the FFT's rounding is relative to each frame's level."""
    z_tc = chan_on_gpu(w, "tc_split")
    z_pl = chan_on_gpu(w, "plain")
    assert z_tc.shape == ref.shape and z_pl.shape == ref.shape
    per_tc = orc.per_channel_error(z_tc, ref)
    per_pl = orc.per_channel_error(z_pl, ref)
    print(f"\n{name}: tc_split normwise {orc.normwise_error(z_tc, ref):.3g}, per channel max "
          f"{per_tc.max():.3g} (channel {int(per_tc.argmax())}), median {np.median(per_tc):.3g}; "
          f"plain normwise {orc.normwise_error(z_pl, ref):.3g}, per channel max "
          f"{per_pl.max():.3g} (channel {int(per_pl.argmax())})")
    assert orc.normwise_error(z_tc, ref) <= TC_NORMWISE
    assert float(per_tc.max()) <= max(TC_NORMWISE, 2.5 * float(per_pl.max()))
    np.testing.assert_allclose(z_pl, ref, rtol=CHAN_RTOL, atol=CHAN_ATOL)


def check_branches(w) -> None:
    u = branches_on_gpu(w)
    u32 = orc.channelize_branch_f32_seq(w.x, w.taps, w.channels)
    assert np.array_equal(u.reshape(-1).view(np.uint32), u32.reshape(-1).view(np.uint32))


def test_pfb64_full_output(pfb64) -> None:
    w, ref = pfb64
    check_channelizer("pfb64", w, ref)
    check_branches(w)


def test_pfb1024_full_output(pfb1024) -> None:
    w, ref = pfb1024
    check_channelizer("pfb1024", w, ref)
    check_branches(w)


# --- batch256 ----------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def batch256():
    return signals.batched_fir().captures


@pytest.mark.parametrize("impl", ["auto", "tc_split"])
def test_batch256_every_capture(batch256, impl: str) -> None:
    caps = batch256
    assert len(caps) == 256
    dev = []
    for x, h in caps:
        xd = torch.from_numpy(np.ascontiguousarray(x)).to(DEV)
        dev.append((xd, torch.empty_like(xd), torch.from_numpy(h).to(DEV)))
    with rfx.FirBatchPlan(dev, impl) as plan:   # the whole batch in one launch
        assert plan.info()["launches"] == 1
        plan.run()
        torch.cuda.synchronize()
    worst = 0.0
    for i, ((x, h), (_, yd, _)) in enumerate(zip(caps, dev)):
        y = yd.cpu().numpy()
        used = rfx.fir_impl_used(impl, h.size, x.size, batch=True)
        if used == "plain":
            ref32 = orc.fir_f32_seq(x, h)
            assert np.array_equal(y.view(np.uint32), ref32.view(np.uint32)), i
        else:
            err = orc.normwise_error(y, orc.fir_fast(x, h))
            worst = max(worst, err)
            assert err <= TC_NORMWISE, (i, x.size, h.size, err)
    print(f"\nbatch256 {impl}: worst tensor-core capture error {worst:.3g}")
