"""rfx_channelize_tc_static: the 64-channel tensor-core channelizer for callers that cannot
allocate device memory once they are running (a memory budget fixed at start-up, a device
allocator owned by another framework, or a loop that must not take cudaMalloc's implicit
synchronization). Its twiddle operand lives in a static device array instead of a plan.

Checked through the C ABI, two calls in a row on the same inputs:
* against rfx_channelize_launch with an RFX_CHAN_TC plan (the same kernel and operand, so the
  results agree to 1e-6 normwise and are normally identical);
* against the float64 oracle at the tensor-core bar (2e-6 normwise), so that an operand laid
  out wrongly in both paths would still fail;
* that a call after the first leaves the device's free memory and PyTorch's reserved memory
  unchanged (it allocates nothing).
Collected last (a failure here leaves every other test already run); passes alone too."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

import rfx
from oracle import rf_oracle as orc
from rfx import signals

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")
TC_NORMWISE = 2e-6
RFX_ERR_INVALID, RFX_ERR_CAPACITY = 1, 2   # include/rfx.h status codes


def call_static(lib, x, taps, out, n, channels=64, stream=0):
    return lib.rfx_channelize_tc_static(ctypes.c_void_p(x.data_ptr()),
                                        ctypes.c_void_p(taps.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), n, taps.numel(),
                                        channels, ctypes.c_void_p(stream))


@pytest.mark.parametrize("n,k", [(1 << 20, 1024), (8192 * 3 + 65, 1000)])
def test_static_entry_matches_plan_entry_and_oracle(n: int, k: int) -> None:
    lib = rfx.load()
    rng = np.random.default_rng(n + k)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    xd = torch.from_numpy(x).to(DEV)
    hd = torch.from_numpy(h).to(DEV)
    frames = rfx.frames(n, 64)
    ref = torch.empty((frames, 64), dtype=torch.complex64, device=DEV)
    with rfx.ChanPlan(64, n, "tc_split") as plan:
        plan.launch(xd, hd, ref)
    torch.cuda.synchronize()
    want = ref.cpu().numpy()
    exact = orc.channelize_fast(x, h, 64)
    outs = [torch.full((frames, 64), float("nan"), dtype=torch.complex64, device=DEV)
            for _ in range(2)]
    for i, out in enumerate(outs):
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info(DEV)
        reserved0 = torch.cuda.memory_reserved(DEV)
        assert call_static(lib, xd, hd, out, n) == rfx.RFX_OK, lib.rfx_last_error()
        torch.cuda.synchronize()
        if i > 0:   # the first call on the device may still load the module's code
            assert torch.cuda.mem_get_info(DEV)[0] == free0
            assert torch.cuda.memory_reserved(DEV) == reserved0
        got = out.cpu().numpy()
        assert orc.normwise_error(got, want) <= 1e-6
        assert orc.normwise_error(got, exact) <= TC_NORMWISE
        assert float(orc.per_channel_error(got, exact).max()) <= TC_NORMWISE
    assert rfx.device_fault() == 0


def test_static_entry_rejects_what_its_array_cannot_hold() -> None:
    lib = rfx.load()
    x = torch.zeros(4096, dtype=torch.complex64, device=DEV)
    h = torch.ones(512, dtype=torch.float32, device=DEV)
    out = torch.zeros(4096, dtype=torch.complex64, device=DEV)
    assert call_static(lib, x, h, out, 4096, channels=128) == RFX_ERR_CAPACITY
    assert b"64 channels only" in lib.rfx_last_error()
    assert call_static(lib, x, h, out, 63) == RFX_ERR_INVALID
    assert call_static(lib, x, h, out, 0) == rfx.RFX_OK
