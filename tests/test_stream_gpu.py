"""rfx_fir_stream (the chunked host-buffer FIR, the project's `rfgpu stream` path) against one
rfx_fir_launch over the whole capture: bit-identical, for every implementation, chunk size,
ring depth and memory mode — the project's own requirement for its stream
(tests/test_pipeline.py:311-329). Chunk sizes cover: shorter than the 1025-tap filter's history,
dividing the input, one chunk for everything, the tensor-core tile (12288 outputs) and sizes
that cut tiles."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import rfx
from rfx import signals

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")


def whole_run(x: np.ndarray, h: np.ndarray, impl: str) -> np.ndarray:
    y = rfx.fir(torch.from_numpy(x).to(DEV), torch.from_numpy(h).to(DEV), impl=impl)
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("impl", ["plain", "tc_split", "auto"])
@pytest.mark.parametrize("chunk,depth", [(1000, 1), (1000, 3), (4096, 2), (100000, 3),
                                         (12288, 2), (30000, 4)])
@pytest.mark.parametrize("memory", ["copy", "registered", "zero-copy"])
def test_stream_matches_whole_run_exactly(impl: str, chunk: int, depth: int, memory: str) -> None:
    x = signals.fixture_signal("tone")
    h = signals.fixture_taps("lowpass_long")
    want = whole_run(x, h, impl)
    got, total_ms, chunks = rfx.fir_stream(x, h, impl=impl, chunk=chunk, depth=depth,
                                           memory=memory)
    assert chunks == -(-x.size // chunk)
    assert total_ms > 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("memory", ["copy", "registered"])
def test_stream_of_a_long_capture_in_pinned_memory(memory: str) -> None:
    rng = np.random.default_rng(5)
    n, k = 300001, 255
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    xp = torch.from_numpy(x).pin_memory()
    yp = torch.empty_like(xp).pin_memory()
    for impl in ["tc_split", "plain"]:
        rfx.fir_stream(xp, h, impl=impl, chunk=50000, depth=3, memory=memory, out=yp)
        assert np.array_equal(yp.numpy().view(np.uint32), whole_run(x, h, impl).view(np.uint32))
    assert rfx.device_fault() == 0


def test_stream_of_input_shorter_than_a_chunk() -> None:
    x = signals.fixture_signal("short")
    h = signals.fixture_taps("lowpass")
    got, _, chunks = rfx.fir_stream(x, h, impl="plain", chunk=3, depth=2)
    assert chunks == -(-x.size // 3)
    assert np.array_equal(got.view(np.uint32), whole_run(x, h, "plain").view(np.uint32))


def test_bad_stream_arguments_are_errors() -> None:
    x = signals.fixture_signal("short")
    h = signals.fixture_taps("lowpass")
    for kwargs in [{"chunk": 0}, {"depth": 0}]:
        with pytest.raises(rfx.RfxError) as e:
            rfx.fir_stream(x, h, **kwargs)
        assert e.value.status == 1
