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


# --- integer recordings streamed as stored (rfx_fir_stream_format) ----------------------------
# The stored components cross the host link and the kernels convert them; the output must be
# the bits of one whole run over the same recording (itself the bits of filtering the
# host-converted samples, tests/test_fir_format_gpu.py).

def whole_run_format(c: np.ndarray, fmt: str, h: np.ndarray, impl: str) -> np.ndarray:
    y = rfx.fir_format(torch.from_numpy(c).to(DEV), torch.from_numpy(h).to(DEV), fmt, impl=impl)
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("fmt", ["ci16", "ci8"])
@pytest.mark.parametrize("impl", ["plain", "tc_split", "auto"])
@pytest.mark.parametrize("chunk,depth", [(1000, 3), (12288, 2), (30000, 4)])
@pytest.mark.parametrize("memory", ["copy", "registered", "zero-copy"])
def test_integer_stream_matches_whole_run(fmt: str, impl: str, chunk: int, depth: int,
                                          memory: str) -> None:
    rng = np.random.default_rng(chunk + depth)
    info = np.iinfo(np.int16 if fmt == "ci16" else np.int8)
    c = rng.integers(info.min, info.max, size=2 * 65537, endpoint=True).astype(info.dtype)
    h = signals.fixture_taps("lowpass_long")
    want = whole_run_format(c, fmt, h, impl)
    got, _, chunks = rfx.fir_stream(c, h, impl=impl, chunk=chunk, depth=depth, memory=memory,
                                    fmt=fmt)
    assert chunks == -(-65537 // chunk)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_integer_stream_of_the_sigmf_fixture_equals_the_converted_stream() -> None:
    c = signals.tone_ci16()
    x = signals.fixture_signal("tone_ci16")
    h = signals.fixture_taps("lowpass_long")
    for impl in ["plain", "tc_split"]:
        a, _, _ = rfx.fir_stream(c, h, impl=impl, chunk=4096, depth=3, fmt="ci16")
        b, _, _ = rfx.fir_stream(x, h, impl=impl, chunk=4096, depth=3)
        if impl == "plain":
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        else:
            # cf32 may take the tuned tensor-core form, integer input the single-CTA one; with
            # the built-in tuning both are the single-CTA form: the same bits.
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert rfx.device_fault() == 0
