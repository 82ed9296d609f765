"""Batched FIR with per-capture taps (rfx_fir_batch_launch) on the GPU, against the oracle.

The tensor-core batch runs every capture in one persistent launch; each capture is held to the
tensor-core FIR's bar (normwise error <= 2e-6 vs float64). The plain batch (one launch per
capture, as the project runs a batch) is bit-exact against the float32 restatement. Edge cases:
empty captures, captures shorter than one block, one-tap filters, capture counts beyond one
launch's table, and replay of the launch from a captured CUDA graph.
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
DEV = torch.device("cuda:0")


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


def to_dev(captures):
    out = []
    for x, h in captures:
        xd = torch.from_numpy(np.ascontiguousarray(x)).to(DEV)
        out.append((xd, torch.empty_like(xd), torch.from_numpy(np.ascontiguousarray(h)).to(DEV)))
    return out


def check(captures, dev_caps, exact: bool) -> None:
    torch.cuda.synchronize()
    for (x, h), (_, y, _) in zip(captures, dev_caps):
        got = y.cpu().numpy()
        if exact:
            assert np.array_equal(got.view(np.uint32), orc.fir_f32_seq(x, h).view(np.uint32))
        else:
            assert orc.normwise_error(got, orc.fir_fast(x, h)) <= TC_NORMWISE


def small_batch(count: int, seed: int, log2_max: float = 16.0):
    return signals.batched_fir(count=count, log2_min=8.0, log2_max=log2_max, seed=seed).captures


@pytest.mark.parametrize("impl", ["tc_split", "auto"])
def test_tc_batch_matches_oracle(impl: str) -> None:
    caps = small_batch(40, seed=41)
    dev = to_dev(caps)
    rfx.fir_batch(dev, impl=impl)
    check(caps, dev, exact=False)


def test_plain_batch_is_bit_exact() -> None:
    caps = small_batch(30, seed=42)
    dev = to_dev(caps)
    rfx.fir_batch(dev, impl="plain")
    check(caps, dev, exact=True)


def test_batch_edge_captures() -> None:
    rng = np.random.default_rng(7)
    caps = []
    for n, k in [(0, 63), (5, 31), (127, 1025), (128, 1025), (129, 2), (20000, 1), (16384, 255),
                 (16385, 511), (70000, 1025), (3, 1)]:
        x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
        h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
        caps.append((x, h))
    dev = to_dev(caps)
    rfx.fir_batch(dev, impl="tc_split")
    torch.cuda.synchronize()
    for (x, h), (_, y, _) in zip(caps, dev):
        got = y.cpu().numpy()
        if x.size == 0:
            continue
        assert orc.normwise_error(got, orc.fir_fast(x, h)) <= TC_NORMWISE, (x.size, h.size)


def test_more_captures_than_one_launch_holds() -> None:
    caps = small_batch(230, seed=43, log2_max=11.0)
    dev = to_dev(caps)
    rfx.fir_batch(dev, impl="tc_split")
    check(caps, dev, exact=False)


def test_batch_replays_from_a_cuda_graph() -> None:
    caps = small_batch(24, seed=44)
    dev = to_dev(caps)
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        rfx.fir_batch(dev, impl="tc_split", stream=stream)   # warm-up (function attributes)
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream, capture_error_mode="relaxed"):
        rfx.fir_batch(dev, impl="tc_split", stream=stream)
    for _, y, _ in dev:
        y.zero_()
    graph.replay()
    check(caps, dev, exact=False)
    for _, y, _ in dev:
        y.zero_()
    graph.replay()
    check(caps, dev, exact=False)


def test_batch_workload_shape() -> None:
    # The benchmark's batch shape at a reduced length range: 256 captures, six tap counts.
    caps = signals.batched_fir(count=256, log2_min=10.0, log2_max=14.0, seed=45).captures
    dev = to_dev(caps)
    rfx.fir_batch(dev, impl="tc_split")
    check(caps, dev, exact=False)


def test_auto_batch_routes_short_filters_to_the_exact_plain_kernel() -> None:
    # auto: filters under 160 taps run the plain FP32 kernel (one launch for all of them), so
    # their outputs are bit-exact; the longer ones go to the tensor-core launch (2e-6).
    rng = np.random.default_rng(46)
    caps = []
    for n, k in [(70000, 31), (3000, 63), (1 << 17, 127), (200000, 1025), (5, 63), (4096, 2),
                 (1 << 16, 255), (2305, 159), (90001, 160)]:
        x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
        h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
        caps.append((x, h))
    dev = to_dev(caps)
    rfx.fir_batch(dev, impl="auto")
    torch.cuda.synchronize()
    for (x, h), (_, y, _) in zip(caps, dev):
        got = y.cpu().numpy()
        if h.size < 160 or x.size < (1 << 16):
            assert np.array_equal(got.view(np.uint32), orc.fir_f32_seq(x, h).view(np.uint32))
        else:
            assert orc.normwise_error(got, orc.fir_fast(x, h)) <= TC_NORMWISE
