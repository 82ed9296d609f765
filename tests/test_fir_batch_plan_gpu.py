"""Batch plans (rfx_fir_batch_plan_create / rfx_fir_batch_run) on the GPU: the whole batch in ONE
persistent launch, whatever its captures — tensor-core captures through the block-Toeplitz
pipelines (2 to 385 taps in the resident-window phase, one phase per number of blocks reached
back, with the tap strip rebuilt per capture; longer filters in the long-filter phase), the rest
(one tap, fewer than 128 samples, more taps than the batch kernel
holds, or everything under plain) through the plain kernel's tile function run by groups of the
same blocks' threads.

Bars: tensor-core captures <= 2e-6 normwise against float64 (the tensor-core FIR's target);
captures on the plain tile function bit-exact against the float32 chain of the project's
kernels. rfx_fir_impl_used(..., batch=True) names the kernel of each capture, and the plan's
own count agrees with it."""
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
        out.append((xd, torch.full_like(xd, float("nan")),
                    torch.from_numpy(np.ascontiguousarray(h)).to(DEV)))
    return out


def check(captures, dev, impl: str) -> dict:
    torch.cuda.synchronize()
    kinds = {"tc_split": 0, "plain": 0}
    for i, ((x, h), (_, y, _)) in enumerate(zip(captures, dev)):
        if x.size == 0:
            continue
        got = y.cpu().numpy()
        kind = rfx.fir_impl_used(impl, h.size, x.size, batch=True)
        kinds[kind] += 1
        if kind == "plain":
            want = orc.fir_f32_seq(x, h)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (i, x.size, h.size)
        else:
            err = orc.normwise_error(got, orc.fir_fast(x, h))
            assert err <= TC_NORMWISE, (i, x.size, h.size, err)
    return kinds


def rand_caps(spec, seed: int):
    rng = np.random.default_rng(seed)
    caps = []
    for n, k in spec:
        x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
        h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
        caps.append((x, h))
    return caps


MIXED = [(0, 63), (5, 31), (127, 1025), (128, 1025), (129, 2), (20000, 1), (16384, 255),
         (16385, 511), (70000, 1025), (3, 1), (70000, 31), (3000, 63), (1 << 17, 127),
         (200000, 1025), (4096, 2), (1 << 16, 255), (2305, 159), (90001, 160), (40000, 3458),
         (30000, 8192)]


@pytest.mark.parametrize("impl", ["auto", "tc_split", "plain"])
def test_plan_runs_every_capture_in_one_launch(impl: str) -> None:
    caps = rand_caps(MIXED, seed=51)
    dev = to_dev(caps)
    with rfx.FirBatchPlan(dev, impl) as plan:
        info = plan.info()
        assert info["launches"] == 1
        plan.run()
        kinds = check(caps, dev, impl)
    assert info["tc_captures"] == kinds["tc_split"]
    assert info["plain_captures"] == kinds["plain"]
    if impl == "plain":
        assert kinds["tc_split"] == 0
    else:
        assert kinds["tc_split"] > 0 and kinds["plain"] > 0


def test_plan_holds_more_captures_than_the_parameter_table() -> None:
    # 300 captures (the kernel-parameter form holds 96 tensor-core captures per launch).
    caps = signals.batched_fir(count=300, log2_min=8.0, log2_max=13.0, seed=52).captures
    dev = to_dev(caps)
    with rfx.FirBatchPlan(dev, "tc_split") as plan:
        assert plan.info()["launches"] == 1
        plan.run()
        check(caps, dev, "tc_split")


@pytest.mark.parametrize("impl", ["auto", "tc_split"])
def test_plan_replays_from_a_cuda_graph(impl: str) -> None:
    caps = signals.batched_fir(count=40, log2_min=10.0, log2_max=17.0, seed=53).captures
    dev = to_dev(caps)
    with rfx.FirBatchPlan(dev, impl) as plan:
        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(stream):
            plan.run(stream)                      # warm-up outside the capture
        stream.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream, capture_error_mode="relaxed"):
            plan.run(stream)
        for _ in range(2):
            for _, y, _ in dev:
                y.fill_(float("nan"))
            graph.replay()
            check(caps, dev, impl)


def test_plan_sees_new_samples_between_runs() -> None:
    caps = rand_caps([(50000, 255), (20000, 63), (1 << 16, 1025)], seed=54)
    dev = to_dev(caps)
    with rfx.FirBatchPlan(dev, "auto") as plan:
        plan.run()
        check(caps, dev, "auto")
        caps2 = rand_caps([(50000, 255), (20000, 63), (1 << 16, 1025)], seed=55)
        for (x2, _), (xd, _, _) in zip(caps2, dev):
            xd.copy_(torch.from_numpy(x2))
        plan.run()
        check([(x2, h) for (x2, _), (_, h) in zip(caps2, caps)], dev, "auto")


def test_plan_of_only_empty_captures_launches_nothing() -> None:
    caps = rand_caps([(0, 63), (0, 1025)], seed=56)
    dev = to_dev(caps)
    with rfx.FirBatchPlan(dev, "auto") as plan:
        assert plan.info() == {"tc_captures": 0, "plain_captures": 0, "launches": 0}
        plan.run()
    torch.cuda.synchronize()


def test_plan_single_long_capture_matches_the_single_capture_kernel() -> None:
    w = signals.long_fir(1 << 20)
    dev = to_dev([(w.x, w.taps)])
    with rfx.FirBatchPlan(dev, "tc_split") as plan:
        plan.run()
    check([(w.x, w.taps)], dev, "tc_split")


@pytest.mark.parametrize("impl", ["plain", "auto"])
def test_plan_plain_tiles_with_tap_counts_changing_between_captures(impl: str) -> None:
    # Plain tiles of consecutive captures share each thread group's two slots: a capture with
    # more taps than the one before lays its taps over where the previous tile's results sat
    # while they were being stored. Tap counts rise and fall from capture to capture, lengths
    # put several tiles of each capture in every group, and the edge tiles of each capture
    # (its first and last) are among them.
    ks = [31, 63, 127, 159, 2, 159, 31, 127, 63, 159, 1, 95]
    spec = [(2304 * 7 + 17 * i + 1, k) for i, k in enumerate(ks)]
    caps = rand_caps(spec, seed=57)
    dev = to_dev(caps)
    with rfx.FirBatchPlan(dev, impl) as plan:
        plan.run()
        kinds = check(caps, dev, impl)
    # auto puts 2 to 385 taps in the plan's resident-window phase, one tap on a plain tile.
    expect = len(ks) if impl == "plain" else sum(1 for k in ks if k < 2)
    assert kinds["plain"] == expect


@pytest.mark.parametrize("span", ["short", "long"])
def test_plan_window_phases_switch_captures_within_blocks(span: str) -> None:
    # Every reach-back of the resident-window phase (C = 1: 2 to 129 taps, 2: 130 to 257,
    # 3: 258 to 385), with captures short enough that each block's range crosses several of
    # them (480 captures of one to three tiles over the blocks): the strip is rebuilt at every
    # switch, into the other of two slots (C = 1) or into the only one once the previous
    # capture's MMAs are done (C = 2, 3). Lengths around tile edges (6144 outputs per tile)
    # and partial last blocks; "long" puts several tiles of each capture in a block.
    ks = [2, 64, 129, 130, 200, 257, 258, 300, 385, 31, 255, 384, 129, 258, 2, 386]
    if span == "short":
        spec = [(6144 * (1 + i % 3) + 37 * (i % 50) + 1, k) for i, k in enumerate(ks * 30)]
    else:
        spec = [(6144 * (20 + 7 * i) - 5 * i, k) for i, k in enumerate(ks)]
    caps = rand_caps(spec, seed=58)
    dev = to_dev(caps)
    with rfx.FirBatchPlan(dev, "auto") as plan:
        assert plan.info()["launches"] == 1
        plan.run()
        kinds = check(caps, dev, "auto")
    assert kinds["plain"] == 0 and kinds["tc_split"] == len(spec)
