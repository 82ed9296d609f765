"""bench.py's arm plan on CPU: which implementations each workload times (the headline first)
and how many kernel launches a step counts (the JSON line's `gpu_launches`), for every
workload shape, without a GPU."""
from __future__ import annotations

import importlib.util
from pathlib import Path

import numpy as np
import pytest

from rfx.signals import Workload

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def workload(taps: int, channels: int = 0, captures: int = 0) -> Workload:
    x = np.zeros(16, np.complex64)
    h = np.zeros(taps, np.float32)
    return Workload("w", x, h, channels=channels, captures=[(x, h)] * captures)


@pytest.mark.parametrize("w,first", [
    (workload(1025), "tc_split"),                 # long FIR: the tensor-core form leads
    (workload(63), "auto"),                       # short FIR: auto leads
    (workload(1024, channels=64), "tc_split"),    # 64-channel channelizer
    (workload(32768, channels=1024), "auto"),     # 1024 channels: auto (= plain) leads
    (workload(1025, captures=3), "auto"),         # the batch
])
def test_headline_arm(bench, w: Workload, first: str) -> None:
    order = bench.arm_order(w)
    assert order[0] == first
    assert "tc_split" in order and "plain" in order


@pytest.mark.parametrize("channels,impl,launches", [
    (64, "tc_split", 1), (64, "auto", 1), (64, "plain", 2),
    (1024, "tc_split", 2), (1024, "auto", 2), (1024, "plain", 2),
    (16, "auto", 2), (16, "plain", 2),
])
def test_channelizer_launches_per_step(bench, channels: int, impl: str, launches: int) -> None:
    assert bench.chan_launches(channels, impl) == launches


def test_rounds_cover_half_a_second_and_at_least_five(bench) -> None:
    assert bench.rounds_for(1.0) == bench.MIN_ROUNDS
    assert bench.rounds_for(0.0028) == 179          # 20 steps of 0.14 ms
    assert bench.rounds_for(1e-9) == bench.MAX_ROUNDS


@pytest.mark.parametrize("steps", [1, 4, 5, 20])
def test_round_graphs_hold_the_rounds_steps(bench, monkeypatch, steps: int) -> None:
    # A timed round replays one graph holding its `steps` launches; the round starting at step
    # `first` must run steps first .. first + steps - 1, i.e. the buffer sets (i % 2) of those
    # steps. The capture is replaced by a recorder (no GPU): each "graph" remembers the step
    # indices enqueued into it, modulo 2.
    class Graph:
        def __init__(self, enqueue):
            self.steps = []
            enqueue(self)          # the stream argument is the graph itself here

        def replay(self):
            replayed.append(list(self.steps))

    class Arm(bench.RoundGraphs):
        def enqueue_step(self, i, stream):
            stream.steps.append(i % 2)

    replayed = []
    monkeypatch.setattr(bench, "capture_graph", Graph)
    arm = Arm()
    arm.prepare(steps)
    for r in range(4):
        first = r * steps
        arm.run_round(first, steps)
        assert replayed[-1] == [(first + i) % 2 for i in range(steps)], (r, steps)
