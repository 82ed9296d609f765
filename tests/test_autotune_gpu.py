"""The autotuner on the GPU: for the five benchmark workloads' (taps, length, channels) cases,
the pick it stores is never slower than the built-in rule's (within timing noise: 5 % plus
2 us), the tuned `auto` still meets the accuracy bar, and a saved table reloads."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import rfx
from oracle import rf_oracle as orc
from rfx import signals

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")


@pytest.fixture(autouse=True)
def clean_table():
    rfx.load()
    rfx.autotune_clear()
    yield
    rfx.autotune_clear()
    assert rfx.device_fault() == 0


def best_ms(fn, reps: int = 30) -> float:
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def rand(n: int, k: int, seed: int):
    rng = np.random.default_rng(seed)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    return x, h


# fir1025, fir63, and batch256's shortest and longest (taps, length) corners.
@pytest.mark.parametrize("k,n", [(1025, 1 << 24), (63, 1 << 24), (31, 1 << 12),
                                 (1025, 1 << 22), (255, 1 << 16)])
def test_tuned_fir_is_not_slower_than_the_builtin_rule(k: int, n: int) -> None:
    x, h = rand(n, k, seed=k + n)
    xd, hd = torch.from_numpy(x).to(DEV), torch.from_numpy(h).to(DEV)
    yd = torch.empty_like(xd)
    builtin = best_ms(lambda: rfx.fir_launch("auto", xd, hd, yd))
    rfx.autotune_fir("auto", k, n)
    tuned = best_ms(lambda: rfx.fir_launch("auto", xd, hd, yd))
    print(f"\nK={k} N={n}: built-in {builtin:.4f} ms, tuned "
          f"({rfx.fir_impl_used('auto', k, n)}) {tuned:.4f} ms")
    assert tuned <= 1.05 * builtin + 0.002
    rfx.fir_launch("auto", xd, hd, yd)
    torch.cuda.synchronize()
    m = min(n, 1 << 18)
    assert orc.normwise_error(yd[:m].cpu().numpy(), orc.fir_fast(x[:m], h)) <= 2e-6


@pytest.mark.parametrize("m,k,n", [(64, 1024, 1 << 24), (1024, 32768, 1 << 26),
                                   (16, 128, 1 << 20)])
def test_tuned_channelizer_is_not_slower_than_the_builtin_rule(m: int, k: int, n: int) -> None:
    x, h = rand(n, k, seed=m)
    xd, hd = torch.from_numpy(x).to(DEV), torch.from_numpy(h).to(DEV)
    z = torch.empty((rfx.frames(n, m), m), dtype=torch.complex64, device=DEV)
    with rfx.ChanPlan(m, n, "auto") as plan:
        builtin = best_ms(lambda: plan.launch(xd, hd, z), reps=10)
    rfx.autotune_channelize(m, k, n)
    with rfx.ChanPlan(m, n, "auto") as plan:
        tuned = best_ms(lambda: plan.launch(xd, hd, z), reps=10)
        plan.launch(xd, hd, z)
        torch.cuda.synchronize()
    print(f"\nM={m} N={n}: built-in {builtin:.4f} ms, tuned {tuned:.4f} ms")
    assert tuned <= 1.05 * builtin + 0.002
    f = min(rfx.frames(n, m), (1 << 18) // m)
    err = orc.normwise_error(z[:f].cpu().numpy(), orc.channelize_fast(x[:f * m], h, m))
    assert err <= 2e-6


def test_saved_table_reloads(tmp_path) -> None:
    rfx.autotune_fir("auto", 1025, 1 << 20)
    rfx.autotune_channelize(64, 1024, 1 << 20)
    picked = rfx.fir_impl_used("auto", 1025, 1 << 20)
    path = tmp_path / "tune.txt"
    rfx.autotune_save(path)
    lines = path.read_text().splitlines()
    assert any(l.startswith("fir ") for l in lines) and any(l.startswith("chan ") for l in lines)
    rfx.autotune_clear()
    rfx.autotune_load(path)
    assert rfx.fir_impl_used("auto", 1025, 1 << 20) == picked
