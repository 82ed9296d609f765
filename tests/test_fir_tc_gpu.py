"""Tensor-core FIR (tc_split) on the GPU through the C ABI, against the float64 oracle.

The split-FP16 form is not bit-exact; it is gated on the normwise relative error
max|y - y_ref| / max|y_ref| <= 2e-6 (TC_NORMWISE), the accuracy target of the workload, and on the
project's FIR tolerance (rtol = atol = 1e-5, tests/test_pipeline.py:116-117) for its fixtures.
One tap is computed by the plain kernel, so identity stays bit-exact; zeros give exact zeros.
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
FIR_RTOL = 1e-5
FIR_ATOL = 1e-5
DEV = torch.device("cuda:0")


def run(x: np.ndarray, h: np.ndarray, impl: str = "tc_split") -> np.ndarray:
    xd = torch.from_numpy(np.ascontiguousarray(x)).to(DEV)
    hd = torch.from_numpy(np.ascontiguousarray(h)).to(DEV)
    y = rfx.fir(xd, hd, impl=impl)
    torch.cuda.synchronize()
    return y.cpu().numpy()


def rand_case(n: int, k: int, seed: int):
    rng = np.random.default_rng(seed)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    return x, h


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


@pytest.mark.parametrize("name,taps", [("tone", "lowpass"), ("tone", "lowpass_long"),
                                       ("tone_odd", "lowpass"), ("tone_odd", "lowpass_long"),
                                       ("short", "lowpass"), ("short", "lowpass_long")])
def test_tc_matches_reference(name: str, taps: str) -> None:
    x, h = signals.fixture_signal(name), signals.fixture_taps(taps)
    y = run(x, h)
    ref = orc.fir_fast(x, h)
    np.testing.assert_allclose(y, ref, rtol=FIR_RTOL, atol=FIR_ATOL)
    assert orc.normwise_error(y, ref) <= TC_NORMWISE


@pytest.mark.parametrize("name", ["tone", "tone_odd", "short"])
def test_tc_identity_is_exact(name: str) -> None:
    x = signals.fixture_signal(name)
    y = run(x, signals.fixture_taps("identity"))
    assert np.array_equal(y.view(np.uint32), x.view(np.uint32))


@pytest.mark.parametrize("taps", ["lowpass", "lowpass_long"])
def test_tc_zeros_are_exact(taps: str) -> None:
    y = run(signals.fixture_signal("zeros"), signals.fixture_taps(taps))
    assert not np.any(y)


# Tap counts whose tap strip, sample ring and operand stages fit the 227 KB of shared memory.
TC_MAX_TAPS = 3457


@pytest.mark.parametrize("k", [2, 3, 16, 31, 63, 64, 127, 128, 129, 255, 256, 257, 1025, 2049,
                               TC_MAX_TAPS])
def test_tc_tap_counts(k: int) -> None:
    x, h = rand_case(40000, k, seed=k)
    y = run(x, h)
    assert orc.normwise_error(y, orc.fir_fast(x, h)) <= TC_NORMWISE


TILE = 96 * 128  # outputs per tensor-core tile


@pytest.mark.parametrize("n", [1, 5, 127, 128, 129, TILE - 1, TILE, TILE + 1, 3 * TILE + 77,
                               200001])
def test_tc_lengths(n: int) -> None:
    x, h = rand_case(n, 1025, seed=n)
    y = run(x, h)
    assert orc.normwise_error(y, orc.fir_fast(x, h)) <= TC_NORMWISE


SHORT_TILE = 48 * 128  # outputs per tile of the resident-window form (2 to 385 taps)


@pytest.mark.parametrize("k", [2, 63, 113, 114, 129, 130, 241, 257, 385])
@pytest.mark.parametrize("n", [128, 129, 255, 49 * 128 + 5, SHORT_TILE - 1, SHORT_TILE,
                               SHORT_TILE + 1, 3 * SHORT_TILE + 77, 152 * SHORT_TILE + 300])
def test_tc_window_form_lengths(k: int, n: int) -> None:
    # Tile edges of the resident-window form, its partial last block (outside the tensor map,
    # read from global memory into the window), windows reaching past the input, and grids with
    # more tiles than SMs; 113 and 114 taps bracket the first K-step that needs the previous
    # block's taps; 130 to 385 taps reach back two and three blocks, in H groups of several
    # K-steps summed into running sums.
    x, h = rand_case(n, k, seed=n + k)
    y = run(x, h)
    assert orc.normwise_error(y, orc.fir_fast(x, h)) <= TC_NORMWISE


def test_tc_window_form_per_tile_scale_spans_extreme_levels() -> None:
    x, h = rand_case(6 * SHORT_TILE, 63, seed=12)
    levels = np.array([1.0, 1e-30, 1e30, 3.0, 1e-12, 1.0])
    x = (x * np.repeat(levels, SHORT_TILE).astype(np.float32)).astype(np.complex64)
    y = run(x, h)
    ref = orc.fir_fast(x, h)
    assert orc.normwise_error(y, ref) <= TC_NORMWISE
    for t in range(6):
        if t > 0 and levels[t - 1] > levels[t]:
            continue
        seg = slice(t * SHORT_TILE + 128, (t + 1) * SHORT_TILE)
        assert orc.normwise_error(y[seg], ref[seg]) <= TC_NORMWISE, t


@pytest.mark.parametrize("fmt", ["ci16", "ci8"])
@pytest.mark.parametrize("k", [63, 300])
def test_tc_window_form_integer_input_matches_converted(fmt: str, k: int) -> None:
    # Integer recordings decoded in the resident-window form's load stage give the bits of a
    # run over the host-converted samples.
    n = 3 * SHORT_TILE + 333
    rng = np.random.default_rng(21)
    info = np.iinfo(np.int16 if fmt == "ci16" else np.int8)
    raw = rng.integers(info.min, info.max + 1, size=2 * n).astype(info.dtype)
    conv = (raw.astype(np.float32) / (32768.0 if fmt == "ci16" else 128.0)).view(np.complex64)
    h = rand_case(1, k, seed=4)[1]
    hd = torch.from_numpy(h).to(DEV)
    yf = torch.empty(n, dtype=torch.complex64, device=DEV)
    rfx.fir_launch_format("tc_split", fmt, torch.from_numpy(raw).to(DEV), hd, yf, num_samples=n)
    yc = rfx.fir(torch.from_numpy(conv).to(DEV), hd, impl="tc_split")
    torch.cuda.synchronize()
    assert np.array_equal(yf.cpu().numpy().view(np.uint32), yc.cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("k", [TC_MAX_TAPS + 1, 8192])
def test_tc_beyond_capacity_uses_the_plain_kernel(k: int) -> None:
    x, h = rand_case(30000, k, seed=3)
    y = run(x, h)
    assert np.array_equal(y.view(np.uint32), orc.fir_f32_seq(x, h).view(np.uint32))


def test_tc_per_tile_scale_spans_extreme_levels() -> None:
    # Tiles (TILE outputs) at 1, 1e-30, 1e30, 3, 1e-12 and 1 times the unit level. Each tile
    # is scaled by the largest sample of its input window, which reaches C = 2 blocks into the
    # previous tile: a tile is held to 2e-6 of its own level when the previous tile is not
    # louder, and the whole capture to 2e-6 normwise.
    x, h = rand_case(6 * TILE, 255, seed=11)
    levels = np.array([1.0, 1e-30, 1e30, 3.0, 1e-12, 1.0])
    x = (x * np.repeat(levels, TILE).astype(np.float32)).astype(np.complex64)
    y = run(x, h)
    ref = orc.fir_fast(x, h)
    assert orc.normwise_error(y, ref) <= TC_NORMWISE
    for t in range(6):
        if t > 0 and levels[t - 1] > levels[t]:
            continue
        seg = slice(t * TILE + 512, (t + 1) * TILE)   # past the previous tile's filter tail
        assert orc.normwise_error(y[seg], ref[seg]) <= TC_NORMWISE, t


def test_tc_sixty_db_workload() -> None:
    w = signals.long_fir(1 << 22)
    y = run(w.x, w.taps)
    assert orc.normwise_error(y, orc.fir_fast(w.x, w.taps)) <= TC_NORMWISE


def test_tc_short_filter_workload() -> None:
    w = signals.plain_fir(1 << 21)
    y = run(w.x, w.taps)
    assert orc.normwise_error(y, orc.fir_fast(w.x, w.taps)) <= TC_NORMWISE


def test_tc_is_deterministic() -> None:
    x, h = rand_case(100000, 1025, seed=5)
    assert np.array_equal(run(x, h).view(np.uint32), run(x, h).view(np.uint32))


def test_tc_batched_entry_points() -> None:
    h = rand_case(1, 511, seed=2)[1]
    xs = [rand_case(n, 1, seed=n)[0] for n in (300, 20000, 70001)]
    xd = [torch.from_numpy(x).to(DEV) for x in xs]
    yd = [torch.empty_like(t) for t in xd]
    rfx.fir_batched(xd, yd, torch.from_numpy(h).to(DEV), impl="tc_split")
    torch.cuda.synchronize()
    for x, y in zip(xs, yd):
        assert orc.normwise_error(y.cpu().numpy(), orc.fir_fast(x, h)) <= TC_NORMWISE


def test_tc_host_path() -> None:
    x, h = rand_case(123457, 1025, seed=9)
    y, bench = rfx.fir_host("tc_split", x, h, warmup=1, runs=2)
    assert orc.normwise_error(y, orc.fir_fast(x, h)) <= TC_NORMWISE
    assert bench.kernel_ms_mean > 0


@pytest.mark.parametrize("k", [63, 255, 1025])
def test_tc_sixty_db_level_steps_per_block(k: int) -> None:
    # Every 128-output block at its own level, 1 or 1e-3 at random (60 dB steps inside every
    # tile, the workload's dynamic range). The split operands are floating point, so a quiet
    # sample keeps its relative precision under its tile's scale; each output block is held to
    # 2e-6 of its own level, or, where an output block's own level is far below the inputs that
    # reach it through the taps, to within 4x of the exact FP32 chain's error there (the plain
    # kernel's, which no float32 arithmetic beats by much).
    n = 40 * TILE // 8
    rng = np.random.default_rng(k)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    levels = np.where(rng.random(n // 128) < 0.5, 1.0, 1e-3)
    x = (x * np.repeat(levels, 128).astype(np.float32)).astype(np.complex64)
    h = signals.long_fir(1 << 12).taps if k == 1025 else rand_case(1, k, seed=k)[1]
    ref = orc.fir_fast(x, h)
    y_tc = run(x, h)
    y_plain = run(x, h, impl="plain")
    blocks = n // 128

    def per_block(y):
        d = np.abs(y.astype(np.complex128) - ref).reshape(blocks, 128).max(axis=1)
        return d / np.abs(ref).reshape(blocks, 128).max(axis=1)

    e_tc, e_plain = per_block(y_tc), per_block(y_plain)
    print(f"\nK={k}: tensor-core per-block error max {e_tc.max():.3g}, median "
          f"{np.median(e_tc):.3g}; plain FP32 max {e_plain.max():.3g}")
    assert np.all(e_tc <= np.maximum(TC_NORMWISE, 4 * e_plain))
