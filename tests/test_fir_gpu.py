"""FIR on the GPU through the C ABI, against the oracle.

Mirrors the project's FIR tests (tests/test_pipeline.py:113-167): fixture signals and filters at
rtol = atol = 1e-5, identity bit-exact, zeros exactly zero. On top of that, the plain kernel is
compared BIT FOR BIT with the oracle's restatement of the project's float32 arithmetic
(oracle.rf_oracle.fir_f32_seq), over sizes around every tile boundary and tap counts around
every unroll boundary.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import rfx
from oracle import rf_oracle as orc
from rfx import signals

pytestmark = pytest.mark.gpu

FIR_RTOL = 1e-5
FIR_ATOL = 1e-5
DEV = torch.device("cuda:0")


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def run_fir(x: np.ndarray, h: np.ndarray, impl="plain") -> np.ndarray:
    y = rfx.fir(dev(x), dev(h), impl=impl)
    torch.cuda.synchronize()
    return y.cpu().numpy()


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a).view(np.uint32)


def rand_case(n: int, k: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
    return x, h


@pytest.fixture(scope="module", autouse=True)
def no_faults():
    rfx.load()
    yield
    assert rfx.device_fault() == 0


# --- the project's fixture cases -----------------------------------------------------------

@pytest.mark.parametrize("impl", ["plain", "register", "naive"])
@pytest.mark.parametrize("name,taps", [("tone", "lowpass"), ("tone", "lowpass_long"),
                                       ("tone_odd", "lowpass"), ("tone_odd", "lowpass_long"),
                                       ("short", "lowpass"), ("short", "lowpass_long")])
def test_fir_matches_reference(impl: str, name: str, taps: str) -> None:
    x, h = signals.fixture_signal(name), signals.fixture_taps(taps)
    y = run_fir(x, h, impl)
    assert y.shape == x.shape
    np.testing.assert_allclose(y, orc.fir_fast(x, h), rtol=FIR_RTOL, atol=FIR_ATOL)
    assert np.array_equal(bits(y), bits(orc.fir_f32_seq(x, h)))


@pytest.mark.parametrize("name", ["tone", "tone_odd", "short"])
def test_fir_identity_returns_the_input_exactly(name: str) -> None:
    x = signals.fixture_signal(name)
    assert np.array_equal(bits(run_fir(x, signals.fixture_taps("identity"))), bits(x))


@pytest.mark.parametrize("taps", ["lowpass", "lowpass_long", "identity"])
def test_fir_of_zeros_is_exactly_zero(taps: str) -> None:
    y = run_fir(signals.fixture_signal("zeros"), signals.fixture_taps(taps))
    assert y.shape == (4096,) and not np.any(y)


# --- bit-exact against the float32 restatement, around every boundary ----------------------

TILE = 2304
EDGE_N = [1, 2, 7, 8, 9, 100, TILE - 1, TILE, TILE + 1, 2 * TILE + 7, 5 * TILE - 3, 30011]
EDGE_K = [1, 2, 8, 9, 10, 17, 18, 19, 31, 63, 64, 65, 127, 128, 255, 1025, 1089, 2305]


@pytest.mark.parametrize("k", EDGE_K)
def test_plain_is_bit_exact_for_tap_counts(k: int) -> None:
    x, h = rand_case(3 * TILE + 5, k, seed=k)
    assert np.array_equal(bits(run_fir(x, h)), bits(orc.fir_f32_seq(x, h)))


@pytest.mark.parametrize("n", EDGE_N)
@pytest.mark.parametrize("k", [1, 63, 1025])
def test_plain_is_bit_exact_for_lengths(n: int, k: int) -> None:
    x, h = rand_case(n, k, seed=n + k)
    assert np.array_equal(bits(run_fir(x, h)), bits(orc.fir_f32_seq(x, h)))


def test_maximum_tap_count() -> None:
    x, h = rand_case(20000, 8192, seed=8192)
    assert np.array_equal(bits(run_fir(x, h)), bits(orc.fir_f32_seq(x, h)))


@pytest.mark.parametrize("k", [63, 1025])
def test_full_size_workload_is_bit_exact(k: int) -> None:
    w = signals.plain_fir(1 << 22) if k == 63 else signals.long_fir(1 << 22)
    y = run_fir(w.x, w.taps)
    assert np.array_equal(bits(y), bits(orc.fir_f32_seq(w.x, w.taps)))


def test_ragged_signed_zero_and_large_values() -> None:
    x = np.zeros(5000, dtype=np.complex64)
    x[::7] = -0.0
    x[3::11] = 3.0e30 + 1j * -2.5e-30
    h = np.array([0.5, -0.25, 0.0, 1e-3] * 9, dtype=np.float32)
    assert np.array_equal(bits(run_fir(x, h)), bits(orc.fir_f32_seq(x, h)))


# --- the other entry points -----------------------------------------------------------------

def test_launch_on_a_side_stream() -> None:
    x, h = rand_case(50000, 255, seed=1)
    s = torch.cuda.Stream()
    xd, hd = dev(x), dev(h)
    y = torch.empty_like(xd)
    with torch.cuda.stream(s):
        rfx.fir_launch("plain", xd, hd, y, stream=s)
    s.synchronize()
    assert np.array_equal(bits(y.cpu().numpy()), bits(orc.fir_f32_seq(x, h)))


def test_batched_shared_taps_equals_separate_calls() -> None:
    h = rand_case(1, 127, seed=5)[1]
    xs = [rand_case(n, 1, seed=n)[0] for n in (1, 100, 4099, 70000, 0, 2304 * 3)]
    xd = [dev(x) for x in xs]
    yd = [torch.empty_like(t) for t in xd]
    rfx.fir_batched(xd, yd, dev(h))
    torch.cuda.synchronize()
    for x, y in zip(xs, yd):
        assert np.array_equal(bits(y.cpu().numpy()), bits(orc.fir_f32_seq(x, h)))


def test_batched_beyond_eight_channels() -> None:
    h = rand_case(1, 31, seed=6)[1]
    xs = [rand_case(1000 + 37 * i, 1, seed=i)[0] for i in range(70)]
    xd = [dev(x) for x in xs]
    yd = [torch.empty_like(t) for t in xd]
    rfx.fir_batched(xd, yd, dev(h))
    torch.cuda.synchronize()
    for x, y in zip(xs, yd):
        assert np.array_equal(bits(y.cpu().numpy()), bits(orc.fir_f32_seq(x, h)))


def test_per_capture_taps_batch() -> None:
    w = signals.batched_fir(count=24, log2_min=8, log2_max=16, seed=44)
    caps = []
    for x, h in w.captures:
        caps.append((dev(x), None, dev(h)))
    caps = [(x, torch.empty_like(x), h) for x, _, h in caps]
    rfx.fir_batch(caps, impl="plain")
    torch.cuda.synchronize()
    for (x, h), (_, y, _) in zip(w.captures, caps):
        assert np.array_equal(bits(y.cpu().numpy()), bits(orc.fir_f32_seq(x, h)))


def test_host_buffer_path_matches_device_path() -> None:
    x, h = rand_case(123457, 1025, seed=9)
    y, bench = rfx.fir_host("plain", x, h, block=96, warmup=1, runs=3)
    assert np.array_equal(bits(y), bits(orc.fir_f32_seq(x, h)))
    assert bench.kernel_ms_mean > 0 and bench.h2d_ms_mean > 0 and bench.d2h_ms_mean > 0
    assert bench.kernel_ms_std >= 0


@pytest.mark.parametrize("block", [32, 96, 1024])
def test_block_size_does_not_change_the_result(block: int) -> None:
    x, h = signals.fixture_signal("tone_odd"), signals.fixture_taps("lowpass_long")
    y, _ = rfx.fir_host("plain", x, h, block=block)
    np.testing.assert_allclose(y, orc.fir_fast(x, h), rtol=FIR_RTOL, atol=FIR_ATOL)


def test_misaligned_device_pointer_is_rejected() -> None:
    xd = dev(rand_case(100, 1, seed=2)[0])
    hd = dev(np.ones(3, np.float32))
    y = torch.empty_like(xd)
    with pytest.raises(rfx.RfxError) as e:
        rfx.fir_launch("plain", xd[1:], hd, y[1:])
    assert e.value.status == 3
