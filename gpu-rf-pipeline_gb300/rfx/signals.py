"""Seeded synthetic inputs for the filtering path: the gpu-rf-pipeline fixture signals and the
five benchmark workloads (plain FIR, long FIR, 64-channel channelizer, batched uneven FIR,
1024-channel channelizer).

Conventions kept from the gpu-rf-pipeline project, so that its fixture files are reproduced
byte for byte (tests check the SHA-256 of each against the project's own files):

* ``complex_noise`` and ``tones_plus_noise`` follow tools/gen_fixtures.py:44-68 — circular
  complex Gaussian noise with the power split evenly between I and Q, plus complex exponentials
  on exact bins of a 1024-point FFT.
* the fixture taps are ``scipy.signal.firwin`` designs (tools/gen_fixtures.py:219-231), stored
  as float32.
* a cf32 array is interleaved little-endian float32 I, Q (src/types.hpp:7-12); here it is a
  NumPy ``complex64`` array, which has that memory layout.
* the SigMF recording ``tone_ci16`` follows tools/gen_fixtures.py:109-128 and :188-193: the
  tone_odd signal (before float32 rounding) scaled to half of full scale, each component
  rounded to int16 of v * 32767, interleaved little-endian.

The benchmark workloads have no generator in the project; their definitions (sizes, seeds,
tap designs, tone and noise statistics) are this library's and are documented per function.
Every workload has its own seed, so adding one never changes another.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SAMPLE_RATE = 1_000_000.0
REF_NFFT = 1024  # fixture tones sit on exact bins of this FFT size

# The fixture tone pair: bin 40 inside the lowpass passband, bin -300 in its stopband.
FIXTURE_TONES = [{"bin": 40, "amplitude": 1.0}, {"bin": -300, "amplitude": 0.5}]


def complex_noise(rng: np.random.Generator, n: int, std: float) -> np.ndarray:
    """Circular complex Gaussian noise, total standard deviation ``std`` (std/sqrt(2) per
    component), drawn as all I values then all Q values."""
    per_component = std / np.sqrt(2.0)
    return per_component * (rng.standard_normal(n) + 1j * rng.standard_normal(n))


def tones_plus_noise(rng: np.random.Generator, n: int, tones: list[dict], noise_std: float
                     ) -> np.ndarray:
    """Complex exponentials on bins of a REF_NFFT-point FFT plus complex Gaussian noise,
    complex128. The expression order matches the fixture generator so the float32 files agree
    bit for bit."""
    t = np.arange(n, dtype=np.float64)
    x = np.zeros(n, dtype=np.complex128)
    for tone in tones:
        x += tone["amplitude"] * np.exp(2j * np.pi * tone["bin"] / REF_NFFT * t)
    return x + complex_noise(rng, n, noise_std)


def to_cf32(x: np.ndarray) -> np.ndarray:
    """complex128 -> complex64 (interleaved float32 I/Q), rounding each component."""
    out = np.empty(len(x), dtype=np.complex64)
    out.real = x.real
    out.imag = x.imag
    return out


def fixture_signal(name: str) -> np.ndarray:
    """The project's test fixture signals as complex64: tone (65536), tone_odd (10007),
    short (7), zeros (4096), and tone_ci16 (10007) as the pipeline reads that SigMF recording
    (each int16 component times 1/32768, exact in float32)."""
    if name == "tone":
        return to_cf32(tones_plus_noise(np.random.default_rng(1001), 65536, FIXTURE_TONES, 0.05))
    if name == "tone_odd":
        return to_cf32(tones_plus_noise(np.random.default_rng(1002), 10007, FIXTURE_TONES, 0.05))
    if name == "short":
        return to_cf32(tones_plus_noise(np.random.default_rng(1003), 7, FIXTURE_TONES, 0.05))
    if name == "zeros":
        return np.zeros(4096, dtype=np.complex64)
    if name == "tone_ci16":
        v = tone_ci16().astype(np.float32) * np.float32(1.0 / 32768.0)
        out = np.empty(v.size // 2, dtype=np.complex64)
        out.real = v[0::2]
        out.imag = v[1::2]
        return out
    raise KeyError(name)


def fixture_taps(name: str) -> np.ndarray:
    """The project's fixture filters as float32: lowpass = firwin(63, 0.2), lowpass_long =
    firwin(1025, 0.2), channelizer_proto = firwin(128, 1/16), identity = [1.0]."""
    from scipy import signal

    if name == "lowpass":
        return signal.firwin(63, 0.2).astype(np.float32)
    if name == "lowpass_long":
        return signal.firwin(1025, 0.2).astype(np.float32)
    if name == "channelizer_proto":
        return signal.firwin(16 * 8, 1 / 16).astype(np.float32)
    if name == "identity":
        return np.array([1.0], dtype=np.float32)
    raise KeyError(name)


def tone_ci16() -> np.ndarray:
    """The project's SigMF fixture ``tone_ci16``: interleaved little-endian int16 I/Q
    components (2 * 10007 values), the contents of tone_ci16.sigmf-data."""
    x = tones_plus_noise(np.random.default_rng(1002), 10007, FIXTURE_TONES, 0.05)
    x = 0.5 * x / np.max(np.abs(x))
    iq = np.empty(2 * len(x), dtype="<i2")
    iq[0::2] = np.round(x.real * 32767)
    iq[1::2] = np.round(x.imag * 32767)
    return iq


def write_sigmf(stem, components: np.ndarray, datatype: str,
                sample_rate: float = SAMPLE_RATE, num_channels: int = 1) -> None:
    """Writes STEM.sigmf-data (the interleaved components as given) and STEM.sigmf-meta with
    the SigMF core fields the pipeline reads (datatype, sample rate, channel count)."""
    import json
    from pathlib import Path

    stem = Path(stem)
    np.ascontiguousarray(components).tofile(stem.with_name(stem.name + ".sigmf-data"))
    meta = {
        "global": {
            "core:datatype": datatype,
            "core:sample_rate": sample_rate,
            "core:version": "1.2.0",
            "core:num_channels": num_channels,
        },
        "captures": [{"core:sample_start": 0}],
        "annotations": [],
    }
    stem.with_name(stem.name + ".sigmf-meta").write_text(json.dumps(meta, indent=2) + "\n")


# --- benchmark workloads ------------------------------------------------------------------

def _tone_bank(rng: np.random.Generator, n: int, count: int, span_db: float,
               snr_db: float) -> np.ndarray:
    """``count`` complex tones with frequencies uniform in [-0.5, 0.5) fs, amplitudes
    log-uniform over ``span_db`` (largest 1.0), uniform random phase, plus circular complex
    Gaussian noise at ``snr_db`` below the total tone power; complex64.

    Each tone is built block-wise as e^{i w (t0 + j)} = e^{i w t0} e^{i w j}, both factors from
    float64 angles reduced modulo 2 pi, which keeps the phase error near 1e-16 at 2^26 samples.
    """
    freqs = rng.uniform(-0.5, 0.5, count)
    amps = 10.0 ** (-rng.uniform(0.0, span_db, count) / 20.0)
    amps[np.argmax(amps)] = 1.0
    phases = rng.uniform(0.0, 2.0 * np.pi, count)
    noise_power = float(np.sum(amps ** 2)) / (10.0 ** (snr_db / 10.0))
    block = 4096
    blocks = -(-n // block)
    j = np.arange(block, dtype=np.float64)
    starts = np.arange(blocks, dtype=np.float64) * block
    x = np.zeros(blocks * block, dtype=np.complex128)
    xv = x.reshape(blocks, block)
    for f, a, p in zip(freqs, amps, phases):
        inner = np.exp(1j * np.mod(2.0 * np.pi * f * j, 2.0 * np.pi))
        outer = a * np.exp(1j * (np.mod(2.0 * np.pi * f * starts, 2.0 * np.pi) + p))
        xv += outer[:, None] * inner[None, :]
    x = x[:n]
    x += complex_noise(rng, n, math.sqrt(noise_power))
    return to_cf32(x)


def white_noise_cf32(rng: np.random.Generator, n: int) -> np.ndarray:
    """I and Q each i.i.d. N(0, 1), complex64."""
    out = np.empty(n, dtype=np.complex64)
    out.real = rng.standard_normal(n, dtype=np.float32)
    out.imag = rng.standard_normal(n, dtype=np.float32)
    return out


@dataclass
class Workload:
    """One benchmark input: a capture (or several) and its filter."""

    name: str
    x: np.ndarray                      # complex64 samples (single capture)
    taps: np.ndarray                   # float32 taps
    channels: int = 0                  # 0 for a FIR, M for a channelizer
    captures: list = field(default_factory=list)  # [(x, taps)] for the batched workload
    meta: dict = field(default_factory=dict)


def plain_fir(n: int = 1 << 24) -> Workload:
    """Plain complex FIR: N(0,1) I/Q (seed 1), 63 taps = Hamming-windowed sinc with cutoff
    0.1 fs (firwin(63, 0.2))."""
    from scipy import signal

    x = white_noise_cf32(np.random.default_rng(1), n)
    taps = signal.firwin(63, 0.2).astype(np.float32)
    return Workload("fir63_white", x, taps, meta={"seed": 1, "taps": "firwin(63, 0.2)"})


def long_fir(n: int = 1 << 24) -> Workload:
    """Long complex FIR: 8 tones over 60 dB plus AWGN at 10 dB SNR (seed 2), 1025 taps =
    Kaiser(beta 8) windowed sinc with cutoff 0.05 fs (firwin(1025, 0.1, ('kaiser', 8)))."""
    from scipy import signal

    x = _tone_bank(np.random.default_rng(2), n, 8, 60.0, 10.0)
    taps = signal.firwin(1025, 0.1, window=("kaiser", 8.0)).astype(np.float32)
    return Workload("fir1025_tones", x, taps,
                    meta={"seed": 2, "taps": "firwin(1025, 0.1, kaiser 8)"})


def channelizer64(n: int = 1 << 24) -> Workload:
    """64-channel critically sampled channelizer: 8 tones over 60 dB + AWGN 10 dB (seed 3),
    prototype firwin(1024, 1/64) (Hamming, cutoff 1/M of Nyquist), 16 taps per branch."""
    from scipy import signal

    x = _tone_bank(np.random.default_rng(3), n, 8, 60.0, 10.0)
    taps = signal.firwin(1024, 1.0 / 64).astype(np.float32)
    return Workload("pfb64", x, taps, channels=64, meta={"seed": 3, "taps": "firwin(1024, 1/64)"})


def channelizer1024(n: int = 1 << 26) -> Workload:
    """1024-channel channelizer: 16 tones over 60 dB + AWGN 10 dB (seed 5), prototype
    firwin(32768, 1/1024, ('kaiser', 10)), 32 taps per branch."""
    from scipy import signal

    x = _tone_bank(np.random.default_rng(5), n, 16, 60.0, 10.0)
    taps = signal.firwin(32768, 1.0 / 1024, window=("kaiser", 10.0)).astype(np.float32)
    return Workload("pfb1024", x, taps, channels=1024,
                    meta={"seed": 5, "taps": "firwin(32768, 1/1024, kaiser 10)"})


BATCH_TAP_CHOICES = (31, 63, 127, 255, 511, 1025)


def batched_fir(count: int = 256, log2_min: float = 12.0, log2_max: float = 22.0,
                seed: int = 4) -> Workload:
    """Batched uneven FIR: ``count`` captures, lengths floor(2^U[log2_min, log2_max]), tap
    counts uniform over BATCH_TAP_CHOICES, Hamming windowed-sinc taps with cutoff
    U[0.02, 0.25] fs; each capture is 4 tones over 60 dB plus AWGN at 10 dB (seed 4, one
    generator for the whole batch)."""
    from scipy import signal

    rng = np.random.default_rng(seed)
    lengths = np.floor(2.0 ** rng.uniform(log2_min, log2_max, count)).astype(np.int64)
    ks = rng.choice(np.array(BATCH_TAP_CHOICES), count)
    cutoffs = rng.uniform(0.02, 0.25, count)
    captures = []
    for n, k, fc in zip(lengths, ks, cutoffs):
        x = _tone_bank(rng, int(n), 4, 60.0, 10.0)
        taps = signal.firwin(int(k), 2.0 * float(fc)).astype(np.float32)
        captures.append((x, taps))
    total = int(lengths.sum())
    return Workload("batch256", np.zeros(0, np.complex64), np.zeros(0, np.float32),
                    captures=captures,
                    meta={"seed": seed, "count": count, "total_samples": total})


WORKLOADS = {
    "fir63": plain_fir,
    "fir1025": long_fir,
    "pfb64": channelizer64,
    "batch256": batched_fir,
    "pfb1024": channelizer1024,
}
