"""CPU oracle for the complex-baseband filtering path.

TEST INFRASTRUCTURE ONLY: this module is the checker. Only tests/, __graft_entry__.smoke() and
bench.py (its cpu_baseline leg and its ``--impl reference`` arm) may import it; the library in
gpu-rf-pipeline_gb300/ never does, and it has no CPU fallback through here.

Restated from the gpu-rf-pipeline project (file:line inside that project):

* ``fir``          tools/reference.py:103-111 — causal FIR with zero initial state, float64,
                   output length N. Written here as a direct-form sum over taps.
* ``channelize``   tools/reference.py:128-146 — z[t][k] = sum_l h[l] x[tM-l] e^{+2 pi i k l/M}
                   for t < ceil(N/M), computed as M polyphase branch sums u[t][m] followed by
                   the unnormalized inverse DFT over m (M * ifft).
* ``fir_f32_seq``  src/fir.cu:30-40 — the reference GPU kernels' float32 arithmetic (one fused
                   multiply-add per tap, taps in ascending order), for bit-exact comparisons.
* ``channelize_branch_f32_seq``  src/channelize.cu:25-49 — the reference's float32 branch sums.
* ``magnitude``    tools/reference.py:98-100 — |z| of each value, float64.
* ``decode``       src/io.cpp:110-148 — SigMF integer samples to cf32: each ci16_le component
                   v * (1 / 32768), each ci8 component v * (1 / 128), in float32.

The float64 functions exist twice: in NumPy here (for small inputs and to pin the C code) and
in C (oracle/rf_oracle.c, threaded, for the large workloads). Golden vectors produced by the
project's own tools/reference.py pin both (tests/golden/).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "librforacle.so"

_lib = None
_lib_lock = threading.Lock()


def build() -> Path:
    """Compile oracle/rf_oracle.c into oracle/_build/librforacle.so (make, then gcc directly)."""
    try:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True, capture_output=True)
    except (OSError, subprocess.CalledProcessError):
        (HERE / "_build").mkdir(exist_ok=True)
        subprocess.run(["gcc", "-O3", "-fPIC", "-std=c11", "-ffp-contract=off", "-shared",
                        "-pthread", "-o", str(LIB_PATH), str(HERE / "rf_oracle.c"), "-lm"],
                       check=True)
    return LIB_PATH


def _load():
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        src = HERE / "rf_oracle.c"
        if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
            build()
        lib = ctypes.CDLL(str(LIB_PATH))
        i64, c_int, vp = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
        lib.rfo_fir_f64.argtypes = [vp, i64, vp, c_int, vp, c_int]
        lib.rfo_fir_f64.restype = None
        lib.rfo_fir_f32_seq.argtypes = [vp, i64, vp, c_int, vp, c_int]
        lib.rfo_fir_f32_seq.restype = None
        lib.rfo_channelize_f64.argtypes = [vp, i64, vp, c_int, c_int, vp, c_int]
        lib.rfo_channelize_f64.restype = c_int
        lib.rfo_channelize_branch_f32_seq.argtypes = [vp, i64, vp, c_int, c_int, vp, c_int]
        lib.rfo_channelize_branch_f32_seq.restype = c_int
        lib.rfo_channelize_frames.argtypes = [i64, c_int]
        lib.rfo_channelize_frames.restype = i64
        _lib = lib
        return lib


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def _cf32(x: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.complex64)


def _taps32(taps: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(taps, dtype=np.float32)


# --- NumPy restatements -------------------------------------------------------------------

def magnitude(z: np.ndarray) -> np.ndarray:
    """|z| of each value, float64, same shape."""
    return np.abs(np.asarray(z, dtype=np.complex128))


SAMPLE_FORMATS = {"cf32": 0, "ci16": 1, "ci8": 2}  # rfx_sample_format


def decode(components: np.ndarray, fmt: str) -> np.ndarray:
    """Interleaved I/Q components in ``fmt`` (cf32: float32; ci16: int16; ci8: int8) as cf32
    samples, converted as the project's SigMF reader does: the component, as float32, times
    1/32768 (ci16) or 1/128 (ci8)."""
    c = np.asarray(components)
    if c.size % 2 != 0:
        raise ValueError("odd number of components, not I/Q pairs")
    if fmt == "cf32":
        v = c.astype(np.float32)
    elif fmt == "ci16":
        v = c.astype("<i2").astype(np.float32) * np.float32(1.0 / 32768.0)
    elif fmt == "ci8":
        v = c.astype(np.int8).astype(np.float32) * np.float32(1.0 / 128.0)
    else:
        raise ValueError(f"unknown sample format {fmt!r}")
    out = np.empty(c.size // 2, dtype=np.complex64)
    out.real = v[0::2]
    out.imag = v[1::2]
    return out

def fir(x: np.ndarray, taps: np.ndarray) -> np.ndarray:
    """y[n] = sum_k taps[k] x[n-k] with x[m<0] = 0, len(y) = len(x), complex128.

    Direct form: one vectorized multiply-add of a shifted copy of x per tap."""
    taps = np.asarray(taps, dtype=np.float64)
    if taps.size < 1:
        raise ValueError("need at least one tap")
    x = np.asarray(x, dtype=np.complex128)
    n = x.size
    y = np.zeros(n, dtype=np.complex128)
    for k in range(min(taps.size, n)):
        y[k:] += taps[k] * x[: n - k]
    return y


def channelize(x: np.ndarray, taps: np.ndarray, channels: int) -> np.ndarray:
    """Critically sampled polyphase channelizer, shape (ceil(N/M), M), complex128.

    Branch m of frame t sums taps l = m, m+M, m+2M, ... against x[tM - l]; the branch vector of
    each frame then goes through the unnormalized inverse DFT (M * ifft)."""
    m = int(channels)
    taps = np.asarray(taps, dtype=np.float64)
    if m < 1 or taps.size < 1:
        raise ValueError("need at least one channel and one tap")
    x = np.asarray(x, dtype=np.complex128)
    frames = -(-x.size // m)
    per_branch = -(-taps.size // m)
    h = np.zeros(per_branch * m)
    h[: taps.size] = taps
    # history[i] = x[i - lead]: lead zeros in front cover every index tM - l >= -(lead).
    lead = per_branch * m
    history = np.concatenate([np.zeros(lead, dtype=np.complex128), x])
    newest = np.arange(frames, dtype=np.int64) * m + lead          # index of x[tM]
    branch = np.arange(m, dtype=np.int64)
    u = np.zeros((frames, m), dtype=np.complex128)
    for p in range(per_branch):
        idx = newest[:, None] - (p * m + branch)[None, :]
        u += h[p * m: (p + 1) * m][None, :] * history[idx]
    return np.fft.ifft(u, axis=1) * m


# --- C restatements -------------------------------------------------------------------------

def fir_fast(x: np.ndarray, taps: np.ndarray, threads: int | None = None) -> np.ndarray:
    """Same as ``fir`` (float64), computed by the threaded C oracle."""
    lib = _load()
    xc, tc = _cf32(x), _taps32(taps)
    if tc.size < 1:
        raise ValueError("need at least one tap")
    y = np.empty(xc.size, dtype=np.complex128)
    lib.rfo_fir_f64(xc.ctypes.data, xc.size, tc.ctypes.data, tc.size, y.ctypes.data,
                    threads or default_threads())
    return y


def fir_f32_seq(x: np.ndarray, taps: np.ndarray, threads: int | None = None) -> np.ndarray:
    """The reference GPU kernels' float32 result, bit for bit: complex64."""
    lib = _load()
    xc, tc = _cf32(x), _taps32(taps)
    y = np.empty(xc.size, dtype=np.complex64)
    lib.rfo_fir_f32_seq(xc.ctypes.data, xc.size, tc.ctypes.data, tc.size, y.ctypes.data,
                        threads or default_threads())
    return y


def channelize_fast(x: np.ndarray, taps: np.ndarray, channels: int,
                    threads: int | None = None) -> np.ndarray:
    """Same as ``channelize`` (float64), computed by the threaded C oracle."""
    lib = _load()
    xc, tc = _cf32(x), _taps32(taps)
    frames = int(lib.rfo_channelize_frames(xc.size, channels))
    z = np.empty(frames * channels, dtype=np.complex128)
    rc = lib.rfo_channelize_f64(xc.ctypes.data, xc.size, tc.ctypes.data, tc.size, channels,
                                z.ctypes.data, threads or default_threads())
    if rc != 0:
        raise ValueError("need at least one channel and one tap")
    return z.reshape(frames, channels)


def channelize_branch_f32_seq(x: np.ndarray, taps: np.ndarray, channels: int,
                              threads: int | None = None) -> np.ndarray:
    """The reference's float32 branch sums u[t][m], bit for bit: complex64 (frames, M)."""
    lib = _load()
    xc, tc = _cf32(x), _taps32(taps)
    frames = int(lib.rfo_channelize_frames(xc.size, channels))
    u = np.empty(frames * channels, dtype=np.complex64)
    rc = lib.rfo_channelize_branch_f32_seq(xc.ctypes.data, xc.size, tc.ctypes.data, tc.size,
                                           channels, u.ctypes.data, threads or default_threads())
    if rc != 0:
        raise ValueError("need at least one channel and one tap")
    return u.reshape(frames, channels)


# --- error measures -------------------------------------------------------------------------

def normwise_error(y: np.ndarray, ref: np.ndarray) -> float:
    """max |y - ref| / max |ref| (0 when both are all zero)."""
    y = np.asarray(y).astype(np.complex128).ravel()
    ref = np.asarray(ref).astype(np.complex128).ravel()
    scale = float(np.max(np.abs(ref))) if ref.size else 0.0
    diff = float(np.max(np.abs(y - ref))) if ref.size else 0.0
    if scale == 0.0:
        return 0.0 if diff == 0.0 else float("inf")
    return diff / scale


def per_channel_error(z: np.ndarray, ref: np.ndarray) -> np.ndarray:
    """Per channel: max_t |z - ref| / max_t |ref| over that channel's frames."""
    z = np.asarray(z).astype(np.complex128)
    ref = np.asarray(ref).astype(np.complex128)
    scale = np.max(np.abs(ref), axis=0)
    diff = np.max(np.abs(z - ref), axis=0)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(scale > 0, diff / np.where(scale > 0, scale, 1.0),
                        np.where(diff > 0, np.inf, 0.0))


def fir_convolve(x: np.ndarray, taps: np.ndarray) -> np.ndarray:
    """``fir`` by the project's own method (tools/reference.py:103-111): the first len(x)
    samples of NumPy's full convolution in float64, on one core. Timed as the CPU baseline of
    the project's implementation; same values as ``fir`` to rounding."""
    x = np.asarray(x)
    if x.size == 0:
        return np.zeros(0, dtype=np.complex128)
    return np.convolve(x.astype(np.complex128), np.asarray(taps, dtype=np.float64))[: x.size]
