"""CPU model of the 1024-channel tensor-core DFT (gpu-rf-pipeline_gb300/csrc/chan_wide.cu).

Restates, in numpy, exactly what the kernel's operands hold: the 64 x 64 real matrix
W = 2^14 [[cos, sin], [-sin, cos]](2 pi k m / 32) with its (K, N) index meaning, the FP16
hi/lo splits of W and of the scaled operands, the three split products summed in float32, the
FP32 twiddle w_1024^(k2 m1) between the stages, the per-frame exponents e1 (from the frame's
largest component) and e2 = e1 - 6, and the output order z[k2 + 32 k1]. Checked against the
float64 inverse DFT (np.fft.ifft * M, the cuFFT CUFFT_INVERSE convention the project uses,
src/channelize.cu:70-71) — the factorization, the index maps and the precision budget
(normwise error <= 2e-6) are pinned without a GPU; the GPU tests then compare the kernel with
the float64 oracle on the same budget.
"""
from __future__ import annotations

import numpy as np
import pytest

M = 1024
R = 32          # radix: m = m1 + 32 m2, k = k2 + 32 k1
W_EXP = 14
NORMWISE = 2e-6


def w_matrix() -> np.ndarray:
    """W[kk][n]: K index kk (Re in for kk < 32, Im in otherwise, input index kk % 32), N index
    n (Re out for n < 32, Im out otherwise, output index n % 32), scaled by 2^14."""
    kk = np.arange(2 * R)[:, None]
    n = np.arange(2 * R)[None, :]
    theta = 2.0 * np.pi * ((n % R) * (kk % R) % R) / R
    c, s = np.cos(theta), np.sin(theta)
    v = np.where(n < R, np.where(kk < R, c, -s), np.where(kk < R, s, c))
    return (v * 2.0 ** W_EXP).astype(np.float32)


def split(v: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """FP16 hi = fp16(v), lo = fp16(v - hi), as the kernel's split2 (float32 v)."""
    v = v.astype(np.float32)
    hi = v.astype(np.float16)
    lo = (v - hi.astype(np.float32)).astype(np.float16)
    return hi, lo


def split_gemm(a: np.ndarray, w_hi: np.ndarray, w_lo: np.ndarray) -> np.ndarray:
    """A (rows x 64, float32, already scaled) times W: a_hi w_hi + a_hi w_lo + a_lo w_hi, each
    product exact and the sum in float32 (the tensor cores' round-toward-zero FP32
    accumulation is modelled as round-to-nearest: the bound below leaves room for both)."""
    a_hi, a_lo = split(a)
    terms = [(a_hi, w_hi), (a_hi, w_lo), (a_lo, w_hi)]
    acc = np.zeros((a.shape[0], 2 * R), np.float32)
    for x, w in terms:
        acc = (acc.astype(np.float64) + x.astype(np.float64) @ w.astype(np.float64)).astype(
            np.float32)
    return acc


def scale_exponent(maxabs: np.ndarray) -> np.ndarray:
    """The kernel's scale_exponent: 2^e brings the magnitude into [2^14, 2^15); 0 for zero;
    clamped to 127 as the kernel does."""
    e = np.zeros(maxabs.shape, np.int64)
    nz = maxabs > 0
    e[nz] = 14 - np.floor(np.log2(maxabs[nz].astype(np.float64))).astype(np.int64)
    return np.minimum(e, 127)


def tensor_core_dft(u: np.ndarray) -> np.ndarray:
    """z (frames x 1024 complex) from u (frames x 1024 complex64) as chan_dft_kernel computes
    it."""
    frames = u.shape[0]
    w = w_matrix()
    w_hi, w_lo = split(w)
    ur = u.real.astype(np.float32)
    ui = u.imag.astype(np.float32)
    maxabs = np.maximum(np.abs(ur), np.abs(ui)).max(axis=1)
    e1 = scale_exponent(maxabs)
    f1 = np.ldexp(np.float32(1), e1).astype(np.float32)[:, None]
    # Stage 1 rows (frame, m1), K = [Re u[m1 + 32 m2], Im u[m1 + 32 m2]] over m2.
    u3r = (ur * f1).reshape(frames, R, R).transpose(0, 2, 1)   # [frame][m1][m2]
    u3i = (ui * f1).reshape(frames, R, R).transpose(0, 2, 1)
    a1 = np.concatenate([u3r, u3i], axis=2).reshape(frames * R, 2 * R)
    d1 = split_gemm(a1, w_hi, w_lo).reshape(frames, R, 2 * R)   # [frame][m1][Re k2 | Im k2]
    # Undo 2^(e1 + 14), twiddle w_1024^(k2 m1) (float32 table from float64), scale by 2^e2.
    s1 = np.ldexp(np.float32(1), -(e1 + W_EXP)).astype(np.float32)[:, None, None]
    re = d1[:, :, :R] * s1
    im = d1[:, :, R:] * s1
    k2 = np.arange(R)[None, :]
    m1 = np.arange(R)[:, None]
    ang = 2.0 * np.pi * (k2 * m1) / M
    tc = np.cos(ang).astype(np.float32)[None]
    ts = np.sin(ang).astype(np.float32)[None]
    e2 = e1 - 6
    f2 = np.ldexp(np.float32(1), e2).astype(np.float32)[:, None, None]
    br = ((re * tc - im * ts) * f2).astype(np.float32)               # [frame][m1][k2]
    bi = ((re * ts + im * tc) * f2).astype(np.float32)
    assert np.max(np.abs(br)) < 2.0 ** 15 and np.max(np.abs(bi)) < 2.0 ** 15
    # Stage 2 rows (frame, k2), K = [Re B[m1][k2], Im B[m1][k2]] over m1.
    a2 = np.concatenate([br.transpose(0, 2, 1), bi.transpose(0, 2, 1)], axis=2)
    d2 = split_gemm(a2.reshape(frames * R, 2 * R), w_hi, w_lo).reshape(frames, R, 2 * R)
    s2 = np.ldexp(np.float32(1), -(e2 + W_EXP)).astype(np.float32)[:, None, None]
    zr = d2[:, :, :R] * s2                                          # [frame][k2][k1]
    zi = d2[:, :, R:] * s2
    # Channel k = k2 + 32 k1.
    z = (zr + 1j * zi.astype(np.float64)).transpose(0, 2, 1).reshape(frames, M)
    return z


def normwise(y: np.ndarray, ref: np.ndarray) -> float:
    return float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))


@pytest.mark.parametrize("kind", ["noise", "tones_60db", "one_channel", "impulse"])
def test_factored_split_dft_matches_the_float64_inverse_dft(kind: str) -> None:
    rng = np.random.default_rng(11)
    frames = 24
    if kind == "noise":
        u = rng.standard_normal((frames, M)) + 1j * rng.standard_normal((frames, M))
    elif kind == "tones_60db":
        t = np.arange(M)
        u = sum(10.0 ** (-3.0 * i / 7) * np.exp(2j * np.pi * (rng.integers(0, M) * t / M
                                                             + rng.random()))
                for i in range(8))[None, :] * (1 + rng.random((frames, 1)))
    elif kind == "one_channel":
        u = np.exp(2j * np.pi * 37 * np.arange(M) / M)[None, :].repeat(frames, axis=0)
    else:
        u = np.zeros((frames, M), complex)
        u[:, 5] = 1e-3
    u = u.astype(np.complex64)
    ref = np.fft.ifft(u.astype(np.complex128), axis=1) * M
    z = tensor_core_dft(u)
    assert normwise(z, ref) <= NORMWISE


def test_frames_at_very_different_levels_keep_their_own_scale() -> None:
    # Per-frame exponents: a frame 2^-40 below its neighbour is exact to the same relative
    # level as the loud one.
    rng = np.random.default_rng(3)
    u = (rng.standard_normal((2, M)) + 1j * rng.standard_normal((2, M))).astype(np.complex64)
    u[1] *= np.float32(2.0 ** -40)
    z = tensor_core_dft(u)
    for f in range(2):
        ref = np.fft.ifft(u[f].astype(np.complex128)) * M
        assert normwise(z[f], ref) <= NORMWISE


def test_silence_is_exact_zero() -> None:
    assert not np.any(tensor_core_dft(np.zeros((3, M), np.complex64)))


def test_output_order_is_k2_plus_32_k1() -> None:
    # The inverse DFT of e^{2 pi i 24 m / M} is M at channel k = -24 mod M = 1000 = 8 + 32 * 31
    # (k2 = 8, k1 = 31): both digits non-trivial, so a swapped order would put it elsewhere.
    u = np.exp(2j * np.pi * 24 * np.arange(M) / M).astype(np.complex64)[None, :]
    z = tensor_core_dft(u)
    assert int(np.argmax(np.abs(z[0]))) == 1000
    assert abs(abs(z[0, 1000]) - M) < 1e-3
