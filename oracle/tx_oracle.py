"""Restatement of the reference's GPU transmit chain.

TEST INFRASTRUCTURE ONLY: imported by tests/ (and bench.py's CPU-baseline leg)
as the checker of the GB300 TX kernels, never as a path of the product.

Follows source/cpp_cuda/uhd_cpp/src/gpu_ofdm_pipeline.cu:
  * generator encoder ``ldpc_encode_generator_kernel`` (:129-150): c = u G mod 2;
  * accumulator encoder (:152-214): systematic copy, each parity row's sum of
    its information columns, then parity[r] = sum[r] ^ parity[r-1];
  * resource grid ``fill_resource_grid_kernel`` (:216-257): pilot symbols from
    the pilot grid, data symbols by ``qam_from_bits_dev`` (:84-109) from the
    coded bits (bits past the coded bits are zero filler here), optional
    precompensation value * conj(h) / max(|h|^2, 1e-10);
  * channel and noise ``apply_actual_channel_and_frequency_awgn_kernel``
    (:282-314): value * actual_h, plus sigma * (n1 + i n2) on data symbols,
    sigma = sqrt(var / 2), n from the hashed Box-Muller deviates of :259-280;
  * unnormalised inverse FFT of each symbol's grid (cuFFT inverse, :1032);
  * ``compose_tx_frame_kernel`` (:316-342): preamble * amplitude, then each
    symbol with its cyclic prefix, scaled by amplitude / nfft.
Single-precision steps are done in float32 where the kernels do; the inverse
FFT is numpy's (double precision), so frames agree with the GPU within a
floating-point tolerance, not bit for bit.
"""
from __future__ import annotations

import numpy as np

_PI_F = np.float32(3.14159265358979323846)


def encode_generator(info: np.ndarray, generator_kn: np.ndarray) -> np.ndarray:
    """info [codewords][k] (0/1) -> coded [codewords][n]."""
    u = np.asarray(info, np.int64) & 1
    g = np.asarray(generator_kn, np.int64) & 1
    return ((u @ g) & 1).astype(np.uint8)


def encode_accumulator(info: np.ndarray, n: int, offsets: np.ndarray, cols: np.ndarray) -> np.ndarray:
    u = np.asarray(info, np.uint8) & 1
    cw, k = u.shape
    m = n - k
    out = np.zeros((cw, n), np.uint8)
    out[:, :k] = u
    sums = np.zeros((cw, m), np.uint8)
    for r in range(m):
        c = np.asarray(cols[offsets[r]:offsets[r + 1]], np.int64)
        if c.size:
            sums[:, r] = np.bitwise_xor.reduce(u[:, c], axis=1)
    out[:, k:] = np.bitwise_xor.accumulate(sums, axis=1)
    return out


def _gray_to_binary(g: np.ndarray) -> np.ndarray:
    b = np.zeros_like(g)
    g = g.copy()
    while np.any(g):
        b ^= g
        g >>= 1
    return b


def qam(bits: np.ndarray, bps: int) -> np.ndarray:
    """bits [..., bps] -> complex64 symbols, as qam_from_bits_dev."""
    b = np.asarray(bits, np.int64) & 1
    if bps == 1:
        return np.where(b[..., 0] != 0, -1.0, 1.0).astype(np.float32).astype(np.complex64)
    if bps == 2:
        s = np.float32(0.7071067811865475)
        re = np.where(b[..., 0] != 0, -s, s).astype(np.float32)
        im = np.where(b[..., 1] != 0, -s, s).astype(np.float32)
        return (re + 1j * im).astype(np.complex64)
    ab = bps // 2
    levels = 1 << ab
    gi = np.zeros(b.shape[:-1], np.int64)
    gq = np.zeros(b.shape[:-1], np.int64)
    for i in range(ab):
        gi = (gi << 1) | b[..., i]
        gq = (gq << 1) | b[..., ab + i]
    scale = np.float32(0.3162277660168379 if bps == 4 else 0.1543033499620919)
    re = ((levels - 1) - 2 * _gray_to_binary(gi)).astype(np.float32) * scale
    im = ((levels - 1) - 2 * _gray_to_binary(gq)).astype(np.float32) * scale
    return (re + 1j * im).astype(np.complex64)


def _hash32(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint32)
    x ^= x >> np.uint32(16)
    x = (x * np.uint32(0x7FEB352D)).astype(np.uint32)
    x ^= x >> np.uint32(15)
    x = (x * np.uint32(0x846CA68B)).astype(np.uint32)
    x ^= x >> np.uint32(16)
    return x


def _uniform(seed: int, idx: np.ndarray) -> np.ndarray:
    h = _hash32(np.uint32(seed) ^ (idx.astype(np.uint32) * np.uint32(0x9E3779B9)).astype(np.uint32))
    return ((h.astype(np.float32) + np.float32(1.0)) * np.float32(2.3283064365386963e-10)).astype(np.float32)


def normal(seed: int, idx: np.ndarray) -> np.ndarray:
    idx = np.asarray(idx, np.uint32)
    with np.errstate(over="ignore"):
        u1 = np.maximum(_uniform(seed, (idx * np.uint32(2)).astype(np.uint32)), np.float32(1e-7))
        u2 = _uniform(seed, (idx * np.uint32(2) + np.uint32(1)).astype(np.uint32))
    return (np.sqrt(np.float64(-2.0) * np.log(u1.astype(np.float64)))
            * np.cos(np.float64(2.0 * _PI_F) * u2.astype(np.float64)))


def frame_seed(noise_seed: int) -> int:
    s = int(noise_seed) & 0xFFFFFFFFFFFFFFFF
    return (s ^ (s >> 32)) & 0xFFFFFFFF


def tx_frames(coded: np.ndarray, *, nfft: int, cp: int, num_symbols: int, active_sc: int, bps: int,
              used_bins: np.ndarray, pilot_symbols: np.ndarray, data_symbols: np.ndarray,
              pilot_grid: np.ndarray, preamble: np.ndarray, amplitude: float,
              precomp_h: np.ndarray | None = None, actual_h: np.ndarray | None = None,
              noise_var: float = 0.0, noise_seed: int = 0) -> np.ndarray:
    """coded [frames][coded_bits] -> complex128 frames [frames][pre + num_symbols * (nfft + cp)].

    Frame f's noise is seeded with noise_seed + f (as the batched GPU entry point)."""
    coded = np.asarray(coded, np.uint8)
    frames, cb = coded.shape
    pre = len(preamble)
    sym_len = nfft + cp
    out = np.zeros((frames, pre + num_symbols * sym_len), np.complex128)
    pil_of = {int(s): q for q, s in enumerate(pilot_symbols)}
    dat_of = {int(s): d for d, s in enumerate(data_symbols)}
    amp = np.float32(amplitude)
    scale = np.float32(amp / np.float32(nfft))
    sigma = np.float64(np.sqrt(np.float32(max(noise_var, 0.0)) * np.float32(0.5)))
    for f in range(frames):
        out[f, :pre] = (np.asarray(preamble, np.complex64) * amp).astype(np.complex64)
        seed = frame_seed(noise_seed + f)
        for sym in range(num_symbols):
            vals = np.zeros(active_sc, np.complex128)
            if sym in pil_of:
                vals[:] = np.asarray(pilot_grid, np.complex64)[pil_of[sym]]
            elif sym in dat_of:
                d = dat_of[sym]
                idx = (d * active_sc + np.arange(active_sc))[:, None] * bps + np.arange(bps)[None, :]
                bits = np.where(idx < cb, coded[f, np.minimum(idx, cb - 1)], 0)
                vals[:] = qam(bits, bps)
            re_idx = sym * active_sc + np.arange(active_sc)
            if precomp_h is not None:
                h = np.asarray(precomp_h, np.complex64).reshape(-1)[re_idx].astype(np.complex128)
                vals = vals * np.conj(h) / np.maximum(np.abs(h) ** 2, 1e-10)
            if actual_h is not None:
                vals = vals * np.asarray(actual_h, np.complex64).reshape(-1)[re_idx]
            if noise_var > 0.0 and sym in dat_of:
                vals = vals + sigma * (normal(seed, re_idx) + 1j * normal(seed ^ 0xA5A5A5A5, re_idx))
            grid = np.zeros(nfft, np.complex128)
            grid[np.asarray(used_bins)] = vals
            y = np.fft.ifft(grid) * nfft  # unnormalised inverse
            body = np.concatenate([y[nfft - cp:], y]) * np.float64(scale)
            out[f, pre + sym * sym_len: pre + (sym + 1) * sym_len] = body
    return out
