"""OFDM frame tables and a seeded synthetic transmitter + channel.

Tables follow the reference PHY configuration (source/cpp_cuda/uhd_cpp/src/
uhd_ldpc_ofdm_link.cpp): active subcarriers on the shifted grid
[n/2 - a/2, n/2 - 1] U [n/2 + 1, n/2 + a/2] (:4020-4027), pilot OFDM symbols
every ``pilot_period`` symbols (:3999-4004), linear interpolation of the pilot
channel estimates between the surrounding pilot symbols (:5401-5427), Gray
square QAM with bits MSB-first, scaled to unit average power (:2362-2414), and
a random-QPSK preamble made of two identical halves, RMS-normalised
(:3861-3880).  The preamble and pilot symbols are drawn here from NumPy PCG64
generators (the reference draws them from mt19937); the receiver takes them as
tables either way.

The transmitter builds frames as the reference does (:4589-4630): encode, map,
insert pilots, inverse FFT of the shifted grid, cyclic prefix, preamble, peak
normalisation.  The channel is a tapped-delay-line Rayleigh fading channel with
an exponential power-delay profile, a carrier frequency offset, an integer
timing offset (noise-only samples before the frame) and AWGN at a given SNR.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np

from .codes import QcCode
from .channel import parity_matrix
from .codes import encode


@dataclass(frozen=True)
class PhyConfig:
    nfft: int = 1024
    cp: int = 72
    num_symbols: int = 14
    active_sc: int = 600
    pre_half_len: int = 512
    modulation: str = "16qam"
    pilot_period: int = 14
    sample_rate: float = 15.36e6
    sync_threshold: float = 0.45
    amplitude: float = 0.70
    preamble_seed: int = 11
    pilot_seed: int = 73

    @property
    def bits_per_symbol(self) -> int:
        return {"bpsk": 1, "qpsk": 2, "16qam": 4, "64qam": 6}[self.modulation]


#: The OFDM receive workload: 14 symbols of 1024 + CP 72, 600 active
#: subcarriers, pilot symbol 0, 16-QAM.
OFDM_C3 = PhyConfig()
#: A small configuration used by fixtures and CPU tests (2048 coded bits/frame).
OFDM_SMALL = PhyConfig(nfft=256, cp=16, num_symbols=6, active_sc=128, pre_half_len=128, pilot_period=3)


@dataclass
class Tables:
    cfg: PhyConfig
    used_indices: np.ndarray       # shifted-grid index of each active subcarrier
    used_bins: np.ndarray          # natural FFT bin of each active subcarrier
    pilot_symbols: np.ndarray
    data_symbols: np.ndarray
    interp_p0: np.ndarray
    interp_p1: np.ndarray
    interp_alpha: np.ndarray
    preamble: np.ndarray           # complex64 [2L]
    pilot_grid: np.ndarray         # complex64 [pilots][active_sc]
    constellation: np.ndarray      # complex64 [2^bps], index bits MSB-first
    axis_levels: np.ndarray        # float32 [2^(bps/2)] amplitude by Gray axis index

    # flat accessors used by the oracle/reference wrappers
    def __getattr__(self, name):
        cfg = self.__dict__.get("cfg")
        if cfg is not None and hasattr(cfg, name):
            return getattr(cfg, name)
        raise AttributeError(name)

    @property
    def coded_bits(self) -> int:
        return len(self.data_symbols) * self.cfg.active_sc * self.cfg.bits_per_symbol

    @property
    def frame_len(self) -> int:
        return 2 * self.cfg.pre_half_len + self.cfg.num_symbols * (self.cfg.nfft + self.cfg.cp)


def _gray_to_binary(g: int) -> int:
    b = 0
    while g:
        b ^= g
        g >>= 1
    return b


def constellation(bps: int) -> tuple[np.ndarray, np.ndarray]:
    """Constellation [2^bps] (index bits MSB-first) and per-axis levels, float32 as the reference."""
    if bps == 1:
        return np.array([1, -1], np.complex64), np.array([1, -1], np.float32)
    if bps == 2:
        s = np.float32(1.0 / np.sqrt(2.0))
        pts = np.array([complex(s if b0 == 0 else -s, s if b1 == 0 else -s)
                        for b0 in (0, 1) for b1 in (0, 1)], np.complex64)
        return pts, np.array([s, -s], np.float32)
    axis = bps // 2
    levels = 1 << axis
    m = 1 << bps
    raw = []
    for idx in range(m):
        gi, gq = idx >> axis, idx & (levels - 1)
        raw.append(((levels - 1) - 2 * _gray_to_binary(gi), (levels - 1) - 2 * _gray_to_binary(gq)))
    avg = sum(float(i * i + q * q) for i, q in raw) / m
    scale = np.float32(1.0 / np.sqrt(avg))
    pts = np.array([complex(np.float32(i) * scale, np.float32(q) * scale) for i, q in raw], np.complex64)
    lv = np.array([np.float32((levels - 1) - 2 * _gray_to_binary(g)) * scale for g in range(levels)], np.float32)
    return pts, lv


def _qpsk(bits: np.ndarray) -> np.ndarray:
    s = np.float32(1.0 / np.sqrt(2.0))
    b = bits.reshape(-1, 2)
    return (np.where(b[:, 0] == 0, s, -s) + 1j * np.where(b[:, 1] == 0, s, -s)).astype(np.complex64)


def reference_tables(cfg: PhyConfig) -> Tables:
    n2, a2 = cfg.nfft // 2, cfg.active_sc // 2
    used = np.array(list(range(n2 - a2, n2)) + list(range(n2 + 1, n2 + a2 + 1)), np.int32)
    bins = ((used + cfg.nfft // 2) % cfg.nfft).astype(np.int32)
    if cfg.pilot_period > 0:
        pilots = np.arange(0, cfg.num_symbols, cfg.pilot_period, dtype=np.int32)
    else:
        pilots = np.unique(np.array([0, cfg.num_symbols // 3, 2 * cfg.num_symbols // 3], np.int32))
    data = np.array([s for s in range(cfg.num_symbols) if s not in set(pilots.tolist())], np.int32)
    p0 = np.zeros(len(data), np.int32)
    p1 = np.zeros(len(data), np.int32)
    al = np.zeros(len(data), np.float32)
    P = len(pilots)
    for i, sym in enumerate(data):
        hi = 0
        while hi + 1 < P and sym > pilots[hi + 1]:
            hi += 1
        a, b = hi, min(hi + 1, P - 1)
        if sym <= pilots[0]:
            a = b = 0
        elif sym >= pilots[-1]:
            a = b = P - 1
        alpha = 0.0 if a == b else (sym - pilots[a]) / (pilots[b] - pilots[a])
        p0[i], p1[i], al[i] = a, b, np.float32(alpha)
    rng = np.random.default_rng(cfg.preamble_seed)
    half = _qpsk(rng.integers(0, 2, 2 * cfg.pre_half_len).astype(np.uint8))[: cfg.pre_half_len]
    pre = np.concatenate([half, half]).astype(np.complex64)
    rms = np.sqrt(np.mean(np.abs(pre.astype(np.complex128)) ** 2))
    pre = (pre / np.float32(rms)).astype(np.complex64)
    prng = np.random.default_rng(cfg.pilot_seed)
    grid = _qpsk(prng.integers(0, 2, 2 * cfg.active_sc * P).astype(np.uint8)).reshape(P, cfg.active_sc)
    pts, lv = constellation(cfg.bits_per_symbol)
    return Tables(cfg, used, bins, pilots, data, p0, p1, al, pre, grid, pts, lv)


@dataclass
class FrameBatch:
    iq: np.ndarray          # complex64 [F][max_len] (zero padded)
    lengths: np.ndarray     # int32 [F]
    info: np.ndarray        # uint8 [F][blocks*k]
    coded: np.ndarray       # uint8 [F][coded_bits]
    noise_var: np.ndarray   # float64 [F] frequency-domain noise variance (per FFT bin)
    offsets: np.ndarray     # int32 [F] true frame start
    cfo_hz: float = 0.0


@dataclass
class FrameGenerator:
    tables: Tables
    code: QcCode
    seed: int = 1
    _rng: np.random.Generator = field(init=False, repr=False)

    def __post_init__(self):
        self._rng = np.random.default_rng(self.seed)

    @property
    def blocks(self) -> int:
        return self.tables.coded_bits // self.code.n

    def modulate(self, coded: np.ndarray) -> np.ndarray:
        t, cfg = self.tables, self.tables.cfg
        bps = cfg.bits_per_symbol
        idx = np.zeros(coded.size // bps, np.int64)
        for b in range(bps):
            idx = (idx << 1) | coded.reshape(-1, bps)[:, b]
        syms = t.constellation[idx].reshape(len(t.data_symbols), cfg.active_sc)
        out = [t.preamble]
        pil = {int(s): i for i, s in enumerate(t.pilot_symbols)}
        dcol = 0
        for sym in range(cfg.num_symbols):
            grid = np.zeros(cfg.nfft, np.complex128)
            if sym in pil:
                grid[t.used_indices] = t.pilot_grid[pil[sym]]
            else:
                grid[t.used_indices] = syms[dcol]
                dcol += 1
            natural = grid[(np.arange(cfg.nfft) + cfg.nfft // 2) % cfg.nfft]
            td = np.fft.ifft(natural).astype(np.complex64)
            out += [td[-cfg.cp:], td]
        frame = np.concatenate(out)
        scale = np.float32(cfg.amplitude) / np.float32(max(np.abs(frame).max(), 1e-12))
        return (frame * scale).astype(np.complex64)

    def batch(self, frames: int, snr_db: float, cfo_subcarriers: float = 0.0, max_offset: int = 0,
              rayleigh_taps: int = 0, decay_db_per_tap: float = 3.0, tail: int = 64) -> FrameBatch:
        t, cfg, rng = self.tables, self.tables.cfg, self._rng
        P = parity_matrix(self.code)
        blocks = self.blocks
        flen = t.frame_len
        max_len = max_offset + flen + tail
        iq = np.zeros((frames, max_len), np.complex64)
        info = rng.integers(0, 2, size=(frames, blocks * self.code.k), dtype=np.uint8)
        coded = np.zeros((frames, t.coded_bits), np.uint8)
        nv = np.zeros(frames)
        offs = np.zeros(frames, np.int32)
        cfo = cfo_subcarriers * cfg.sample_rate / cfg.nfft
        for f in range(frames):
            cw = encode(P, info[f].reshape(blocks, self.code.k)).reshape(-1)
            fill = rng.integers(0, 2, size=t.coded_bits - cw.size, dtype=np.uint8)
            coded[f] = np.concatenate([cw, fill])
            tx = self.modulate(coded[f])
            x = tx.astype(np.complex128)
            if rayleigh_taps > 0:
                p = 10.0 ** (-decay_db_per_tap * np.arange(rayleigh_taps) / 10.0)
                p /= p.sum()
                h = np.sqrt(p / 2) * (rng.standard_normal(rayleigh_taps) + 1j * rng.standard_normal(rayleigh_taps))
                x = np.convolve(x, h)[:flen + rayleigh_taps - 1]
            off = int(rng.integers(0, max_offset + 1)) if max_offset > 0 else 0
            # SNR per active subcarrier, as uhd_ldpc_ofdm_link.cpp:4843-4862 / 10525-10540
            # (the fading taps have unit average power, so it is also the mean received SNR)
            freq_noise = active_subcarrier_power(tx, t) / 10.0 ** (snr_db / 10.0)
            sigma2 = freq_noise / cfg.nfft
            y = np.zeros(max_len, np.complex128)
            y[off:off + x.size] = x
            n = np.arange(max_len)
            y = y * np.exp(2j * np.pi * cfo * (n - off) / cfg.sample_rate)
            y += np.sqrt(sigma2 / 2) * (rng.standard_normal(max_len) + 1j * rng.standard_normal(max_len))
            iq[f] = y.astype(np.complex64)
            nv[f] = freq_noise
            offs[f] = off
        return FrameBatch(iq=iq, lengths=np.full(frames, max_len, np.int32), info=info, coded=coded,
                          noise_var=nv, offsets=offs, cfo_hz=cfo)


def active_subcarrier_power(frame: np.ndarray, t: Tables) -> float:
    """Mean |Y|^2 over the active subcarriers of every OFDM symbol of a frame."""
    cfg = t.cfg
    off = 2 * cfg.pre_half_len
    acc, cnt = 0.0, 0
    for _ in range(cfg.num_symbols):
        body = frame[off + cfg.cp: off + cfg.cp + cfg.nfft].astype(np.complex128)
        nat = np.fft.fft(body)
        acc += float(np.sum(np.abs(nat[t.used_bins]) ** 2))
        cnt += cfg.active_sc
        off += cfg.nfft + cfg.cp
    return acc / max(cnt, 1)


def with_cfg(cfg: PhyConfig, **kw) -> PhyConfig:
    return replace(cfg, **kw)
