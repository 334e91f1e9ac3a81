"""The restated GPU transmitter (oracle/tx_oracle.py), checked on the CPU.

Pins: the generator encoder yields codewords of the code (H c = 0) equal to the
systematic encoder; the accumulator encoder equals its sequential definition
(gpu_ofdm_pipeline.cu:169-214); the QAM map equals the reference constellation
(uhd_ldpc_ofdm_link.cpp:2362-2414 as restated in sicc_gb300.ofdm); the noise
deviates are standard normal; a frame demodulated back by FFT returns its bits;
and frames equal, up to the frame's scale, those of the reference's own CPU
transmitter (tests/golden/tx_reference_small.npz, made by build_tx_frame_from_info,
uhd_ldpc_ofdm_link.cpp:4589-4630).
"""
import os

import numpy as np

import tx_oracle
from sicc_gb300 import codes, ofdm


def _generator(code):
    P = codes.gf2_parity_matrix(code)
    return np.concatenate([np.eye(code.k, dtype=np.uint8), P], axis=1)


def test_generator_encoder_gives_codewords():
    c = codes.short_code()
    G = _generator(c)
    info = np.random.default_rng(1).integers(0, 2, size=(32, c.k), dtype=np.uint8)
    cw = tx_oracle.encode_generator(info, G)
    assert not np.any((c.dense_h().astype(np.int64) @ cw.T.astype(np.int64)) & 1)
    assert np.array_equal(cw, codes.encode(codes.gf2_parity_matrix(c), info))


def test_accumulator_encoder_matches_its_definition():
    rng = np.random.default_rng(2)
    n, k = 96, 40
    m = n - k
    deg = rng.integers(0, 6, size=m)
    offsets = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    cols = rng.integers(0, k, size=int(offsets[-1])).astype(np.int32)
    info = rng.integers(0, 2, size=(5, k), dtype=np.uint8)
    got = tx_oracle.encode_accumulator(info, n, offsets, cols)
    for b in range(5):
        prev = 0
        for r in range(m):
            s = 0
            for q in range(offsets[r], offsets[r + 1]):
                s ^= int(info[b, cols[q]])
            prev = s ^ (prev if r else 0)
            assert got[b, k + r] == prev
        assert np.array_equal(got[b, :k], info[b])


def test_qam_map_equals_the_reference_constellation():
    for bps in (1, 2, 4, 6):
        pts, _ = ofdm.constellation(bps)
        idx = np.arange(1 << bps)
        bits = (idx[:, None] >> (bps - 1 - np.arange(bps))[None, :]) & 1
        assert np.max(np.abs(tx_oracle.qam(bits, bps) - pts)) < 1e-6


def test_noise_deviates_are_standard_normal():
    z = tx_oracle.normal(12345, np.arange(200_000))
    assert abs(z.mean()) < 0.01 and abs(z.var() - 1.0) < 0.02
    assert not np.array_equal(z[:100], tx_oracle.normal(12346, np.arange(100)))


def test_frame_returns_its_bits_through_an_fft():
    cfg = ofdm.OFDM_SMALL
    t = ofdm.reference_tables(cfg)
    coded = np.random.default_rng(3).integers(0, 2, size=(1, t.coded_bits), dtype=np.uint8)
    fr = tx_oracle.tx_frames(coded, nfft=cfg.nfft, cp=cfg.cp, num_symbols=cfg.num_symbols, active_sc=cfg.active_sc,
                             bps=cfg.bits_per_symbol, used_bins=t.used_bins, pilot_symbols=t.pilot_symbols,
                             data_symbols=t.data_symbols, pilot_grid=t.pilot_grid, preamble=t.preamble,
                             amplitude=cfg.amplitude)[0]
    pre = len(t.preamble)
    scale = cfg.amplitude / cfg.nfft
    pts, _ = ofdm.constellation(cfg.bits_per_symbol)
    bits = []
    for sym in t.data_symbols:
        body = fr[pre + sym * (cfg.nfft + cfg.cp) + cfg.cp: pre + (sym + 1) * (cfg.nfft + cfg.cp)]
        y = np.fft.fft(body / scale) / cfg.nfft
        v = y[t.used_bins]
        idx = np.argmin(np.abs(v[:, None] - pts[None, :]), axis=1)
        bits.append(((idx[:, None] >> (cfg.bits_per_symbol - 1 - np.arange(cfg.bits_per_symbol))) & 1).reshape(-1))
    assert np.array_equal(np.concatenate(bits), coded[0])
    assert np.allclose(fr[:pre], t.preamble * cfg.amplitude, atol=1e-6)


GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def reference_tx_fixture():
    return dict(np.load(os.path.join(GOLDEN, "tx_reference_small.npz")))


def scaled_like_reference(frames, amplitude):
    """The reference CPU transmitter normalises each frame to peak `amplitude`; the GPU
    transmitter (gpu_ofdm_pipeline.cu:316-342) scales the preamble by the amplitude and the
    unnormalised inverse FFT by amplitude / nfft.  The two differ by one factor per frame."""
    f = np.asarray(frames, np.complex128)
    return f * (amplitude / np.max(np.abs(f), axis=-1, keepdims=True))


def test_restated_transmitter_matches_the_reference_cpu_transmitter():
    d = reference_tx_fixture()
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    assert np.array_equal(d["used_indices"], t.used_indices)
    assert np.array_equal(d["pilot_symbols"], t.pilot_symbols) and np.array_equal(d["data_symbols"], t.data_symbols)
    assert np.array_equal(d["constellation"], t.constellation)
    c = codes.short_code()
    coded = tx_oracle.encode_generator(d["info"].reshape(-1, c.k), _generator(c)).reshape(d["info"].shape[0], -1)
    cfg = t.cfg
    got = tx_oracle.tx_frames(coded, nfft=cfg.nfft, cp=cfg.cp, num_symbols=cfg.num_symbols, active_sc=cfg.active_sc,
                              bps=cfg.bits_per_symbol, used_bins=t.used_bins, pilot_symbols=t.pilot_symbols,
                              data_symbols=t.data_symbols, pilot_grid=t.pilot_grid, preamble=t.preamble,
                              amplitude=cfg.amplitude)
    ref = d["frames"].astype(np.complex128)
    err = np.max(np.abs(scaled_like_reference(got, cfg.amplitude) - ref))
    assert err <= 2e-6 * cfg.amplitude, err
