"""The GB300 transmit chain against the reference's CPU transmitter, the restated
GPU transmitter, and TX -> RX.

The oracle (oracle/tx_oracle.py) restates gpu_ofdm_pipeline.cu:129-343 and
922-1075.  The coded bits must be identical (a wrong bit moves a QAM point by
at least one constellation step, far above the tolerance); the frame samples
agree within 2e-5 of the frame's peak (the GPU inverse FFT is single
precision, the oracle's double).  The round trip sends frames through the
receive chain (sync, demodulation, BP), which must return the information
bits exactly.
"""
import numpy as np
import pytest

import tx_oracle
from sicc_gb300 import codes, fec, ofdm
from sicc_gb300.pipeline import RxPipeline

pytestmark = pytest.mark.gpu


def _gen(code):
    return np.ascontiguousarray(np.concatenate([np.eye(code.k, dtype=np.uint8), codes.gf2_parity_matrix(code)], 1))


def _kw(t):
    cfg = t.cfg
    return dict(nfft=cfg.nfft, cp=cfg.cp, num_symbols=cfg.num_symbols, active_sc=cfg.active_sc,
                bps=cfg.bits_per_symbol, used_bins=t.used_bins, pilot_symbols=t.pilot_symbols,
                data_symbols=t.data_symbols, pilot_grid=t.pilot_grid, preamble=t.preamble, amplitude=cfg.amplitude)


def _pipe(cfg, code, **kw):
    t = ofdm.reference_tables(cfg)
    blocks = t.coded_bits // code.n
    return RxPipeline(t, code.n, code.k, blocks, 1e-3, slots=2, **kw), t, blocks


def _close(got, ref, what):
    assert got.shape == ref.shape
    err = np.max(np.abs(got - ref))
    assert err <= 2e-5 * np.max(np.abs(ref)), (what, err)


def test_tx_frames_match_the_reference_cpu_transmitter(cuda):
    """Pinned to the reference itself: frames of its CPU transmitter (build_tx_frame_from_info,
    uhd_ldpc_ofdm_link.cpp:4589-4630, tests/golden/tx_reference_small.npz) equal the GPU frames up
    to the frame's scale (the reference normalises each frame to peak amplitude, the GPU
    transmitter scales by the amplitude as gpu_ofdm_pipeline.cu:316-342 does), within 2e-5 of the
    peak (single-precision inverse FFT on the GPU, double precision in the reference)."""
    from test_tx_oracle import reference_tx_fixture, scaled_like_reference
    torch = cuda
    d = reference_tx_fixture()
    code = codes.short_code()
    p, t, blocks = _pipe(ofdm.OFDM_SMALL, code)
    p.upload_tx_tables(generator_kn=_gen(code))
    F = d["info"].shape[0]
    d_fr = torch.zeros((F, t.frame_len), dtype=torch.complex64, device="cuda")
    p.tx_batch(torch.from_numpy(d["info"]).cuda(), F, d_fr, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    got = scaled_like_reference(d_fr.cpu().numpy(), t.cfg.amplitude)
    err = np.max(np.abs(got - d["frames"].astype(np.complex128)))
    assert err <= 2e-5 * t.cfg.amplitude, err


def test_tx_frames_match_the_restated_transmitter(cuda):
    torch = cuda
    code = codes.short_code()
    p, t, blocks = _pipe(ofdm.OFDM_SMALL, code)
    G = _gen(code)
    p.upload_tx_tables(generator_kn=G)
    F = 5
    info = np.random.default_rng(1).integers(0, 2, size=(F, blocks * code.k), dtype=np.uint8)
    coded = tx_oracle.encode_generator(info.reshape(-1, code.k), G).reshape(F, -1)
    d_info = torch.from_numpy(info).cuda()
    d_fr = torch.zeros((F, t.frame_len), dtype=torch.complex64, device="cuda")
    p.tx_batch(d_info, F, d_fr, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    ref = tx_oracle.tx_frames(coded, **_kw(t))
    _close(d_fr.cpu().numpy(), ref, "batch")
    _close(p.tx_frame(1, info[2]), ref[2], "slot")  # submit_tx_frame_async + synchronize_tx


def test_tx_channel_precompensation_and_noise(cuda):
    torch = cuda
    code = codes.short_code()
    p, t, blocks = _pipe(ofdm.OFDM_SMALL, code)
    cfg = t.cfg
    rng = np.random.default_rng(2)
    re = cfg.num_symbols * cfg.active_sc
    pre_h = (rng.standard_normal(re) + 1j * rng.standard_normal(re)).astype(np.complex64)
    act_h = (rng.standard_normal(re) + 1j * rng.standard_normal(re)).astype(np.complex64)
    G = _gen(code)
    p.upload_tx_tables(generator_kn=G, precomp_h=pre_h, actual_h=act_h)
    F = 3
    info = rng.integers(0, 2, size=(F, blocks * code.k), dtype=np.uint8)
    coded = tx_oracle.encode_generator(info.reshape(-1, code.k), G).reshape(F, -1)
    d_fr = torch.zeros((F, t.frame_len), dtype=torch.complex64, device="cuda")
    p.tx_batch(torch.from_numpy(info).cuda(), F, d_fr, noise_var=0.05, seed=77, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    ref = tx_oracle.tx_frames(coded, **_kw(t), precomp_h=pre_h, actual_h=act_h, noise_var=0.05, noise_seed=77)
    _close(d_fr.cpu().numpy(), ref, "channel+noise")
    # without noise the two channel tables alone
    p.tx_batch(torch.from_numpy(info).cuda(), F, d_fr, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    _close(d_fr.cpu().numpy(), tx_oracle.tx_frames(coded, **_kw(t), precomp_h=pre_h, actual_h=act_h), "channel")


def test_tx_accumulator_encoder(cuda):
    torch = cuda
    code = codes.short_code()
    p, t, blocks = _pipe(ofdm.OFDM_SMALL, code)
    rng = np.random.default_rng(3)
    m = code.n - code.k
    deg = rng.integers(1, 7, size=m)
    offsets = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    cols = rng.integers(0, code.k, size=int(offsets[-1])).astype(np.int32)
    p.upload_tx_tables(accumulator=(offsets, cols))
    F = 2
    info = rng.integers(0, 2, size=(F, blocks * code.k), dtype=np.uint8)
    coded = tx_oracle.encode_accumulator(info.reshape(-1, code.k), code.n, offsets, cols).reshape(F, -1)
    d_fr = torch.zeros((F, t.frame_len), dtype=torch.complex64, device="cuda")
    p.tx_batch(torch.from_numpy(info).cuda(), F, d_fr, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    _close(d_fr.cpu().numpy(), tx_oracle.tx_frames(coded, **_kw(t)), "accumulator")


def test_tx_then_rx_returns_the_information_bits(cuda):
    """OFDM receive workload's PHY and (1024,512) code: frames from the GPU transmitter decode to their bits."""
    torch = cuda
    code = codes.ofdm_code()
    p, t, blocks = _pipe(ofdm.OFDM_C3, code, max_batch_frames=8)
    p.upload_tx_tables(generator_kn=_gen(code))
    F = 6
    info = np.random.default_rng(4).integers(0, 2, size=(F, blocks * code.k), dtype=np.uint8)
    st = torch.cuda.current_stream()
    d_fr = torch.zeros((F, t.frame_len), dtype=torch.complex64, device="cuda")
    p.tx_batch(torch.from_numpy(info).cuda(), F, d_fr, stream=st)
    d_llr = torch.zeros((F, blocks * code.n), dtype=torch.float32, device="cuda")
    d_sync = torch.zeros(F * 6, dtype=torch.int32, device="cuda")
    p.demod_batch(d_fr, t.frame_len, t.frame_len, F, d_llr, d_sync, stream=st)
    torch.cuda.synchronize()
    sync = d_sync.cpu().numpy().reshape(F, 6)
    assert np.all(sync[:, 0] == 1) and np.all(sync[:, 1] == 0)  # found, at the first sample
    dec = fec.CsrBpDecoder.for_code(code, max_batch=F * blocks)
    bits, ok, _ = dec.decode(d_llr.reshape(F * blocks, code.n), device=True)
    assert np.all(ok == 1)
    assert np.array_equal(bits[:, : code.k].reshape(F, -1), info)
