"""Generates the golden fixtures under tests/golden/ from the reference's own CPU
receive and transmit path (oracle/_ref/libref.so, compiled from the reference
sources by oracle/Makefile).  Run where the reference tree exists:

    make -C oracle ref && python tests/golden/make_golden.py [fec] [ofdm] [tx]

The fixtures let the CPU and GPU tests check parity on machines without the
reference tree.  Inputs are seeded synthetic data (no dataset is involved).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "sicc-baseband-proto_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from oracle import Reference, ref_root  # noqa: E402
from sicc_gb300 import channel, codes, ofdm  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def fec_fixture(ref: Reference) -> dict:
    code = codes.short_code()
    rc = ref.code(code.n, code.m, code.row_ptr, code.col_ind)
    info_cols, pivot_cols = rc.info_cols()
    parity = rc.systematic_parity()
    rng = np.random.default_rng(7)
    info = rng.integers(0, 2, size=(16, code.k), dtype=np.uint8)
    enc = np.stack([rc.encode(i) for i in info])
    frames = []
    for ebn0, seed in ((1.0, 11), (2.0, 12), (3.0, 13), (4.0, 14)):
        _, _, llr = channel.awgn_llrs(code, 64, ebn0, seed)
        frames.append(llr)
    llr = np.concatenate(frames)
    ok, bits, iters = rc.decode_min_sum(llr, 20, 0.75)
    ok8, bits8, iters8 = rc.decode_min_sum(llr, 8, 0.80)
    # CCSDS (128,64), the reference library's default code
    n, m, rp, ci = ccsds = ccsds_csr()
    rcc = ref.code(n, m, rp, ci)
    cc_parity = rcc.systematic_parity()
    return dict(row_ptr=code.row_ptr, col_ind=code.col_ind, info_cols=info_cols, pivot_cols=pivot_cols,
                parity=parity, info=info, enc=enc, llr=llr, flood_ok=ok.astype(np.uint8), flood_bits=bits,
                flood_iter=iters, flood8_ok=ok8.astype(np.uint8), flood8_bits=bits8, flood8_iter=iters8,
                ccsds_row_ptr=rp, ccsds_col_ind=ci, ccsds_parity=cc_parity)


def ccsds_csr():
    path = os.path.join(ref_root(), "data", "code_matrices", "Code_Matrices_Lib", "LDPC", "CCSDS_ldpc_n128_k64.alist")
    return codes.read_alist(path)


def ofdm_fixture(ref: Reference) -> dict:
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    rp = ref.phy(t)
    rng = np.random.default_rng(21)
    x = (rng.standard_normal(t.nfft) + 1j * rng.standard_normal(t.nfft)).astype(np.complex64)
    fft = ref.fft_shifted(x)
    pts = (rng.standard_normal(64) + 1j * rng.standard_normal(64)).astype(np.complex64) * 0.5
    sig2 = rng.uniform(0.01, 1.0, 64)
    llr = rp.llr_maxlog(pts, sig2, t.bits_per_symbol)
    code = codes.qc_code(4, 8, 16, codes.SHORT_CODE_SEED)  # coded bits per frame are a multiple of 128
    rc = ref.code(code.n, code.m, code.row_ptr, code.col_ind)
    gen = ofdm.FrameGenerator(t, code, seed=5)
    batch = gen.batch(8, snr_db=20.0, cfo_subcarriers=0.1, max_offset=150, rayleigh_taps=6)
    sync = [rp.find_frame_earliest(batch.iq[i][: batch.lengths[i]]) for i in range(8)]
    dec = []
    for i in range(8):
        found, start, _, _, cfo = sync[i]
        if found != 1:
            dec.append(np.zeros(batch.info.shape[1], np.uint8))
            continue
        frame = batch.iq[i][start:start + rp.frame_len]
        bits, _ = rp.decode_frame(rc, frame, cfo, 25, 0.75, batch.noise_var[i])
        dec.append(bits)
    return dict(fft_in=x, fft_out=fft, llr_pts=pts, llr_sig2=sig2, llr_out=llr, iq=batch.iq, lengths=batch.lengths,
                noise_var=batch.noise_var, info=batch.info, offsets=batch.offsets,
                sync=np.array([[s[0], s[1], s[2], s[3], s[4]] for s in sync]), decoded=np.stack(dec))


def tx_fixture(ref: Reference) -> dict:
    """Frames of the reference's own CPU transmitter (build_tx_frame_from_info,
    uhd_ldpc_ofdm_link.cpp:4589-4630: encode, map, pilots, inverse FFT, CP, preamble, peak
    normalisation) for the small PHY and the (128,64) code, whose 16 codewords fill the frame."""
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    rp = ref.phy(t)
    code = codes.short_code()
    rc = ref.code(code.n, code.m, code.row_ptr, code.col_ind)
    blocks = t.coded_bits // code.n
    rng = np.random.default_rng(404)
    info = rng.integers(0, 2, size=(4, blocks * code.k), dtype=np.uint8)
    info[0] = 0  # the all-zero frame: pilots and preamble only carry structure
    frames = np.stack([rp.build_tx_frame(rc, info[i]) for i in range(info.shape[0])])
    used = np.zeros(t.active_sc, np.int32)
    pil = np.zeros(len(t.pilot_symbols), np.int32)
    dat = np.zeros(len(t.data_symbols), np.int32)
    const = np.zeros(1 << t.bits_per_symbol, np.complex64)
    ref.L.ref_phy_tables(rp.h, used, pil, dat, const.view(np.float32))
    return dict(info=info, frames=frames, used_indices=used, pilot_symbols=pil, data_symbols=dat,
                constellation=const)


def main(which=("fec", "ofdm", "tx")):
    ref = Reference()
    if "fec" in which:
        np.savez_compressed(os.path.join(OUT, "fec_short_code.npz"), **fec_fixture(ref))
    if "ofdm" in which:
        np.savez_compressed(os.path.join(OUT, "ofdm_small.npz"), **ofdm_fixture(ref))
    if "tx" in which:
        np.savez_compressed(os.path.join(OUT, "tx_reference_small.npz"), **tx_fixture(ref))
    print("wrote fixtures to", OUT)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]) or ("fec", "ofdm", "tx"))
