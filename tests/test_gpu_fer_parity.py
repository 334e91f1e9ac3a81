"""Same-frame error-rate parity of the GPU decoders against the reference's decoder.

Every comparison decodes IDENTICAL seeded frames on both sides.

Reference decoders (restated in the oracle, pinned to the reference's own code):
  * BP + OSD: cpu_bp_osd_decode.m (MB:55-62) -- flooding normalized min-sum
    with the operations of uhd_ldpc_ofdm_link.cpp:3013-3094 (no damping, no
    offset at these configs), OSD order 2 on the lowest-syndrome-weight
    posterior (MB:160-171) when the syndrome fails;
  * plain BP: ldpc_decode_min_sum (L:3013-3094);
  * OFDM receive: the reference CPU receiver's sync (L:5214-5329) and demod
    (L:5331-5521) restated bit-exactly, then BP of every codeword.

Checks, per Eb/N0 (or SNR) point:
  * the GPU flooding schedule equals the reference decoder bit for bit on
    every frame, so its FER and BER are the reference's exactly;
  * the GPU layered schedule (the configs' schedule) is bit-exact with its
    oracle, and its FER and BER are not above the upper end of the reference's
    95% interval (Wilson for FER; frames as the sampling unit for BER).  The
    layered schedule converges faster than flooding within the same iteration
    cap, so at 65,536 frames its FER can fall below the reference's interval;
    the test reports where it falls and the paired (McNemar) comparison;
  * OFDM: the GPU chain (single precision) and the reference chain (double
    precision) find the same frames at the same starts, and their codeword
    and frame error rates lie inside each other's 95% intervals.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

from sicc_gb300 import channel, codes, errstats

pytestmark = pytest.mark.gpu

C2_FRAMES = 65536
C1_FRAMES = 1024


@pytest.fixture(scope="module")
def pool():
    p = mp.get_context("spawn").Pool(os.cpu_count() or 1)
    yield p
    p.close()
    p.join()


def _stream_decode(torch, code, llr, schedule):
    from sicc_gb300 import fec
    B = llr.shape[0]
    dec = fec.StreamBpOsdDecoder(code, max_batch=B, max_iter=20, normalization=0.75, offset=0.0, damping=0.0,
                                 min_abs_llr_accept=0.0, schedule=schedule, osd_order=2, osd_max_flip=64,
                                 osd_max_tests=4096)
    d_info = torch.zeros((B, code.k), dtype=torch.uint8, device="cuda")
    d_used = torch.zeros(B, dtype=torch.uint8, device="cuda")
    dec.decode_device_batch(torch.from_numpy(llr).cuda(), d_info, None, d_used, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    out = d_info.cpu().numpy(), d_used.cpu().numpy()
    dec.close()
    return out


def _report(name, ref, got, fail_ref, fail_got):
    pair = errstats.mcnemar(fail_got, fail_ref)
    side = "inside" if errstats.inside(got["fer"], ref["fer_ci95"]) else (
        "below" if got["fer"] < ref["fer_ci95"][0] else "above")
    print(f"{name}: reference FER {ref['fer']:.5f} {np.round(ref['fer_ci95'], 5).tolist()} "
          f"BER {ref['ber']:.6f}; GPU layered FER {got['fer']:.5f} ({side}) BER {got['ber']:.6f}; "
          f"frames only GPU fails {pair['only_a']}, only reference fails {pair['only_b']}, p={pair['p_value']:.3g}")


@pytest.mark.parametrize("ebn0,seed", [(2.0, 1200), (3.0, 1300)])
def test_c2_bp_osd_fer_parity(cuda, oracle, pool, ebn0, seed):
    """C2: (128,64), 65,536 frames, order-2 OSD on syndrome failures (the bench's first batch)."""
    from oracle import bp_osd_parallel
    torch = cuda
    code = codes.short_code()
    info, _, llr = channel.awgn_llrs(code, C2_FRAMES, ebn0, seed=seed)
    kw = dict(max_iter=20, alpha=0.75, osd_order=2, osd_max_flip=64, osd_max_tests=4096)
    _, ref_info, ref_used = bp_osd_parallel(pool, code, llr, schedule=0, **kw)
    _, lay_oracle, lay_oracle_used = bp_osd_parallel(pool, code, llr, schedule=3, **kw)

    fl_info, fl_used = _stream_decode(torch, code, llr, 0)
    bad = np.flatnonzero(np.any(fl_info != ref_info, axis=1) | (fl_used != ref_used))
    assert bad.size == 0, f"flooding + OSD differs from the reference on {bad.size} frames, first {bad[:5]}"

    lay_info, lay_used = _stream_decode(torch, code, llr, 3)
    bad = np.flatnonzero(np.any(lay_info != lay_oracle, axis=1) | (lay_used != lay_oracle_used))
    assert bad.size == 0, f"layered + OSD differs from its oracle on {bad.size} frames, first {bad[:5]}"

    ref = errstats.rate_summary(ref_info, info)
    got = errstats.rate_summary(lay_info, info)
    _report(f"C2 {ebn0:g} dB", ref, got, errstats.frame_errors(ref_info, info) > 0,
            errstats.frame_errors(lay_info, info) > 0)
    assert got["fer"] <= ref["fer_ci95"][1], (got["fer"], ref["fer_ci95"])
    assert got["ber"] <= ref["ber_ci95"][1], (got["ber"], ref["ber_ci95"])


def test_c1_plain_bp_fer_parity(cuda, oracle):
    """C1: plain BP on (128,64), 1,024 frames at each of 1, 2, 3, 4 dB."""
    from sicc_gb300 import fec
    torch = cuda
    code = codes.short_code()
    oc = oracle.code(code.n, code.m, code.row_ptr, code.col_ind)
    for i, ebn0 in enumerate((1.0, 2.0, 3.0, 4.0)):
        info, _, llr = channel.awgn_llrs(code, C1_FRAMES, ebn0, seed=4100 + i)
        ref = np.stack([oc.flooding_ref(x, 20, 0.75)[1] for x in llr])
        lay_o = np.stack([oc.layered(x, 20, 0.75)[1] for x in llr])
        out = {}
        for sched in (fec.FLOODING, fec.FLAT_LAYERED):
            dec = fec.CsrBpDecoder.for_code(code, max_batch=C1_FRAMES, max_iter=20, normalization=0.75,
                                            schedule=sched)
            bits = torch.zeros((C1_FRAMES, code.n), dtype=torch.uint8, device="cuda")
            dec.decode_device_batch(torch.from_numpy(llr).cuda(), bits, stream=torch.cuda.current_stream())
            torch.cuda.synchronize()
            out[sched] = bits.cpu().numpy()
            dec.close()
        assert np.array_equal(out[fec.FLOODING], ref), ebn0
        assert np.array_equal(out[fec.FLAT_LAYERED], lay_o), ebn0
        r = errstats.rate_summary(ref[:, : code.k], info)
        g = errstats.rate_summary(out[fec.FLAT_LAYERED][:, : code.k], info)
        _report(f"C1 {ebn0:g} dB", r, g, errstats.frame_errors(ref[:, : code.k], info) > 0,
                errstats.frame_errors(out[fec.FLAT_LAYERED][:, : code.k], info) > 0)
        assert g["fer"] <= r["fer_ci95"][1] and g["ber"] <= r["ber_ci95"][1], (ebn0, g, r)


@pytest.mark.parametrize("snr", [8.0, 12.0, 16.0])
def test_c3_ofdm_chain_fer_parity(cuda, oracle, pool, snr):
    """C3: 256 frames of the 16-QAM OFDM workload (the bench's first batch at this SNR) through the
    GPU chain (batched sync + demod, layered BP of 25 iterations) and through the reference chain."""
    from oracle import ofdm_chain_parallel
    from sicc_gb300 import fec, ofdm
    from sicc_gb300.pipeline import RxPipeline, SYNC_RECORD
    torch = cuda
    t = ofdm.reference_tables(ofdm.OFDM_C3)
    code = codes.ofdm_code()
    frames = 256
    i = (8.0, 12.0, 16.0).index(snr)
    gen = ofdm.FrameGenerator(t, code, seed=500 + 10 * i)
    b = gen.batch(frames, snr_db=snr, cfo_subcarriers=0.1, max_offset=200, rayleigh_taps=6)
    blocks = gen.blocks
    nv = float(np.float32(np.mean(b.noise_var)))
    L = b.iq.shape[1]

    p = RxPipeline(t, code.n, code.k, blocks, nv, max_batch_frames=frames)
    d_llr = torch.zeros((frames * blocks, code.n), dtype=torch.float32, device="cuda")
    d_sync = torch.zeros(frames * SYNC_RECORD.itemsize, dtype=torch.uint8, device="cuda")
    p.demod_batch(torch.from_numpy(b.iq).cuda(), L, L, frames, d_llr, d_sync, torch.cuda.current_stream())
    dec = fec.CsrBpDecoder.for_code(code, max_batch=frames * blocks, max_iter=25, normalization=0.75)
    bits = torch.zeros((frames * blocks, code.n), dtype=torch.uint8, device="cuda")
    dec.decode_device_batch(d_llr, bits, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    sync = d_sync.cpu().numpy().view(SYNC_RECORD)
    g_info = bits.cpu().numpy()[:, : code.k].reshape(frames, blocks, code.k)

    found, start, cfo, r_info = ofdm_chain_parallel(pool, ofdm.OFDM_C3, code, b.iq, nv, 25, 0.75)
    r_info = r_info.reshape(frames, blocks, code.k)

    # the same frames found, at the same starts (CFO within 1e-3 relative)
    g_found = sync["found"].astype(np.int32)
    assert np.array_equal(g_found == 1, found == 1), np.flatnonzero((g_found == 1) != (found == 1))
    hit = found == 1
    assert np.array_equal(sync["start"][hit], start[hit])
    np.testing.assert_allclose(sync["cfo_hz"][hit], cfo[hit], rtol=1e-3, atol=1.0)

    sent = b.info.reshape(frames, blocks, code.k)
    g_cw_fail = np.any(g_info != sent, axis=2)
    r_cw_fail = np.any(r_info != sent, axis=2)
    g_cw_fail[~hit] = True  # a frame that is not found loses all its codewords on both sides
    r_cw_fail[~hit] = True
    agree = float(np.mean(g_cw_fail == r_cw_fail))
    g_cer = errstats.wilson(int(g_cw_fail.sum()), g_cw_fail.size)
    r_cer = errstats.wilson(int(r_cw_fail.sum()), r_cw_fail.size)
    g_fer = errstats.wilson(int(g_cw_fail.any(axis=1).sum()), frames)
    r_fer = errstats.wilson(int(r_cw_fail.any(axis=1).sum()), frames)
    print(f"C3 {snr:g} dB: frames found {int(hit.sum())}/{frames}; codeword outcome agreement {agree:.4f}; "
          f"CER GPU {g_cer[0]:.4f} reference {r_cer[0]:.4f} {np.round(r_cer[1:], 4).tolist()}; "
          f"FER GPU {g_fer[0]:.4f} reference {r_fer[0]:.4f} {np.round(r_fer[1:], 4).tolist()}")
    assert agree >= 0.99
    from sicc_gb300.pipeline import wait_timeouts
    assert wait_timeouts() == 0  # every staged-sample copy of the demodulator landed in time
    assert errstats.inside(g_cer[0], r_cer[1:]) and errstats.inside(r_cer[0], g_cer[1:])
    assert errstats.inside(g_fer[0], r_fer[1:]) and errstats.inside(r_fer[0], g_fer[1:])
