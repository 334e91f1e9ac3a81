"""GPU parity of the OFDM receive path (sync, demod, decode) against the reference.

References: the golden fixture produced by the reference's own CPU receiver
(tests/golden/ofdm_small.npz: sync results and decode_frame outputs) and the
oracle restatement of its demodulator (bit-exact with it, see
tests/test_oracle_pins.py).

Tolerances (single-precision FFT and derotation against the reference's double
precision): frame start and found flag exact; CFO within 1e-3 relative + 1 Hz;
LLRs within 2e-4 of the frame's largest |LLR| (absolute) and 1e-3 relative;
hard decisions equal wherever |LLR| exceeds that tolerance; decoded bits equal.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from sicc_gb300 import codes, ofdm

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.gpu


def _fixture():
    return dict(np.load(os.path.join(GOLDEN, "ofdm_small.npz")))


def _pipe(t, noise_var, blocks=16, code=None, **kw):
    from sicc_gb300.pipeline import RxPipeline
    code = code or codes.short_code()
    return RxPipeline(t, code.n, code.k, blocks, noise_var, **kw)


def _llr_close(got, ref):
    scale = max(float(np.max(np.abs(ref))), 1.0)
    err = np.abs(got - ref)
    ok = err <= 2e-4 * scale + 1e-3 * np.abs(ref)
    assert ok.all(), (float(err.max()), scale)
    sure = np.abs(ref) > 2e-4 * scale
    assert np.array_equal(got[sure] < 0, ref[sure] < 0)


def test_find_frame_matches_reference_receiver(cuda):
    d = _fixture()
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    p = _pipe(t, 1.0, max_rx_search_samples=d["iq"].shape[1])
    for i in range(d["iq"].shape[0]):
        start, metric, cfo = p.find_frame(0, d["iq"][i][: d["lengths"][i]])
        found, rstart, coarse, fine, rcfo = d["sync"][i]
        if abs(fine - t.cfg.sync_threshold) < 1e-3:
            continue  # single vs double precision may land on either side of the threshold
        if int(found) == 1:
            assert start == int(rstart)
            assert metric == pytest.approx(fine, rel=1e-4)
            assert cfo == pytest.approx(rcfo, rel=1e-3, abs=1.0)
        else:
            assert start == -1


def test_demod_matches_oracle(cuda, oracle):
    """Given the same start and CFO, the GPU demodulator matches the reference's arithmetic."""
    d = _fixture()
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    ph = oracle.phy(t)
    flen = t.frame_len
    checked = 0
    for i in range(d["iq"].shape[0]):
        found, start, _, _, _ = d["sync"][i]
        if int(found) != 1:
            continue
        nv = float(np.float32(d["noise_var"][i]))
        p = _pipe(t, nv)
        frame = d["iq"][i][int(start):int(start) + flen]
        got, (s, _, gcfo) = p.demod_to_host(0, frame)
        assert s == 0
        ref = oracle.demod_frame(ph, frame, float(gcfo), nv)
        _llr_close(got, ref)
        checked += 1
    assert checked >= 4


def test_demod_to_host_and_decode_match_reference(cuda, oracle):
    """Full chain on the reference fixture frames: GPU sync + demod + flooding decode."""
    from sicc_gb300 import fec
    d = _fixture()
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    code = codes.short_code()
    dec = fec.CsrBpDecoder.for_code(code, max_batch=64, max_iter=25, normalization=0.75, schedule=fec.FLOODING)
    flen = t.frame_len
    checked = 0
    for i in range(d["iq"].shape[0]):
        found, start, _, fine, cfo = d["sync"][i]
        if int(found) != 1 or abs(fine - t.cfg.sync_threshold) < 1e-3:
            continue
        p = _pipe(t, float(d["noise_var"][i]))
        llr, (s, metric, gcfo) = p.demod_to_host(0, d["iq"][i][int(start):int(start) + flen])
        assert s == 0  # the frame handed over starts at the preamble
        bits, ok, _ = dec.decode(llr.reshape(-1, code.n))
        got = bits[:, : code.k].reshape(-1)
        assert np.array_equal(got, d["decoded"][i])
        checked += 1
    assert checked >= 4


def test_batched_search_and_demod(cuda, oracle):
    torch = cuda
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    code = codes.short_code()
    gen = ofdm.FrameGenerator(t, code, seed=31)
    b = gen.batch(24, snr_db=18.0, cfo_subcarriers=0.1, max_offset=120, rayleigh_taps=0)
    p = _pipe(t, float(b.noise_var[0]), max_batch_frames=32)
    from sicc_gb300.pipeline import SYNC_RECORD
    d_iq = torch.from_numpy(b.iq).cuda()
    d_llr = torch.zeros((24, p.coded_bits), dtype=torch.float32, device="cuda")
    d_sync = torch.zeros(24 * SYNC_RECORD.itemsize, dtype=torch.uint8, device="cuda")
    p.demod_batch(d_iq, b.iq.shape[1], b.iq.shape[1], 24, d_llr, d_sync, torch.cuda.current_stream())
    torch.cuda.synchronize()
    sync = d_sync.cpu().numpy().view(SYNC_RECORD)
    llr = d_llr.cpu().numpy()
    ph = oracle.phy(t)
    for f in range(24):
        r = oracle.sync_earliest(ph, b.iq[f])
        assert sync[f]["found"] == r[0]
        if r[0] != 1:
            continue
        assert sync[f]["start"] == r[1]
        ref = oracle.demod_frame(ph, b.iq[f][r[1]:r[1] + t.frame_len], float(sync[f]["cfo_hz"]),
                                 float(np.float32(b.noise_var[0])))
        _llr_close(llr[f], ref)
        assert np.mean((llr[f] < 0) != b.coded[f]) < 0.02
    sms, dms = p.last_batch_ms()
    assert sms > 0 and dms > 0


def test_gathered_demod_matches_batched(cuda):
    """Frames scattered in device memory (reversed, gaps) demodulate exactly as the strided batch."""
    torch = cuda
    from sicc_gb300.pipeline import SYNC_RECORD
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    code = codes.short_code()
    gen = ofdm.FrameGenerator(t, code, seed=41)
    b = gen.batch(10, snr_db=9.0, cfo_subcarriers=0.2, max_offset=150)
    L = b.iq.shape[1]
    p = _pipe(t, float(np.float32(np.mean(b.noise_var))), max_batch_frames=16)
    d_iq = torch.from_numpy(b.iq).cuda()
    d_llr = torch.zeros((10, p.coded_bits), dtype=torch.float32, device="cuda")
    d_sync = torch.zeros(10 * SYNC_RECORD.itemsize, dtype=torch.uint8, device="cuda")
    p.demod_batch(d_iq, L, L, 10, d_llr, d_sync, torch.cuda.current_stream())
    # gathered: frame f at slot 2*(9-f) of a buffer twice as long, LLRs reversed with a gap
    big = torch.zeros((20, L), dtype=torch.complex64, device="cuda")
    order = np.arange(10)[::-1].copy()
    for f in range(10):
        big[2 * order[f]] = d_iq[f]
    f_off = torch.from_numpy((2 * order * L).astype(np.int64)).cuda()
    gap = p.coded_bits + 64
    l_off = torch.from_numpy((order * gap).astype(np.int64)).cuda()
    g_llr = torch.full((10 * gap,), 7.0, dtype=torch.float32, device="cuda")
    g_sync = torch.zeros(10 * SYNC_RECORD.itemsize, dtype=torch.uint8, device="cuda")
    p.demod_gather(big, f_off, L, 10, g_llr, l_off, g_sync, torch.cuda.current_stream())
    torch.cuda.synchronize()
    ref_llr = d_llr.cpu().numpy()
    ref_sync = d_sync.cpu().numpy().view(SYNC_RECORD)
    got = g_llr.cpu().numpy()
    got_sync = g_sync.cpu().numpy().view(SYNC_RECORD)
    for f in range(10):
        o = order[f] * gap
        assert np.array_equal(got[o:o + p.coded_bits], ref_llr[f])
        assert np.all(got[o + p.coded_bits:o + gap] == 7.0)
        assert got_sync[f] == ref_sync[f]


def test_ofdm_rx_workload_frames(cuda, oracle):
    """The 1024-point, 600-subcarrier 16-QAM workload: 30 codewords + 480 filler bits per frame."""
    torch = cuda
    from sicc_gb300 import fec
    from sicc_gb300.pipeline import SYNC_RECORD
    t = ofdm.reference_tables(ofdm.OFDM_C3)
    code = codes.ofdm_code()
    gen = ofdm.FrameGenerator(t, code, seed=9)
    assert gen.blocks == 30
    b = gen.batch(8, snr_db=16.0, cfo_subcarriers=0.1, max_offset=200, rayleigh_taps=6)
    p = _pipe(t, float(np.mean(b.noise_var)), blocks=30, code=code, max_batch_frames=8)
    d_iq = torch.from_numpy(b.iq).cuda()
    d_llr = torch.zeros((8, p.coded_bits), dtype=torch.float32, device="cuda")
    d_sync = torch.zeros(8 * SYNC_RECORD.itemsize, dtype=torch.uint8, device="cuda")
    p.demod_batch(d_iq, b.iq.shape[1], b.iq.shape[1], 8, d_llr, d_sync, torch.cuda.current_stream())
    torch.cuda.synchronize()
    sync = d_sync.cpu().numpy().view(SYNC_RECORD)
    ph = oracle.phy(t)
    llr = d_llr.cpu().numpy()
    nv = float(np.float32(np.mean(b.noise_var)))
    for f in range(8):
        r = oracle.sync_earliest(ph, b.iq[f])
        assert sync[f]["found"] == r[0]
        if r[0] == 1:
            assert sync[f]["start"] == r[1]
            ref = oracle.demod_frame(ph, b.iq[f][r[1]:r[1] + t.frame_len], float(sync[f]["cfo_hz"]), nv)
            _llr_close(llr[f], ref[: p.coded_bits])
    # decode chain parity: the GPU decoder on GPU LLRs against the oracle decoder on oracle LLRs
    # (the reference receiver's FER under this channel is high: single-pilot LS estimation and the
    # biased MMSE symbol estimate in fades; the check is that both chains agree frame by frame)
    dec = fec.CsrBpDecoder.for_code(code, max_batch=240, max_iter=25, normalization=0.75)
    bits, ok, _ = dec.decode(d_llr.reshape(-1, code.n), device=True)
    info = bits[:, : code.k].reshape(8, -1)
    oc = oracle.code(code.n, code.m, code.row_ptr, code.col_ind)
    agree = 0
    found = 0
    for f in range(8):
        r = oracle.sync_earliest(ph, b.iq[f])
        if r[0] != 1:
            continue
        found += 1
        ref_llr = oracle.demod_frame(ph, b.iq[f][r[1]:r[1] + t.frame_len], float(sync[f]["cfo_hz"]), nv)
        ref_info, _ = oc.bp_osd_batch(ref_llr[: p.coded_bits], schedule=3, max_iter=25, alpha=0.75, osd_order=-1)
        # frame outcome (decoded correctly or not) agrees; bits of undecodable frames are not compared
        agree += np.array_equal(info[f], b.info[f]) == np.array_equal(ref_info.reshape(-1), b.info[f])
    assert found >= 6 and agree >= found - 1


def test_demod_shapes_give_identical_llrs(cuda):
    """Data symbols per demodulator CTA changes the grid and the pilot transforms each CTA
    repeats, never the LLRs; every staged-sample wait lands in time."""
    torch = cuda
    from sicc_gb300.pipeline import SYNC_RECORD, wait_timeouts
    t = ofdm.reference_tables(ofdm.OFDM_C3)
    code = codes.ofdm_code()
    gen = ofdm.FrameGenerator(t, code, seed=31)
    b = gen.batch(12, snr_db=14.0, cfo_subcarriers=0.1, max_offset=200, rayleigh_taps=6)
    p = _pipe(t, float(np.mean(b.noise_var)), blocks=30, code=code, max_batch_frames=12)
    d_iq = torch.from_numpy(b.iq).cuda()
    L = b.iq.shape[1]

    def run():
        d_llr = torch.full((12, p.coded_bits), 7.0, dtype=torch.float32, device="cuda")
        d_sync = torch.zeros(12 * SYNC_RECORD.itemsize, dtype=torch.uint8, device="cuda")
        p.demod_batch(d_iq, L, L, 12, d_llr, d_sync, torch.cuda.current_stream())
        torch.cuda.synchronize()
        return d_llr.cpu().numpy()

    ref = run()
    for spc in (1, 2, 3, 5, 7, 13):
        p.set_demod_shape(spc)
        assert np.array_equal(run().view(np.uint32), ref.view(np.uint32)), spc
    from sicc_gb300 import _lib
    with pytest.raises(_lib.SiccError):
        p.set_demod_shape(14)
    assert wait_timeouts() == 0


def test_no_frame_in_noise(cuda):
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    p = _pipe(t, 1.0, max_rx_search_samples=4000)
    noise = (np.random.default_rng(1).standard_normal(4000) * 0.01).astype(np.complex64)
    start, metric, cfo = p.find_frame(0, noise)
    assert start == -1 and cfo == 0.0
    llr, (s, _, _) = p.demod_to_host(0, noise[: t.frame_len])
    assert s == -1 and np.all(llr == 0)


def tx_oracle_generator(code):
    """[k][n] systematic generator [I | P] of a QC code."""
    P = codes.gf2_parity_matrix(code)
    return np.ascontiguousarray(np.concatenate([np.eye(code.k, dtype=np.uint8), P], axis=1), np.uint8)


def test_cpp_pipeline_class_drop_in(cuda):
    """The C++ class of include/gpu_ofdm_pipeline.hpp, compiled and run as a caller would."""
    from sicc_gb300 import _lib
    d = _fixture()
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    code = codes.short_code()
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "pbc")
        libdir = os.path.dirname(_lib.LIB_PATH)
        cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(cuda_home, "include"),
                        os.path.join(ROOT, "tests", "cpp", "pipeline_bridge_check.cpp"), "-o", exe,
                        "-L" + libdir, "-lsicc_gb300", "-L" + os.path.join(cuda_home, "lib64"), "-lcudart",
                        "-Wl,-rpath," + libdir + ":" + os.path.join(cuda_home, "lib64")], check=True)
        i = 0
        cfg = t.cfg
        np.array([cfg.nfft, cfg.cp, cfg.pre_half_len, cfg.num_symbols, cfg.active_sc, cfg.bits_per_symbol,
                  code.n, code.k, 16], np.int32).tofile(os.path.join(tmp, "cfg_int.bin"))
        np.array([cfg.sample_rate, cfg.sync_threshold, d["noise_var"][i]], np.float32).tofile(
            os.path.join(tmp, "cfg_float.bin"))
        for name, arr, dt in (("used", t.used_indices, np.int32), ("pilots", t.pilot_symbols, np.int32),
                              ("data", t.data_symbols, np.int32), ("p0", t.interp_p0, np.int32),
                              ("p1", t.interp_p1, np.int32), ("alpha", t.interp_alpha, np.float32),
                              ("grid", t.pilot_grid, np.complex64), ("pre", t.preamble, np.complex64),
                              ("frame", d["iq"][i][: d["lengths"][i]], np.complex64)):
            np.ascontiguousarray(arr, dt).tofile(os.path.join(tmp, name + ".bin"))
        gen = tx_oracle_generator(code)
        info = np.random.default_rng(5).integers(0, 2, size=16 * code.k, dtype=np.uint8)
        gen.tofile(os.path.join(tmp, "gen.bin"))
        info.tofile(os.path.join(tmp, "tx_info.bin"))
        r = subprocess.run([exe, tmp], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        vals = open(os.path.join(tmp, "sync.txt")).read().split()
        start = int(vals[0])
        assert start == int(d["sync"][i][1]) and vals[6] == "1" and vals[7] == "1"
        host = np.fromfile(os.path.join(tmp, "llr_host.bin"), np.float32)
        dev = np.fromfile(os.path.join(tmp, "llr_device.bin"), np.float32)
        assert host.size == 16 * 128
        # the host path re-searches the frame (start 0) and the device path is told the CFO: same LLRs
        assert np.max(np.abs(host - dev)) <= 1e-3 * max(np.max(np.abs(host)), 1.0)
        # the transmit members against the restated GPU transmitter (tolerance: fp32 inverse FFT)
        import tx_oracle
        coded = tx_oracle.encode_generator(info.reshape(16, code.k), gen).reshape(1, -1)
        kw = dict(nfft=cfg.nfft, cp=cfg.cp, num_symbols=cfg.num_symbols, active_sc=cfg.active_sc,
                  bps=cfg.bits_per_symbol, used_bins=t.used_bins, pilot_symbols=t.pilot_symbols,
                  data_symbols=t.data_symbols, pilot_grid=t.pilot_grid, preamble=t.preamble,
                  amplitude=0.20)  # the bridge Config's tx_amplitude default (PH:30), which the check keeps
        for name, extra in (("tx_frame", {}), ("tx_frame_noise", dict(noise_var=0.05, noise_seed=99))):
            got = np.fromfile(os.path.join(tmp, name + ".bin"), np.complex64)
            ref = tx_oracle.tx_frames(coded, **kw, **extra)[0]
            assert got.size == ref.size
            assert np.max(np.abs(got - ref)) <= 2e-5 * np.max(np.abs(ref)), name
