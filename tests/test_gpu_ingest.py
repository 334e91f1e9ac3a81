"""Real-time ingest: device IQ ring, frame pool and the extraction loop.

A continuous stream of frames from the restated transmitter, separated by
random noise-only gaps, with AWGN and a carrier offset over the whole stream,
is pushed in chunks of random size; after every push one step runs, as the
reference's RX loop does (uhd_ldpc_ofdm_link.cpp:8480-8567).  Every frame must
be found at the sample where it was placed, its pool slot must hold exactly
those stream samples, its CFO must be the applied one, and demodulating and
decoding the pool frames must return the transmitted bits.  Overflow drops the
oldest samples and restarts acquisition on the newest; an exhausted pool skips
frames and counts them.
"""
import ctypes as C
import os

import numpy as np
import pytest

import tx_oracle
from sicc_gb300 import codes, fec, ofdm
from sicc_gb300.ingest import Ingest
from sicc_gb300.pipeline import RxPipeline, SYNC_RECORD

pytestmark = pytest.mark.gpu

CFG = ofdm.OFDM_SMALL


def _cudart():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    lib = C.CDLL(os.path.join(home, "lib64", "libcudart.so"))
    lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    return lib


def _d2h(ptr, n):
    out = np.zeros(n, np.complex64)
    assert _cudart().cudaMemcpy(out.ctypes.data, ptr, out.nbytes, 2) == 0  # device to host
    return out


def _stream(frames, seed, cfo_sc=0.05, noise=1e-3, max_gap=200):
    t = ofdm.reference_tables(CFG)
    code = codes.short_code()
    blocks = t.coded_bits // code.n
    G = np.concatenate([np.eye(code.k, dtype=np.uint8), codes.gf2_parity_matrix(code)], 1)
    rng = np.random.default_rng(seed)
    info = rng.integers(0, 2, size=(frames, blocks * code.k), dtype=np.uint8)
    coded = tx_oracle.encode_generator(info.reshape(-1, code.k), G).reshape(frames, -1)
    tx = tx_oracle.tx_frames(coded, nfft=CFG.nfft, cp=CFG.cp, num_symbols=CFG.num_symbols, active_sc=CFG.active_sc,
                             bps=CFG.bits_per_symbol, used_bins=t.used_bins, pilot_symbols=t.pilot_symbols,
                             data_symbols=t.data_symbols, pilot_grid=t.pilot_grid, preamble=t.preamble,
                             amplitude=CFG.amplitude)
    parts, pos, at = [np.zeros(int(rng.integers(300, 800)))], [], 0
    at = parts[0].size
    for f in range(frames):
        pos.append(at)
        parts.append(tx[f])
        gap = np.zeros(int(rng.integers(0, max_gap)))
        parts.append(gap)
        at += tx[f].size + gap.size
    parts.append(np.zeros(3000))
    x = np.concatenate(parts).astype(np.complex128)
    n = np.arange(x.size)
    x = x * np.exp(2j * np.pi * (cfo_sc * CFG.sample_rate / CFG.nfft) * n / CFG.sample_rate)
    x += noise * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    return t, code, blocks, x.astype(np.complex64), np.array(pos), info, cfo_sc * CFG.sample_rate / CFG.nfft


def _pipe(t, code, blocks):
    return RxPipeline(t, code.n, code.k, blocks, 2e-6, slots=2, max_batch_frames=32)


def _model(oracle, t, chunks, bmin, bmax, acq, trk):
    """The RX loop's device branch (L:8480-8567) restated on the host over the oracle's frame search:
    stream positions of the frames it extracts (no overflow, late-peak check off)."""
    ph = oracle.phy(t)
    fl, pre = t.frame_len, 2 * t.cfg.pre_half_len
    ring = np.zeros(0, np.complex64)
    read, tracking, found = 0, False, []
    for chunk in chunks:
        ring = np.concatenate([ring, chunk])
        if ring.size == 0:
            continue
        n = min(ring.size, max(bmin, bmax))
        base = 0
        while True:
            available = n - base
            if available < pre:
                break
            count = min(available, trk if tracking else acq)
            r, start, _, fine, _ = oracle.sync_earliest(ph, ring[base: base + count])
            if r == 0:
                tracking = False
                break
            if start + fl > available:
                break
            found.append(read + base + start)
            tracking = True
            base += start + fl
        used = base if base > 0 else (n - fl if n > fl else 0)
        if base == 0 and n > fl:
            tracking = False
        ring = ring[used:]
        read += used
    return found


@pytest.mark.parametrize("max_gap", [200, 400])
def test_ingest_extracts_as_the_receive_loop(cuda, oracle, max_gap):
    """Gaps within the tracking window: every frame; wider gaps: the frames the loop itself keeps."""
    torch = cuda
    t, code, blocks, x, pos, info, cfo = _stream(12, seed=1, max_gap=max_gap)
    p = _pipe(t, code, blocks)
    ing = Ingest(p, ring_samples=1 << 15, pool_frames=8)
    fl = t.frame_len
    rng = np.random.default_rng(2)
    cuts = [0]
    while cuts[-1] < x.size:
        cuts.append(min(x.size, cuts[-1] + int(rng.integers(500, 2500))))
    chunks = [x[a:b] for a, b in zip(cuts[:-1], cuts[1:])]
    dec = fec.CsrBpDecoder.for_code(code, max_batch=32 * blocks)
    got = []
    for chunk in chunks:
        ing.push(chunk)
        new = []
        for slot, position, peak, cfo_hz in ing.step(timeout_ms=0):
            frame = _d2h(ing.frame_ptr(slot), fl)
            assert np.array_equal(frame, x[position: position + fl])  # the pool holds the stream samples
            assert abs(cfo_hz - cfo) < 0.01 * CFG.sample_rate / CFG.nfft
            new.append((slot, position))
        if new:  # demodulate and decode this step's frames from the pool, then release them
            pool, fs = ing.pool()
            offs = torch.tensor([s_ * fs for s_, _ in new], dtype=torch.int64, device="cuda")
            d_llr = torch.zeros((len(new), blocks * code.n), dtype=torch.float32, device="cuda")
            llr_off = torch.arange(len(new), dtype=torch.int64, device="cuda") * (blocks * code.n)
            d_sync = torch.zeros(len(new) * SYNC_RECORD.itemsize, dtype=torch.uint8, device="cuda")
            p.demod_gather(pool, offs, fl, len(new), d_llr, llr_off, d_sync, stream=torch.cuda.current_stream())
            torch.cuda.synchronize()
            bits, ok, _ = dec.decode(d_llr.reshape(-1, code.n), device=True)
            for i, (slot, position) in enumerate(new):
                k = int(np.nonzero(pos == position)[0][0])  # a transmitted frame, at its own position
                assert np.array_equal(bits[i * blocks:(i + 1) * blocks, : code.k].reshape(-1), info[k])
                ing.release(slot)
                got.append(position)
    pre = 2 * CFG.pre_half_len
    expect = _model(oracle, t, chunks, fl, 2 * fl, 2 * fl, pre + 256)
    assert got == expect
    if max_gap <= 200:
        assert got == list(pos)
    st = ing.stats()
    assert st["found"] == len(got) and st["dropped_samples"] == 0 and st["pool_exhausted"] == 0
    assert st["free_slots"] == 8


def test_ingest_overflow_keeps_the_newest_samples(cuda):
    t, code, blocks, x, pos, info, cfo = _stream(10, seed=3)
    p = _pipe(t, code, blocks)
    fl = t.frame_len
    ing = Ingest(p, ring_samples=8192, pool_frames=8)
    x = x[: pos[-1] + fl + 50]  # the stream ends just after its last frame
    for at in range(0, x.size, 4000):  # no step while pushing: the ring overflows
        ing.push(x[at: at + 4000])
    st = ing.stats()
    assert st["dropped_samples"] == x.size - 8192 and st["buffered"] == 8192
    frames = ing.step(timeout_ms=0)  # more than 3/4 full: the newest buffered_max samples, acquisition
    tail0 = x.size - 2 * fl
    expect = [q for q in pos if q >= tail0 and q + fl <= x.size]
    assert expect and [f[1] for f in frames] == expect
    for slot, position, _, _ in frames:
        assert np.array_equal(_d2h(ing.frame_ptr(slot), fl), x[position: position + fl])
    assert ing.stats()["buffered"] == 0


def test_ingest_pool_exhaustion_skips_frames(cuda):
    t, code, blocks, x, pos, info, cfo = _stream(8, seed=4)
    p = _pipe(t, code, blocks)
    ing = Ingest(p, ring_samples=1 << 15, pool_frames=4)
    found = []
    for at in range(0, x.size, 1500):
        ing.push(x[at: at + 1500])
        found += ing.step(timeout_ms=0)
    st = ing.stats()
    assert len(found) == 4 and st["pool_exhausted"] >= 1 and st["free_slots"] == 0
    assert [f[1] for f in found] == list(pos[:4])
    for f in found:
        ing.release(f[0])
    assert ing.stats()["free_slots"] == 4
    from sicc_gb300._lib import SiccError
    with pytest.raises(SiccError):
        ing.release(found[0][0])  # not leased any more
