"""The device-resident request loop against decoding each request alone.

The loop (include/sicc_devloop.h) admits, lays out, decodes and completes
requests inside one CUDA graph repeated on the GPU.  Every request of a mixed
stream (several codes, BP-only and BP+OSD protection, requests arriving while
earlier ones decode) must come back with the bits the oracle's BP -> OSD chain
gives for it alone (LLR requests), or that the pipeline's batched demodulator
followed by the mixed engine give for it alone (OFDM IQ requests, demodulated
inside the loop); the loop must end by itself when idle and start again on
the next request, stop when asked, and reject buffers the GPU cannot address.
"""
import time

import numpy as np
import pytest

from sicc_gb300 import channel, codes, engine, ofdm

pytestmark = pytest.mark.gpu


def _codes():
    cs = [c for c in codes.mixed_codes() if engine.osd_supported(c)][:3] + [codes.short_code()]
    cs.append(next(c for c in codes.mixed_codes() if c.n == 1024))
    return cs


def _loop(cs, **kw):
    from sicc_gb300.devloop import DevLoop
    lp = DevLoop(**kw)
    for c in cs:
        lp.add_code(c, engine.iteration_cap(c.n), osd_order=2 if engine.osd_supported(c) else -1)
    return lp


def _expected(oracle, c, llr, protection):
    oc = oracle.code(c.n, c.m, c.row_ptr, c.col_ind)
    table = oc.systematic_parity() if engine.osd_supported(c) else None
    out = []
    for x in llr:
        r = oc.layered(x, engine.iteration_cap(c.n), 0.75)
        if r[0] or not protection or table is None:
            out.append(r[1][: c.k])
        else:
            out.append(oracle.osd(table, c.n, c.k, r[3], 2, 64, 4096)[0][: c.k])
    return np.array(out, np.uint8)


def _pinned_llrs(c, cnt, ebn0, seed):
    from sicc_gb300.devloop import pinned
    _, _, llr = channel.awgn_llrs(c, cnt, ebn0, seed=seed)
    buf = pinned(llr.shape, np.float32)
    buf[:] = llr
    return buf


@pytest.mark.parametrize("lanes", [1, 3])
def test_device_loop_matches_requests_decoded_alone(cuda, oracle, lanes):
    """One lane, and three lanes sharing the rings (batches decoded side by side, finishing out of order)."""
    cs = _codes()
    lp = _loop(cs, max_batch_codewords=2048, max_batch_llr_floats=2048 * 1024, ring_requests=64, lanes=lanes)
    lp.start()
    rng = np.random.default_rng(15)
    reqs = []
    for r in range(48):
        ci = int(rng.integers(0, len(cs)))
        cnt = int(rng.integers(1, 60))
        llr = _pinned_llrs(cs[ci], cnt, rng.uniform(1.0, 3.5, cnt), 1900 + r)
        prot = int(rng.integers(0, 2))
        req, x, out = lp.request(ci, llr, protection=prot, tag=r)
        rid = lp.submit_request(req, keep=(x, out))
        while rid is None:
            time.sleep(0.0002)
            rid = lp.submit_request(req, keep=(x, out))
        reqs.append((ci, llr, prot, rid, out))
        if r % 7 == 3:
            time.sleep(0.002)  # some requests arrive while earlier iterations decode
    done = {}
    t0 = time.time()
    while len(done) < len(reqs) and time.time() - t0 < 60:
        for d in lp.poll(wait_us=100000):
            done[d.request_id] = d
    assert len(done) == len(reqs)
    st = lp.stats()
    assert st.completed == len(reqs) and st.iterations >= 1 and st.codewords >= sum(r[1].shape[0] for r in reqs)
    assert st.lanes == lanes
    for ci, llr, prot, rid, out in reqs:
        c = cs[ci]
        d = done[rid]
        assert d.status == 0 and d.codewords == llr.shape[0]
        assert d.latency_us > 0.0 and d.batch_gpu_us >= 0.0
        assert np.array_equal(out, _expected(oracle, c, llr, prot)), (c.name(), rid)
        if not prot or not engine.osd_supported(c):
            assert d.osd_codewords == 0
    lp.stop()
    assert lp.stats().running == 0
    lp.close()


def test_device_loop_ends_when_idle_and_restarts(cuda, oracle):
    c = codes.short_code()
    lp = _loop([c], max_batch_codewords=256, max_batch_llr_floats=256 * 128, ring_requests=16, idle_timeout_ms=30)
    lp.start()
    t0 = time.time()
    while lp.stats().running and time.time() - t0 < 5.0:
        time.sleep(0.02)
    assert lp.stats().running == 0  # the loop ended by itself after its idle timeout
    llr = _pinned_llrs(c, 20, 2.0, 77)
    req, x, out = lp.request(0, llr, protection=1)
    rid = lp.submit_request(req, keep=(x, out))
    got = []
    t0 = time.time()
    while not got and time.time() - t0 < 30:
        got = lp.poll(wait_us=100000)
    assert got and got[0].request_id == rid
    assert lp.stats().launches == 2
    assert np.array_equal(out, _expected(oracle, c, llr, 1))
    lp.close()


def test_device_loop_rejects_what_it_cannot_serve(cuda):
    from sicc_gb300 import _lib
    c = codes.short_code()
    lp = _loop([c], max_batch_codewords=64, max_batch_llr_floats=64 * 128, ring_requests=8)
    pageable = np.zeros((4, c.n), np.float32)
    req, x, out = lp.request(0, pageable)
    with pytest.raises(_lib.SiccError):
        lp.submit_request(req, keep=(x, out))
    big = _pinned_llrs(c, 65, 2.0, 5)
    req, x, out = lp.request(0, big)
    with pytest.raises(_lib.SiccError):
        lp.submit_request(req, keep=(x, out))
    lp.start()
    lp.stop(wait_ms=5000)
    assert lp.stats().running == 0
    lp.close()


def test_device_loop_iq_requests_match_pipeline_then_engine(cuda):
    """IQ requests are searched and demodulated inside the loop, beside LLR requests of other codes."""
    torch = cuda
    from sicc_gb300.devloop import pinned
    from sicc_gb300.pipeline import RxPipeline, SYNC_RECORD
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    code = codes.short_code()
    gen = ofdm.FrameGenerator(t, code, seed=78)
    blocks = gen.blocks
    b = gen.batch(12, snr_db=14.0, cfo_subcarriers=0.1, max_offset=100)
    stride = b.iq.shape[1]
    nv = float(np.float32(np.mean(b.noise_var)))
    cs = _codes()
    cid = len(cs) - 2  # the short code
    assert cs[cid].n == code.n and cs[cid].k == code.k
    lp = _loop(cs, max_batch_codewords=1024, max_batch_llr_floats=1024 * 1024, ring_requests=32,
               max_batch_frames=8, max_batch_iq_samples=8 * stride, lanes=2)
    pid = lp.add_phy(t, cid, blocks, nv, stride)
    lp.start()
    iq_reqs = []
    for r in range(4):
        sl = pinned((3, stride), np.complex64)
        sl[:] = b.iq[3 * r: 3 * r + 3]
        req, x, out = lp.iq_request(pid, sl, protection=r % 2, tag=r)
        rid = lp.submit_request(req, keep=(x, out))
        iq_reqs.append((sl, rid, out))
        llr = _pinned_llrs(cs[0], 16, 2.0, r)
        req, x, o2 = lp.request(0, llr, protection=1)
        lp.submit_request(req, keep=(x, o2))
    want = {rid for _, rid, _ in iq_reqs}
    got = {}
    t0 = time.time()
    while not want <= set(got) and time.time() - t0 < 60:
        for d in lp.poll(wait_us=100000):
            got[d.request_id] = d
    assert want <= set(got)
    pipe = RxPipeline(t, code.n, code.k, blocks, nv, max_rx_search_samples=stride, max_batch_frames=16)
    eng = engine.Engine(max_codewords=3 * blocks, max_llr_floats=3 * blocks * code.n)
    for c in cs:
        eng.add_code(c, engine.iteration_cap(c.n), osd_order=2 if engine.osd_supported(c) else -1)
    for r, (sl, rid, out) in enumerate(iq_reqs):
        d_iq = torch.from_numpy(np.ascontiguousarray(sl)).cuda()
        d_llr = torch.zeros((3, blocks * code.n), dtype=torch.float32, device="cuda")
        d_sync = torch.zeros(3 * SYNC_RECORD.itemsize, dtype=torch.uint8, device="cuda")
        pipe.demod_batch(d_iq, stride, stride, 3, d_llr, d_sync, torch.cuda.current_stream())
        cw = 3 * blocks
        code_ids = torch.full((cw,), cid, dtype=torch.uint8, device="cuda")
        prot = torch.full((cw,), r % 2, dtype=torch.uint8, device="cuda")
        llr_off = torch.arange(cw, dtype=torch.int64, device="cuda") * code.n
        info_off = torch.arange(cw, dtype=torch.int64, device="cuda") * code.k
        info = torch.zeros(cw * code.k, dtype=torch.uint8, device="cuda")
        eng.decode_device(cw, code_ids, d_llr, llr_off, info, info_off, stream=torch.cuda.current_stream(),
                          d_protection=prot)
        torch.cuda.synchronize()
        assert got[rid].codewords == cw
        assert np.array_equal(out.reshape(-1), info.cpu().numpy()), r
    good = sum(np.array_equal(out.reshape(3, -1)[i], b.info[3 * r + i])
               for r, (_, _, out) in enumerate(iq_reqs) for i in range(3))
    assert good >= 9
    from sicc_gb300.pipeline import wait_timeouts
    assert wait_timeouts() == 0
    lp.close()


def test_device_loop_serves_requests_arriving_as_it_goes_idle(cuda, oracle):
    """With a 1 ms idle timeout and gaps of 0-3 ms between requests, many requests arrive while the loop
    is deciding to end: each one is served (by the running loop or by a relaunch) and none is left behind."""
    c = codes.short_code()
    lp = _loop([c], max_batch_codewords=64, max_batch_llr_floats=64 * 128, ring_requests=64, idle_timeout_ms=1,
               lanes=2)
    lp.start()
    rng = np.random.default_rng(5)
    llr = _pinned_llrs(c, 8, 2.5, 91)
    want = _expected(oracle, c, llr, 1)
    outs, ids, got = [], set(), {}
    for r in range(150):
        req, x, out = lp.request(0, llr, protection=1, tag=r)
        rid = lp.submit_request(req, keep=(x, out))
        assert rid is not None  # completions are drained below, so the rings never fill
        outs.append(out)
        ids.add(rid)
        time.sleep(float(rng.uniform(0.0, 0.003)))
        for d in lp.poll(wait_us=0):
            got[d.request_id] = d
    t0 = time.time()
    while len(got) < len(ids) and time.time() - t0 < 30:
        for d in lp.poll(wait_us=100000):
            got[d.request_id] = d
    assert set(got) == ids
    st = lp.stats()
    assert st.launches >= 2  # the loop did end and start again along the way
    assert st.busy_iterations <= st.iterations and st.busy_iterations >= 1
    for out in outs:
        assert np.array_equal(out, want)
    lp.close()
