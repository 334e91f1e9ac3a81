"""The continuous-batching decode service against decoding each request alone.

A codeword's result must not depend on the batch it lands in: every request
submitted into a concurrent mixed stream (several codes, BP-only and BP+OSD
protection, OFDM IQ requests that are demodulated first) must come back with
the bits the oracle's BP -> OSD chain gives for it alone (LLR requests), or
that the pipeline's batched demodulator followed by the mixed engine give for
it alone (IQ requests; both are kernel paths already pinned to the oracle).
"""
import numpy as np
import pytest

from sicc_gb300 import channel, codes, engine, ofdm

pytestmark = pytest.mark.gpu


def _codes():
    cs = [c for c in codes.mixed_codes() if engine.osd_supported(c)][:3] + [codes.short_code()]
    cs.append(next(c for c in codes.mixed_codes() if c.n == 1024))
    return cs


def _server(cs, budget=256 << 20, **kw):
    from sicc_gb300.server import Server
    srv = Server(hbm_budget_bytes=budget, **kw)
    for c in cs:
        srv.add_code(c, engine.iteration_cap(c.n), osd_order=2 if engine.osd_supported(c) else -1)
    return srv


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


def test_mixed_stream_matches_requests_decoded_alone(cuda, oracle):
    cs = _codes()
    srv = _server(cs, max_batch_codewords=4096, max_inflight_batches=3)
    srv.start()
    rng = np.random.default_rng(5)
    reqs = []
    for r in range(40):
        ci = int(rng.integers(0, len(cs)))
        cnt = int(rng.integers(1, 40))
        _, _, llr = channel.awgn_llrs(cs[ci], cnt, rng.uniform(1.0, 3.5, cnt), seed=900 + r)
        prot = int(rng.integers(0, 2))
        rid, out = srv.submit(0, ci, llr, protection=prot, tag=r)
        while rid is None:
            srv.poll(wait_us=100)
            rid, out = srv.submit(0, ci, llr, protection=prot, tag=r)
        reqs.append((ci, llr, prot, rid, out))
    done = {}
    while len(done) < len(reqs):
        for d in srv.poll(wait_us=200000):
            done[d.request_id] = d
    st = srv.stats()
    assert st.completed == len(reqs) and st.batches >= 1
    assert st.arena_bytes_in_use == 0
    for ci, llr, prot, rid, out in reqs:
        c = cs[ci]
        d = done[rid]
        assert d.status == 0 and d.codewords == llr.shape[0]
        assert d.latency_us >= d.queue_us >= 0.0
        assert np.array_equal(out, _expected(oracle, c, llr, prot)), (c.name(), rid)
        if not prot or not engine.osd_supported(c):
            assert d.osd_codewords == 0
    srv.close()


def test_small_arena_admits_first_in_first_out(cuda, oracle):
    c = codes.short_code()
    budget = 1 << 20
    srv = _server([c], budget=budget, max_batch_codewords=1024, max_inflight_batches=2, max_pending_requests=4)
    srv.start()
    per = 1000  # 1000 x (128 x 4 + 64) bytes = 0.55 MiB: at most one request resident at a time
    reqs = []
    for r in range(12):
        _, _, llr = channel.awgn_llrs(c, per, 2.5, seed=70 + r)
        reqs.append(srv.request(0, 0, llr, protection=1, tag=r))
    res, wall = srv.replay(reqs, np.zeros(len(reqs)))
    assert wall > 0
    st = srv.stats()
    assert st.completed == len(reqs) and st.arena_bytes_peak <= budget
    for (req, llr, out), d in zip(reqs, res):
        assert d.tag == req.tag and d.status == 0
        assert np.array_equal(out, _expected(oracle, c, llr, 1))
    # admission follows submission order, so queueing delays do not decrease much out of order
    q = np.array([d.queue_us for d in res])
    assert q[-1] >= q[0]
    srv.close()


def test_request_validation(cuda):
    from sicc_gb300 import _lib
    c = codes.short_code()
    srv = _server([c], budget=1 << 20, max_batch_codewords=256)
    _, _, llr = channel.awgn_llrs(c, 8, 3.0, seed=1)
    with pytest.raises(_lib.SiccError):
        srv.submit(0, 0, llr)  # not started
    srv.start()
    from sicc_gb300.server import Request
    out = np.zeros((8, c.k), np.uint8)
    bad = Request(kind=0, code_id=5, phy_id=-1, count=8, protection=0, host_input=llr.ctypes.data,
                  host_info=out.ctypes.data, tag=0)
    with pytest.raises(_lib.SiccError):
        srv.submit_request(bad)  # unknown code
    bad.code_id, bad.kind = 0, 2
    with pytest.raises(_lib.SiccError):
        srv.submit_request(bad)  # unknown kind
    with pytest.raises(_lib.SiccError):
        srv.submit(0, 0, np.zeros((300, c.n), np.float32))  # more than max_batch_codewords
    rid, out = srv.submit(0, 0, llr)
    assert rid is not None
    while not srv.poll(wait_us=100000):
        pass
    srv.close()


def test_iq_requests_match_pipeline_then_engine(cuda):
    torch = cuda
    from sicc_gb300.pipeline import RxPipeline, SYNC_RECORD
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    code = codes.short_code()
    gen = ofdm.FrameGenerator(t, code, seed=77)
    blocks = gen.blocks
    b = gen.batch(12, snr_db=14.0, cfo_subcarriers=0.1, max_offset=100)
    stride = b.iq.shape[1]
    nv = float(np.float32(np.mean(b.noise_var)))
    cs = _codes()
    srv = _server(cs, max_batch_codewords=4096)
    cid = len(cs) - 2  # the short code
    assert cs[cid].n == code.n and cs[cid].k == code.k
    pid = srv.add_phy(t, cid, blocks, nv, stride)
    srv.start()
    # IQ requests interleaved with LLR requests of other codes
    iq_reqs = []
    rng = np.random.default_rng(3)
    for r in range(4):
        sl = b.iq[3 * r: 3 * r + 3]
        iq_reqs.append((sl, *srv.submit(1, pid, sl, protection=r % 2)))
        _, _, llr = channel.awgn_llrs(cs[0], 16, 2.0, seed=r)
        srv.submit(0, 0, llr, protection=1)
    want = {rid for _, rid, _ in iq_reqs}
    got = {}
    while not want <= set(got):
        for d in srv.poll(wait_us=200000):
            got[d.request_id] = d
    # alone: batched demodulation, then the mixed engine with the same protection
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
    # most frames decode to the transmitted bits at this SNR
    good = sum(np.array_equal(out.reshape(3, -1)[i], b.info[3 * r + i])
               for r, (_, _, out) in enumerate(iq_reqs) for i in range(3))
    assert good >= 9
    srv.close()
