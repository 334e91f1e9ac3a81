"""Mixed-code batched decoding against the single-code decoders and the oracle.

A batch mixing the 15 codes of the mixed workload (lengths 128..2048, three
rates) plus the (128,64) code decodes in one persistent launch; every codeword
must come out exactly as the single-code flat-layered decoder (itself
bit-exact with the oracle) produces it: information bits, success flag and
iteration count.  With the OSD fallback on, codes the OSD kernel covers must
match the oracle's BP -> OSD chain bit for bit.
"""
import numpy as np
import pytest

from sicc_gb300 import channel, codes, engine, fec

pytestmark = pytest.mark.gpu


def _upload(torch, w):
    d = dict(code=torch.from_numpy(w.code_of).cuda(), llr=torch.from_numpy(w.llr).cuda(),
             llr_off=torch.from_numpy(w.llr_off).cuda(), info_off=torch.from_numpy(w.info_off).cuda())
    d["info"] = torch.full((w.info_bits,), 0xAA, dtype=torch.uint8, device="cuda")
    d["ok"] = torch.full((w.count,), 0xAA, dtype=torch.uint8, device="cuda")
    d["used"] = torch.full((w.count,), 0xAA, dtype=torch.uint8, device="cuda")
    d["it"] = torch.zeros(w.count, dtype=torch.uint8, device="cuda")
    return d


def _decode(torch, eng, w, d):
    eng.decode_device(w.count, d["code"], d["llr"], d["llr_off"], d["info"], d["info_off"], d["ok"], d["used"], d["it"],
                      stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    return d["info"].cpu().numpy(), d["ok"].cpu().numpy(), d["used"].cpu().numpy(), d["it"].cpu().numpy()


def test_mixed_batch_matches_single_code_decoders(cuda):
    torch = cuda
    cs = codes.mixed_codes() + [codes.short_code()]
    w = engine.mixed_workload(total=2500, seed=11, max_burst=48, code_set=cs)
    eng = engine.Engine(max_codewords=w.count, max_llr_floats=w.llr.size)
    ids = [eng.add_code(c, engine.iteration_cap(c.n)) for c in cs]
    assert ids == list(range(len(cs)))
    info, ok, used, it = _decode(torch, eng, w, _upload(torch, w))
    assert np.all(used == 0)
    for ci, c in enumerate(cs):
        sel = np.nonzero(w.code_of == ci)[0]
        if sel.size == 0:
            continue
        llr = np.stack([w.llr[w.llr_off[i]:w.llr_off[i] + c.n] for i in sel])
        dec = fec.CsrBpDecoder.for_code(c, max_batch=sel.size, max_iter=engine.iteration_cap(c.n), normalization=0.75)
        bits, sok, _ = dec.decode(llr)
        d_it = torch.zeros(sel.size, dtype=torch.uint8, device="cuda")
        dec.decode_device_batch(torch.from_numpy(llr).cuda(), None, None, None, d_it)
        torch.cuda.synchronize()
        for j, i in enumerate(sel):
            got = info[w.info_off[i]:w.info_off[i] + c.k]
            assert np.array_equal(got, bits[j, : c.k]), (c.name(), i)
            assert ok[i] == sok[j] and it[i] == d_it[j].item(), (c.name(), i)


def test_mixed_batch_with_osd_matches_oracle(cuda, oracle):
    torch = cuda
    cs = [c for c in codes.mixed_codes() if engine.osd_supported(c)] + [codes.qc_code(8, 16, 64, 5)]
    assert len(cs) >= 4
    w = engine.mixed_workload(total=900, seed=12, max_burst=40, code_set=cs, ebn0_range=(1.0, 3.0))
    eng = engine.Engine(max_codewords=w.count, max_llr_floats=w.llr.size)
    for c in cs:
        eng.add_code(c, engine.iteration_cap(c.n), osd_order=2 if engine.osd_supported(c) else -1)
    info, ok, used, it = _decode(torch, eng, w, _upload(torch, w))
    assert used.sum() > 50
    tables = {}
    for i in range(w.count):
        c = cs[w.code_of[i]]
        key = w.code_of[i]
        if key not in tables:
            oc = oracle.code(c.n, c.m, c.row_ptr, c.col_ind)
            tables[key] = (oc, oc.systematic_parity())
        oc, table = tables[key]
        x = w.llr[w.llr_off[i]:w.llr_off[i] + c.n]
        r = oc.layered(x, engine.iteration_cap(c.n), 0.75)
        if r[0] or not engine.osd_supported(c):
            exp = r[1][: c.k]
            assert used[i] == 0
        else:
            exp = oracle.osd(table, c.n, c.k, r[3], 2, 64, 4096)[0][: c.k]
            assert used[i] == 1
        assert np.array_equal(info[w.info_off[i]:w.info_off[i] + c.k], exp), (c.name(), i)


def test_unregistered_code_ids_are_skipped(cuda):
    torch = cuda
    c = codes.short_code()
    eng = engine.Engine(max_codewords=64, max_llr_floats=64 * 128)
    eng.add_code(c, 20)
    _, _, llr = channel.awgn_llrs(c, 64, 3.0, seed=2)
    code_of = np.zeros(64, np.uint8)
    code_of[::2] = 7  # not registered
    w = engine.MixedWorkload(codes=[c], req_code=np.zeros(1, np.int32), req_start=np.array([0, 64]), code_of=code_of,
                             llr=llr.reshape(-1), llr_off=np.arange(64, dtype=np.int64) * 128, info=[],
                             info_true=np.zeros(64 * 64, np.uint8), info_off=np.arange(64, dtype=np.int64) * 64,
                             ebn0=np.full(64, 3.0))
    info, ok, used, it = _decode(torch, eng, w, _upload(torch, w))
    assert np.all(ok[::2] == 0xAA) and np.all(ok[1::2] <= 1)
    assert np.all(info.reshape(64, 64)[::2] == 0xAA)
