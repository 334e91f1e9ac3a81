"""The CTA-per-codeword OSD (codes with n > 256 or k > 128) against the oracle.

The oracle restates the reference's generator-based OSD (cpu_bp_osd_decode.m:
187-305); the kernel eliminates on H instead.  Both must give the same
codeword, the same winning metric and so the same information bits, bit for
bit: after BP (the engine's chain against the oracle's layered BP -> OSD), and
on soft values with many equal reliabilities (quantised LLRs straight into
OSD), where the sort order, the flip pool and the first-minimum rule decide.
"""
import numpy as np
import pytest

from sicc_gb300 import channel, codes, engine

pytestmark = pytest.mark.gpu


def _large_codes():
    mc = codes.mixed_codes()
    pick = [c for c in mc if c.n == 256 and c.k > 128]
    pick += [c for c in mc if c.n in (512, 1024, 2048)]
    return pick


def _tables(oracle, c):
    oc = oracle.code(c.n, c.m, c.row_ptr, c.col_ind)
    return oc, oc.systematic_parity()


def _upload(torch, code_ids, rows, ks):
    lo = np.concatenate([[0], np.cumsum([r.size for r in rows])[:-1]]).astype(np.int64)
    io = np.concatenate([[0], np.cumsum(ks)[:-1]]).astype(np.int64)
    d = dict(code=torch.from_numpy(np.asarray(code_ids, np.uint8)).cuda(),
             llr=torch.from_numpy(np.concatenate(rows).astype(np.float32)).cuda(),
             lo=torch.from_numpy(lo).cuda(), io=torch.from_numpy(io).cuda(),
             info=torch.full((int(np.sum(ks)),), 0xAA, dtype=torch.uint8, device="cuda"),
             used=torch.zeros(len(rows), dtype=torch.uint8, device="cuda"),
             metric=torch.zeros(len(rows), dtype=torch.float32, device="cuda"))
    return d, io


@pytest.mark.parametrize("order", [1, 2])
def test_bp_then_large_osd_matches_oracle(cuda, oracle, order):
    torch = cuda
    cs = _large_codes()
    eng = engine.Engine(max_codewords=512, max_llr_floats=512 * 2048)
    for c in cs:
        eng.add_code(c, engine.iteration_cap(c.n), osd_order=order)
    rows, ids, ks, llrs = [], [], [], []
    for ci, c in enumerate(cs):
        cnt = 6 if c.n >= 1024 else 10
        _, _, llr = channel.awgn_llrs(c, cnt, 1.2, seed=40 + ci)
        for x in llr:
            rows.append(x)
            ids.append(ci)
            ks.append(c.k)
    d, io = _upload(torch, ids, rows, ks)
    cnt = len(rows)
    ok = torch.zeros(cnt, dtype=torch.uint8, device="cuda")
    eng.decode_device(cnt, d["code"], d["llr"], d["lo"], d["info"], d["io"], ok, d["used"],
                      stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    info = d["info"].cpu().numpy()
    used = d["used"].cpu().numpy()
    tabs = {}
    n_osd = 0
    for i, (ci, x) in enumerate(zip(ids, rows)):
        c = cs[ci]
        if ci not in tabs:
            tabs[ci] = _tables(oracle, c)
        oc, table = tabs[ci]
        r = oc.layered(x, engine.iteration_cap(c.n), 0.75)
        if r[0]:
            exp = r[1][: c.k]
            assert used[i] == 0
        else:
            exp = oracle.osd(table, c.n, c.k, r[3], order, 64, 4096)[0][: c.k]
            assert used[i] == 1
            n_osd += 1
        assert np.array_equal(info[io[i]:io[i] + c.k], exp), (c.name(), i)
    assert n_osd >= 20


def test_large_osd_on_tied_reliabilities(cuda, oracle):
    torch = cuda
    cs = _large_codes()[:4]
    eng = engine.Engine(max_codewords=64, max_llr_floats=64 * 1024)
    for c in cs:
        eng.add_code(c, 20, osd_order=2)
    rows, ids, ks = [], [], []
    for ci, c in enumerate(cs):
        _, _, llr = channel.awgn_llrs(c, 5, 1.0, seed=70 + ci)
        for x in llr:
            rows.append((np.round(x * 2.0) / 2.0).astype(np.float32))  # many equal |llr|, some exact zeros
            ids.append(ci)
            ks.append(c.k)
    d, io = _upload(torch, ids, rows, ks)
    eng.osd_device(len(rows), d["code"], d["llr"], d["lo"], d["info"], d["io"], d["used"], d["metric"],
                   stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    info = d["info"].cpu().numpy()
    metric = d["metric"].cpu().numpy()
    assert np.all(d["used"].cpu().numpy() == 1)
    for i, (ci, x) in enumerate(zip(ids, rows)):
        c = cs[ci]
        _, table = _tables(oracle, c)
        code_bits, m, _, _ = oracle.osd(table, c.n, c.k, x, 2, 64, 4096)
        assert np.array_equal(info[io[i]:io[i] + c.k], code_bits[: c.k]), (c.name(), i)
        assert metric[i] == np.float32(m)


def test_short_and_long_osd_in_one_batch(cuda, oracle):
    """Warp-kernel and CTA-kernel codes share one hand-off list; each kernel takes its own."""
    torch = cuda
    cs = [codes.short_code()] + _large_codes()[1:3]
    eng = engine.Engine(max_codewords=64, max_llr_floats=64 * 1024)
    for c in cs:
        eng.add_code(c, 20, osd_order=2)
    rows, ids, ks = [], [], []
    for j in range(18):
        ci = j % len(cs)
        _, _, llr = channel.awgn_llrs(cs[ci], 1, 1.0, seed=90 + j)
        rows.append(llr[0])
        ids.append(ci)
        ks.append(cs[ci].k)
    d, io = _upload(torch, ids, rows, ks)
    eng.osd_device(len(rows), d["code"], d["llr"], d["lo"], d["info"], d["io"], d["used"], d["metric"],
                   stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    info = d["info"].cpu().numpy()
    for i, (ci, x) in enumerate(zip(ids, rows)):
        c = cs[ci]
        _, table = _tables(oracle, c)
        exp = oracle.osd(table, c.n, c.k, x, 2, 64, 4096)[0][: c.k]
        assert np.array_equal(info[io[i]:io[i] + c.k], exp), (c.name(), i)
