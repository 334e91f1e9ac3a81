"""Host-side logic: code construction, channel inputs, tables, C-ABI surface."""
import ctypes as C
import os
import re
import tempfile

import numpy as np
import pytest

from sicc_gb300 import channel, codes, ofdm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_short_code_shape():
    c = codes.short_code()
    assert (c.n, c.m, c.k, c.z) == (128, 64, 64, 16)
    assert c.edges == 23 * 16
    deg = np.diff(c.row_ptr)
    assert sorted(set(deg.tolist())) == [5, 6]
    for r in range(c.m):
        row = c.col_ind[c.row_ptr[r]:c.row_ptr[r + 1]]
        assert np.all(np.diff(row) > 0)


def test_codes_are_seeded_and_systematic(oracle):
    a, b = codes.short_code(), codes.short_code()
    assert np.array_equal(a.shifts, b.shifts)
    for c in [codes.short_code(), codes.ofdm_code()] + codes.mixed_codes()[:6]:
        oc = oracle.code(c.n, c.m, c.row_ptr, c.col_ind)
        info, _ = oc.info_cols()
        assert oc.k == c.k and np.array_equal(info, np.arange(c.k))
        P = channel.parity_matrix(c)
        assert np.array_equal(codes.unpack_parity_table(oc.systematic_parity(), c.n, c.k), P)


def test_mixed_code_set():
    cs = codes.mixed_codes()
    assert len(cs) == 15
    assert {c.n for c in cs} == set(codes.MIXED_LENGTHS)
    assert {round(c.rate, 4) for c in cs} == {0.5, 0.6875, 0.75}


def test_alist_round_trip():
    c = codes.short_code()
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "c.alist")
        codes.write_alist(p, c.n, c.m, c.row_ptr, c.col_ind)
        n, m, rp, ci = codes.read_alist(p)
    assert (n, m) == (c.n, c.m) and np.array_equal(rp, c.row_ptr) and np.array_equal(ci, c.col_ind)


def test_awgn_llr_convention():
    c = codes.short_code()
    info, cw, llr = channel.awgn_llrs(c, 2000, 6.0, seed=1)
    assert llr.dtype == np.float32
    s2 = channel.sigma2_for(c.rate, 6.0)
    # mean LLR of a 0 bit is 2/sigma^2 (BPSK +1), negative for 1 bits
    assert np.mean(llr[cw == 0]) == pytest.approx(2.0 / s2, rel=0.02)
    assert np.mean(llr[cw == 1]) == pytest.approx(-2.0 / s2, rel=0.02)
    assert info.shape == (2000, 64) and np.array_equal(cw[:, :64], info)


def test_ofdm_tables_match_reference_layout():
    t = ofdm.reference_tables(ofdm.OFDM_C3)
    assert t.coded_bits == 13 * 600 * 4 == 31200
    assert t.frame_len == 1024 + 14 * 1096
    assert list(t.pilot_symbols) == [0] and list(t.data_symbols) == list(range(1, 14))
    assert np.all(t.interp_p0 == 0) and np.all(t.interp_alpha == 0)
    assert len(t.used_indices) == 600 and 512 not in set(t.used_indices.tolist())
    assert np.allclose(np.mean(np.abs(t.constellation) ** 2), 1.0, atol=1e-6)


def _declared_symbols():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"SICC_API\s+[\w\s\*]+?\b(\w+)\s*\(", txt)
    return names


def test_library_exports_every_declared_symbol():
    from sicc_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from importlib import import_module
        import sys
        sys.path.insert(0, os.path.join(ROOT, "sicc-baseband-proto_gb300"))
        import_module("build").build()
    L = _lib.load()
    names = _declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_invalid_arguments_are_reported_without_a_gpu():
    from sicc_gb300 import _lib
    L = _lib.load()
    h = _lib.u64(0)
    assert L.cuda_osd_create_stream_decoder(None, C.byref(h)) == _lib.INVALID_ARGUMENT
    assert "null" in _lib.last_error()
    cfg = _lib.StreamConfig(n=128, k=60, m=64, max_batch_size=16, min_batch_size=1, bp_max_iterations=20)
    assert L.cuda_osd_create_stream_decoder(C.byref(cfg), C.byref(h)) == _lib.INVALID_ARGUMENT
    assert h.value == 0 and "n = k + m" in _lib.last_error()
    cfg = _lib.StreamConfig(n=512, k=256, m=256, max_batch_size=16, min_batch_size=1, bp_max_iterations=20)
    assert L.cuda_osd_create_stream_decoder(C.byref(cfg), C.byref(h)) == _lib.INVALID_ARGUMENT
    rp = np.array([0, 2, 5], np.int32)
    ci = np.array([0, 1, 1, 2, 3], np.int32)
    bad = _lib.BpCsrConfig(n=4, m=2, max_batch_size=8, max_iterations=10, normalization=0.75, nnz=4, schedule=3)
    assert L.cuda_osd_create_bp_csr_decoder(C.byref(bad), rp.ctypes.data, ci.ctypes.data, C.byref(h)) == \
        _lib.INVALID_ARGUMENT
    assert "nnz" in _lib.last_error()
    assert L.cuda_osd_destroy_stream_decoder(12345) == _lib.INVALID_ARGUMENT
    assert L.cuda_osd_flush(0) == _lib.INVALID_ARGUMENT
