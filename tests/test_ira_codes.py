"""Host checks of the long irregular repeat-accumulate codes (DVB-S2 frame sizes).

The synthetic codes must have the shapes of the reference's DVB-S2 matrices
(data/code_matrices/Code_Matrices_Lib/LDPC/DVB_S2_*.alist, exported by
source/matlab/uhd_cpp/matlab/export_dvbs2_alist.m): length, dimension, edge
count and column-degree distribution.  Where the reference tree is present the
comparison reads those files; the numbers are also written here so the test
runs without it.
"""
import os

import numpy as np
import pytest

from sicc_gb300 import channel, codes

from oracle import ref_root

REF_LDPC = os.path.join(ref_root(), "data", "code_matrices", "Code_Matrices_Lib", "LDPC")
# (profile, reference alist file, edges, {column degree: columns})
SHAPES = [
    ("N64800_R1/2", "DVB_S2_N64800_R12.alist", 226799, {1: 1, 2: 32399, 3: 19440, 8: 12960}),
    ("N16200_R1/4", "DVB_S2_short_N16200_rate_1_4.alist", 48599, {1: 1, 2: 12959, 3: 1800, 12: 1440}),
    ("N16200_R1/2", "DVB_S2_short_N16200_rate_1_2.alist", 48599, {1: 1, 2: 8999, 3: 5400, 8: 1800}),
    ("N16200_R5/6", "DVB_S2_short_N16200_rate_5_6.alist", 49319, {1: 1, 2: 2879, 3: 12960, 13: 360}),
]


def _column_degrees(n, col_ind):
    deg = np.bincount(col_ind, minlength=n)
    vals, counts = np.unique(deg, return_counts=True)
    return {int(v): int(c) for v, c in zip(vals, counts)}


@pytest.mark.parametrize("name,alist,edges,coldeg", SHAPES)
def test_shape_matches_the_dvbs2_matrix(name, alist, edges, coldeg):
    c = codes.dvbs2_code(name)
    assert c.edges == edges
    assert _column_degrees(c.n, c.col_ind) == coldeg
    path = os.path.join(REF_LDPC, alist)
    if os.path.exists(path):
        n, m, rp, ci = codes.read_alist(path)
        assert (n, m) == (c.n, c.m) and int(rp[-1]) == edges
        assert _column_degrees(n, ci) == coldeg


@pytest.mark.parametrize("name", list(codes.DVBS2_PROFILES))
def test_encoded_words_satisfy_every_check(name):
    c = codes.dvbs2_code(name)
    info, cw, llr = channel.awgn_llrs(c, 3, 2.0, seed=5)
    assert np.array_equal(cw[:, : c.k], info)
    rows = np.repeat(np.arange(c.m), np.diff(c.row_ptr))
    for x in cw:
        par = np.bincount(rows, weights=x[c.col_ind].astype(np.float64), minlength=c.m).astype(np.int64) & 1
        assert not par.any()
    assert llr.shape == (3, c.n) and llr.dtype == np.float32


def test_rows_are_balanced_and_sorted():
    c = codes.dvbs2_code("N64800_R1/2")
    deg = np.diff(c.row_ptr)
    assert set(deg.tolist()) <= {6, 7}  # 5 information bits per row, 2 parity (the first row: 1)
    for r in (0, 1, 777, c.m - 1):
        row = c.col_ind[c.row_ptr[r]:c.row_ptr[r + 1]]
        assert np.all(np.diff(row) > 0)
        assert row[-1] == c.k + r and (r == 0 or row[-2] == c.k + r - 1)


def test_seeded_and_reproducible():
    a, b = codes.dvbs2_code("N16200_R1/2"), codes.dvbs2_code("N16200_R1/2")
    assert np.array_equal(a.col_ind, b.col_ind)
    other = codes.dvbs2_code("N16200_R1/2", seed=codes.IRA_CODE_SEED + 1)
    assert not np.array_equal(a.col_ind, other.col_ind)


def test_oracle_decodes_a_long_code(oracle):
    """The oracle the long-code GPU tests compare against: a noiseless frame in one pass, a noisy
    one to the transmitted word, both schedules the GPU tests use."""
    c = codes.dvbs2_code("N16200_R1/2")
    oc = oracle.code(c.n, c.m, c.row_ptr, c.col_ind)
    order, _, ncolors = oc.color_order()
    assert 1 < ncolors <= 64
    info, cw, llr = channel.awgn_llrs(c, 1, 30.0, seed=11)
    ok, bits, _, _, it, _ = oc.layered(llr[0], 25, 0.75, row_order=order)
    assert ok and it == 1 and np.array_equal(bits, cw[0])
    info, cw, llr = channel.awgn_llrs(c, 1, 2.5, seed=12)
    ok, bits, _, _, it, _ = oc.layered(llr[0], 25, 0.75, row_order=order)
    assert ok and np.array_equal(bits, cw[0])
    ok, bits, _, _, it, _ = oc.flooding(llr[0], 40, 0.8, 0.15, 0.0)
    assert ok and np.array_equal(bits, cw[0])
