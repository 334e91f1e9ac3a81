"""Pins the C oracle to the reference's own CPU receive path.

Every check compares oracle/sicc_oracle.c against outputs of the reference
code compiled from its sources (oracle/_ref): live where that build exists,
and always against the committed fixtures in tests/golden/ that it produced
(tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

from sicc_gb300 import codes, ofdm

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def fec():
    return dict(np.load(os.path.join(GOLDEN, "fec_short_code.npz")))


@pytest.fixture(scope="module")
def ofd():
    return dict(np.load(os.path.join(GOLDEN, "ofdm_small.npz")))


def test_code_construction_matches_reference(oracle, fec):
    code = codes.short_code()
    assert np.array_equal(code.row_ptr, fec["row_ptr"]) and np.array_equal(code.col_ind, fec["col_ind"])
    oc = oracle.code(code.n, code.m, code.row_ptr, code.col_ind)
    info, piv = oc.info_cols()
    assert np.array_equal(info, fec["info_cols"]) and np.array_equal(piv, fec["pivot_cols"])
    assert np.array_equal(oc.systematic_parity(), fec["parity"])
    for u, c in zip(fec["info"], fec["enc"]):
        assert np.array_equal(oc.encode(u), c)
        assert oc.syndrome_weight(c) == 0


@pytest.mark.parametrize("iters,norm,key", [(20, 0.75, "flood"), (8, 0.80, "flood8")])
def test_flooding_min_sum_matches_reference(oracle, fec, iters, norm, key):
    code = codes.short_code()
    oc = oracle.code(code.n, code.m, code.row_ptr, code.col_ind)
    for i, llr in enumerate(fec["llr"]):
        ok, bits, app, it = oc.flooding_ref(llr, iters, norm)
        assert ok == bool(fec[key + "_ok"][i])
        assert it == fec[key + "_iter"][i]
        assert np.array_equal(bits, fec[key + "_bits"][i])
        # the generalised single-precision flooding reduces to it with no offset/damping
        ok2, bits2, app2, _, it2, _ = oc.flooding(llr, iters, norm)
        assert ok2 == ok and it2 == it and np.array_equal(bits2, bits) and np.array_equal(app2, app)


def test_ccsds_default_code_parity_table(oracle, fec):
    n, m = 128, 64
    oc = oracle.code(n, m, fec["ccsds_row_ptr"], fec["ccsds_col_ind"])
    assert oc.k == 64
    assert np.array_equal(oc.systematic_parity(), fec["ccsds_parity"])


def test_fft_matches_reference(oracle, ofd):
    out = oracle.fft_shifted(ofd["fft_in"])
    assert np.array_equal(out, ofd["fft_out"])


def test_maxlog_llr_matches_reference(oracle, ofd):
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    ph = oracle.phy(t)
    out = oracle.llr_maxlog(ph, ofd["llr_pts"], ofd["llr_sig2"])
    assert np.array_equal(out, ofd["llr_out"])


def test_sync_matches_reference(oracle, ofd):
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    ph = oracle.phy(t)
    for i in range(ofd["iq"].shape[0]):
        r = oracle.sync_earliest(ph, ofd["iq"][i][: ofd["lengths"][i]])
        exp = ofd["sync"][i]
        assert r[0] == int(exp[0])
        if r[0] == 1:
            assert r[1] == int(exp[1])
            assert r[2] == pytest.approx(exp[2], rel=1e-12)
            assert r[3] == pytest.approx(exp[3], rel=1e-12)
            assert r[4] == pytest.approx(exp[4], rel=1e-9, abs=1e-9)


def test_demod_and_decode_match_reference(oracle, ofd):
    t = ofdm.reference_tables(ofdm.OFDM_SMALL)
    ph = oracle.phy(t)
    code = codes.short_code()
    oc = oracle.code(code.n, code.m, code.row_ptr, code.col_ind)
    flen = t.frame_len
    for i in range(ofd["iq"].shape[0]):
        found, start, _, _, cfo = ofd["sync"][i]
        if int(found) != 1:
            continue
        start = int(start)
        llr = oracle.demod_frame(ph, ofd["iq"][i][start:start + flen], cfo, ofd["noise_var"][i])
        blocks = llr.size // code.n
        bits = np.concatenate([oc.flooding_ref(llr[b * code.n:(b + 1) * code.n], 25, 0.75)[1][: code.k]
                               for b in range(blocks)])
        assert np.array_equal(bits, ofd["decoded"][i])


def test_live_reference_agrees_on_new_inputs(oracle, reference):
    """Fresh seeded inputs against the compiled reference (skipped where it is absent)."""
    code = codes.qc_code(8, 16, 16, 99)
    rc = reference.code(code.n, code.m, code.row_ptr, code.col_ind)
    oc = oracle.code(code.n, code.m, code.row_ptr, code.col_ind)
    assert np.array_equal(rc.systematic_parity(), oc.systematic_parity())
    from sicc_gb300 import channel
    _, _, llr = channel.awgn_llrs(code, 32, 1.5, seed=3)
    ok, bits, it = rc.decode_min_sum(llr, 15, 0.7)
    for i in range(32):
        o = oc.flooding_ref(llr[i], 15, 0.7)
        assert o[0] == ok[i] and o[3] == it[i] and np.array_equal(o[1], bits[i])
