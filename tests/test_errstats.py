"""Host statistics used by the error-rate parity checks (no GPU)."""
import numpy as np
import pytest

from sicc_gb300 import errstats


def test_wilson_matches_scipy():
    stats = pytest.importorskip("scipy.stats")
    for k, n in [(0, 10), (3, 10), (10, 10), (6947, 65536), (902, 65536), (1, 1024)]:
        p, lo, hi = errstats.wilson(k, n)
        ci = stats.binomtest(k, n).proportion_ci(confidence_level=0.95, method="wilson")
        assert p == k / n
        assert lo == pytest.approx(ci.low, abs=1e-12) and hi == pytest.approx(ci.high, abs=1e-12)


def test_mcnemar_exact_matches_binomtest():
    stats = pytest.importorskip("scipy.stats")
    rng = np.random.default_rng(0)
    a = rng.random(5000) < 0.10
    b = a.copy()
    flip = rng.random(5000) < 0.03
    b[flip] = ~b[flip]
    r = errstats.mcnemar(a, b)
    n = r["only_a"] + r["only_b"]
    assert r["p_value"] == pytest.approx(stats.binomtest(r["only_a"], n, 0.5).pvalue, rel=1e-9)
    assert errstats.mcnemar(a, a) == {"only_a": 0, "only_b": 0, "p_value": 1.0}


def test_rate_summary_counts_and_clustered_ber():
    sent = np.zeros((4, 8), np.uint8)
    dec = sent.copy()
    dec[1, :4] = 1  # one frame with 4 bit errors
    dec[3, 0] = 1   # one frame with 1 bit error
    s = errstats.rate_summary(dec, sent)
    assert s["frames"] == 4 and s["frame_errors"] == 2 and s["bit_errors"] == 5
    assert s["fer"] == 0.5 and s["ber"] == 5 / 32
    lo, hi = s["ber_ci95"]
    # frames as the sampling unit: the interval comes from the per-frame error fractions
    per = np.array([0, 4, 0, 1]) / 8
    half = errstats.Z95 * per.std(ddof=1) / 2
    assert lo == pytest.approx(max(0.0, 5 / 32 - half)) and hi == pytest.approx(5 / 32 + half)
