"""Error-rate statistics for decoder comparisons on identical frames.

Frame error rate (FER): a frame is in error when any of its information bits
differs from what was sent.  Its 95% interval is the Wilson score interval,
which stays inside [0, 1] and is accurate at the small error counts of high
Eb/N0 points.

Bit error rate (BER): information-bit errors over information bits.  Bits of
one frame fail together (a decoder failure flips many at once), so the bits
are not independent draws; the interval treats frames as the sampling unit
(ratio estimator: total errors over total bits, with the variance of the
per-frame error counts), which is wider than a per-bit binomial interval and
honest about that clustering.

Two decoders run on the same frames are also compared pairwise: the frames
only one of them gets wrong (McNemar's discordant pairs) tell whether their
error rates differ by more than chance, without the noise of the shared
channel draws.
"""
from __future__ import annotations

import math

import numpy as np

Z95 = 1.959963984540054


def wilson(errors: int, trials: int, z: float = Z95) -> tuple[float, float, float]:
    """(rate, low, high) of the Wilson score interval for `errors` out of `trials`."""
    if trials <= 0:
        return 0.0, 0.0, 1.0
    p = errors / trials
    z2 = z * z
    den = 1.0 + z2 / trials
    centre = (p + z2 / (2 * trials)) / den
    half = z * math.sqrt(p * (1 - p) / trials + z2 / (4 * trials * trials)) / den
    return p, max(0.0, centre - half), min(1.0, centre + half)


def frame_errors(decoded: np.ndarray, sent: np.ndarray) -> np.ndarray:
    """Per-frame information-bit error counts of `decoded` [F][k] against `sent` [F][k]."""
    d = np.asarray(decoded).reshape(len(sent), -1)
    s = np.asarray(sent).reshape(len(sent), -1)
    return np.count_nonzero(d != s, axis=1)


def ber_interval(errors_per_frame: np.ndarray, bits_per_frame: int, z: float = Z95) -> tuple[float, float, float]:
    """(BER, low, high) with frames as the sampling unit (cluster-robust normal interval)."""
    e = np.asarray(errors_per_frame, dtype=np.float64)
    f = e.size
    if f == 0:
        return 0.0, 0.0, 1.0
    ber = float(e.sum()) / (f * bits_per_frame)
    if f < 2:
        return ber, 0.0, 1.0
    per = e / bits_per_frame
    half = z * float(np.std(per, ddof=1)) / math.sqrt(f)
    return ber, max(0.0, ber - half), min(1.0, ber + half)


def rate_summary(decoded: np.ndarray, sent: np.ndarray) -> dict:
    """FER and BER of one decoder on a set of frames, each with its 95% interval."""
    errs = frame_errors(decoded, sent)
    f = errs.size
    k = int(np.asarray(sent).reshape(f, -1).shape[1]) if f else 0
    fe = int(np.count_nonzero(errs))
    fer, flo, fhi = wilson(fe, f)
    ber, blo, bhi = ber_interval(errs, max(k, 1))
    return {"frames": f, "frame_errors": fe, "fer": fer, "fer_ci95": [flo, fhi],
            "bit_errors": int(errs.sum()), "ber": ber, "ber_ci95": [blo, bhi]}


def mcnemar(fail_a: np.ndarray, fail_b: np.ndarray) -> dict:
    """Paired comparison of two decoders' frame failures on the same frames.

    Returns the discordant counts (only A fails, only B fails) and the two-sided
    exact binomial p-value of the hypothesis that both decoders fail equally often.
    """
    a = np.asarray(fail_a, dtype=bool)
    b = np.asarray(fail_b, dtype=bool)
    only_a = int(np.count_nonzero(a & ~b))
    only_b = int(np.count_nonzero(b & ~a))
    n = only_a + only_b
    if n == 0:
        return {"only_a": 0, "only_b": 0, "p_value": 1.0}
    lo = min(only_a, only_b)
    # two-sided exact test: 2 * P(X <= lo), X ~ Binomial(n, 1/2), summed in log space
    logs = [math.lgamma(n + 1) - math.lgamma(i + 1) - math.lgamma(n - i + 1) - n * math.log(2.0)
            for i in range(lo + 1)]
    mx = max(logs)
    tail = math.exp(mx) * sum(math.exp(x - mx) for x in logs)
    return {"only_a": only_a, "only_b": only_b, "p_value": min(1.0, 2.0 * tail)}


def inside(value: float, interval) -> bool:
    return interval[0] <= value <= interval[1]
