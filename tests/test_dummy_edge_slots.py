"""Empty edge slots on a +inf dummy posterior leave the layered NMS unchanged (no GPU).

The layered BP kernels unroll a check row to D edge slots.  A row shorter than D
points its missing slots at a dummy posterior held at +inf instead of testing each
slot (bp_kernels.cu, engine.cu, bp_wide.cu): such a slot's extrinsic input is +inf,
so it never becomes a row minimum, the argmin or a sign, never flips a parity, and
its own update leaves it at +inf.  This test restates that slot arithmetic on the
host, single-precision operation by operation in the kernels' form (compressed
messages, fminf/fmaxf minima, first strict argmin), and checks it bit for bit
against the oracle's row-sequential layered decoder, which has no empty slots, on
codes with irregular row degrees and on zero, signed-zero, tied and infinite LLRs.
"""
import numpy as np
import pytest

F32 = np.float32
FLT_MAX = F32(np.finfo(np.float32).max)


def _nms(alpha, beta, mn):
    a = F32(alpha) * mn
    if beta == 0.0:
        return a
    d = a - F32(beta)
    return d if d > F32(0.0) else F32(0.0)


def _layered_with_dummy(n, rows, order, llr, max_iter, alpha, beta, slots):
    """The kernels' row update over `slots` edge slots per row, empty slots on app[n] = +inf."""
    dummy = n
    app = np.empty(n + 1, np.float32)
    app[:n] = llr
    app[dummy] = np.inf
    vr = [list(r) + [dummy] * (slots - len(r)) for r in rows]
    m1r = [F32(0.0)] * len(rows)
    m2r = [F32(0.0)] * len(rows)
    mr = [0] * len(rows)

    def weight():
        return sum(sum(1 for v in r if app[v] < F32(0.0)) & 1 for r in vr)

    def rebuild(i, j):
        mag = m2r[i] if j == (mr[i] >> 27) else m1r[i]
        return -mag if (mr[i] >> j) & 1 else mag

    best_w = weight()
    best = app[:n].copy()
    used = 0
    for it in range(max_iter):
        used = it + 1
        for i in order:
            q = []
            m1 = m2 = FLT_MAX
            idx, neg = 0, 0
            for j, v in enumerate(vr[i]):
                qj = F32(app[v] - rebuild(i, j))
                q.append(qj)
                neg |= (1 << j) if qj < F32(0.0) else 0
                a = F32(abs(qj))
                idx = j if a < m1 else idx
                m2 = min(m2, max(m1, a))
                m1 = min(m1, a)
            tot = bin(neg).count("1") & 1
            n1, n2 = _nms(alpha, beta, m1), _nms(alpha, beta, m2)
            nm = ((neg ^ -tot) & 0x07FFFFFF) | (idx << 27)
            for j, v in enumerate(vr[i]):
                mag = n2 if j == idx else n1
                app[v] = F32(q[j] + (-mag if (nm >> j) & 1 else mag))
            m1r[i], m2r[i], mr[i] = n1, n2, nm
        assert np.isposinf(app[dummy])  # the dummy never leaves +inf
        w = weight()
        if w < best_w:
            best_w = w
            best = app[:n].copy()
        if w == 0:
            break
    return (app[:n] < 0).astype(np.uint8), app[:n].copy(), best, used, best_w


def _irregular_code(n, m, dmin, dmax, seed):
    rng = np.random.default_rng(seed)
    rows = [sorted(rng.choice(n, size=int(rng.integers(dmin, dmax + 1)), replace=False).tolist()) for _ in range(m)]
    row_ptr = np.zeros(m + 1, np.int32)
    row_ptr[1:] = np.cumsum([len(r) for r in rows])
    col_ind = np.array([v for r in rows for v in r], np.int32)
    return rows, row_ptr, col_ind


def _frames(n, count, seed):
    rng = np.random.default_rng(seed)
    x = (1.0 - 2.0 * rng.integers(0, 2, (count, n))) * 2.0 + rng.normal(0.0, 1.6, (count, n))
    x = x.astype(np.float32)
    x[0::4] = np.round(x[0::4] * 2.0) / 2.0     # quantised: ties among |q|
    x[1::4, ::7] = 0.0                          # erasures
    x[2::4, 3::11] = -0.0                       # signed zeros
    x[3::4, 5] = np.inf                         # saturated LLRs
    x[3::4, 9] = -np.inf
    return x


@pytest.mark.parametrize("beta", [0.0, 0.25])
@pytest.mark.parametrize("seed", [1, 2])
def test_dummy_slots_match_the_oracle_layered_decoder(oracle, seed, beta):
    n, m = 60, 30
    rows, row_ptr, col_ind = _irregular_code(n, m, 2, 7, seed)
    oc = oracle.code(n, m, row_ptr, col_ind, systematic_front=False)
    order = np.random.default_rng(seed + 10).permutation(m).astype(np.int32)
    for x in _frames(n, 12, seed + 20):
        ok, bits, app, best, it, bw = oc.layered(x, 12, 0.75, beta, row_order=order)
        g_bits, g_app, g_best, g_it, g_bw = _layered_with_dummy(n, rows, order.tolist(), x, 12, 0.75, beta, 9)
        assert g_it == it and g_bw == bw
        assert np.array_equal(g_bits, bits)
        assert np.array_equal(g_app.view(np.uint32), app.view(np.uint32))
        assert np.array_equal(g_best.view(np.uint32), best.view(np.uint32))
