"""Quasi-cyclic LDPC codes used by the decoder workloads, plus alist I/O.

A code is described by a base matrix of ``mb x nb`` circulant slots lifted by
``Z``.  The information part (the first ``nb - mb`` base columns) is fully
populated and the parity part is dual-diagonal (lower bidiagonal): parity base
column ``j`` has circulants in base rows ``j`` and ``j + 1``.  Every populated
slot carries a cyclic shift drawn uniformly from ``[0, Z)`` by a NumPy PCG64
generator seeded with the code seed, in row-major slot order.  Circulant
``P^s`` puts row ``t`` of its block on column ``(t + s) mod Z``.

Because the parity part is block lower-triangular with permutation matrices on
the diagonal it is invertible over GF(2), so the codes are full rank with the
information bits first ("systematic-front"), which is the layout the
reference's BP-OSD entry points require
(source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp:3096-3118, 3189-3205).

Parity-check matrices are exchanged as CSR (``row_ptr``, ``col_ind``, columns
ascending within a row), the layout of the reference's ``CsrMatrix``
(source/cpp_cuda/uhd_cpp/src/fec_config.hpp:24-33) and of
``cuda_osd_create_bp_csr_decoder``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass(frozen=True)
class QcCode:
    """A lifted quasi-cyclic LDPC code (systematic-front, full rank)."""

    n: int
    m: int
    k: int
    z: int
    mb: int
    nb: int
    seed: int
    shifts: np.ndarray  # [mb, nb] int32, -1 = empty slot
    row_ptr: np.ndarray = field(repr=False)  # [m+1] int32
    col_ind: np.ndarray = field(repr=False)  # [E] int32

    @property
    def edges(self) -> int:
        return int(self.row_ptr[-1])

    @property
    def rate(self) -> float:
        return self.k / self.n

    def dense_h(self) -> np.ndarray:
        h = np.zeros((self.m, self.n), dtype=np.uint8)
        for r in range(self.m):
            h[r, self.col_ind[self.row_ptr[r]:self.row_ptr[r + 1]]] = 1
        return h

    def name(self) -> str:
        return f"qc({self.n},{self.k})z{self.z}s{self.seed}"


def dual_diagonal_base(mb: int, nb: int) -> np.ndarray:
    """Boolean slot-occupancy mask: full information block, lower bidiagonal parity."""
    if not (0 < mb < nb):
        raise ValueError("need 0 < mb < nb")
    kb = nb - mb
    present = np.zeros((mb, nb), dtype=bool)
    present[:, :kb] = True
    for j in range(mb):
        present[j, kb + j] = True
        if j + 1 < mb:
            present[j + 1, kb + j] = True
    return present


def qc_code(mb: int, nb: int, z: int, seed: int) -> QcCode:
    """Lift the dual-diagonal base matrix with seeded circulant shifts."""
    present = dual_diagonal_base(mb, nb)
    rng = np.random.default_rng(seed)
    draws = rng.integers(0, z, size=int(present.sum()))
    shifts = np.full((mb, nb), -1, dtype=np.int32)
    shifts[present] = draws.astype(np.int32)  # row-major slot order
    m, n = mb * z, nb * z
    row_ptr = np.zeros(m + 1, dtype=np.int32)
    cols = []
    for L in range(mb):
        slot_cols = np.nonzero(shifts[L] >= 0)[0]
        for t in range(z):
            r = L * z + t
            row = [int(c) * z + (t + int(shifts[L, c])) % z for c in slot_cols]
            cols.extend(row)
            row_ptr[r + 1] = row_ptr[r] + len(row)
    col_ind = np.asarray(cols, dtype=np.int32)
    return QcCode(n=n, m=m, k=n - m, z=z, mb=mb, nb=nb, seed=seed, shifts=shifts,
                  row_ptr=row_ptr, col_ind=col_ind)


# Workload codes -----------------------------------------------------------

#: Seed of the (128,64) code of the short-code BP and BP+OSD workloads.
SHORT_CODE_SEED = 20260101
#: Seed of the (1024,512) code of the OFDM receive workload.
OFDM_CODE_SEED = 20260102
#: Base seed of the mixed-code workload (code i uses MIXED_CODE_SEED + i).
MIXED_CODE_SEED = 20260200
#: Base-matrix row counts for the three mixed-workload rates over 16 base
#: columns: 1/2 -> 8 rows, "2/3" -> 5 rows (rate 11/16, the nearest integral
#: base shape), 3/4 -> 4 rows.
MIXED_RATE_ROWS = {"1/2": 8, "2/3": 5, "3/4": 4}
MIXED_LENGTHS = (128, 256, 512, 1024, 2048)


def short_code() -> QcCode:
    """QC (128,64): 4x8 base, Z = 16."""
    return qc_code(4, 8, 16, SHORT_CODE_SEED)


def ofdm_code() -> QcCode:
    """QC (1024,512): 8x16 base, Z = 64."""
    return qc_code(8, 16, 64, OFDM_CODE_SEED)


def mixed_codes() -> list[QcCode]:
    """The 15 codes of the mixed-length, mixed-rate workload (length-major)."""
    out = []
    i = 0
    for n in MIXED_LENGTHS:
        for rate, mb in MIXED_RATE_ROWS.items():
            out.append(qc_code(mb, 16, n // 16, MIXED_CODE_SEED + i))
            i += 1
    return out


# Long irregular repeat-accumulate codes -----------------------------------

@dataclass(frozen=True)
class IraCode:
    """An irregular repeat-accumulate LDPC code with the structure of the DVB-S2 codes.

    The information bits come in groups of 360.  Group g has a list of d_g
    base addresses x; bit j of the group (j < 360) joins the parity
    accumulators (x + j q) mod m for every x, q = m / 360 (the construction of
    ETSI EN 302 307 5.3.2).  The parity part is the accumulator chain:
    p_0 = s_0, p_r = p_{r-1} + s_r, so row r of H holds its information bits
    and parity columns k + r - 1 (r > 0) and k + r.  The base addresses are
    drawn from a NumPy PCG64 generator seeded with ``seed``, balanced over the
    q residues so every row gets the same number of information bits (up to
    one).  The degree profile is the standard's for the named frame and rate
    (information column degrees per group), the address tables are synthetic.
    """

    n: int
    m: int
    k: int
    q: int
    seed: int
    degrees: tuple  # information column degree of each 360-column group
    row_ptr: np.ndarray = field(repr=False)  # [m+1] int32
    col_ind: np.ndarray = field(repr=False)  # [E] int32
    label: str = ""

    @property
    def edges(self) -> int:
        return int(self.row_ptr[-1])

    @property
    def rate(self) -> float:
        return self.k / self.n

    def name(self) -> str:
        return f"ira({self.n},{self.k})s{self.seed}"

    def encode_bits(self, info: np.ndarray) -> np.ndarray:
        """Systematic-front codewords [B][n] of info [B][k] (uint8) through the accumulator."""
        info = np.asarray(info, np.uint8) & 1
        b = info.shape[0]
        rows = np.repeat(np.arange(self.m), np.diff(self.row_ptr))
        info_edges = self.col_ind < self.k
        cols = self.col_ind[info_edges]
        starts = np.searchsorted(rows[info_edges], np.arange(self.m))
        s = np.add.reduceat(info[:, cols].astype(np.int64), starts, axis=1) & 1
        empty = np.diff(np.append(starts, cols.size)) == 0
        s[:, empty] = 0
        parity = np.bitwise_xor.accumulate(s.astype(np.uint8), axis=1)
        return np.concatenate([info, parity], axis=1).astype(np.uint8).reshape(b, self.n)


#: Information-column degree profiles of DVB-S2 frames: (n, k, [(groups, degree), ...]).
DVBS2_PROFILES = {
    "N64800_R1/2": (64800, 32400, [(36, 8), (54, 3)]),
    "N16200_R1/4": (16200, 3240, [(4, 12), (5, 3)]),
    "N16200_R1/2": (16200, 7200, [(5, 8), (15, 3)]),
    "N16200_R5/6": (16200, 13320, [(1, 13), (36, 3)]),
}
#: Seed of the synthetic address tables of the long-code workload.
IRA_CODE_SEED = 20260300


def ira_code(n: int, k: int, profile, seed: int, label: str = "") -> IraCode:
    """Build an IRA code of length n, dimension k, information-group degrees ``profile``."""
    m = n - k
    if k % 360 or m % 360:
        raise ValueError("k and n - k must be multiples of 360")
    q = m // 360
    degrees = tuple(d for cnt, d in profile for _ in range(cnt))
    if len(degrees) != k // 360:
        raise ValueError("profile must cover k / 360 groups")
    rng = np.random.default_rng(seed)
    total = sum(degrees)
    residues = np.resize(rng.permutation(q), total)  # each residue (total / q) times, up to one
    rng.shuffle(residues)
    pairs_r, pairs_c = [], []
    at = 0
    j = np.arange(360)
    for g, d in enumerate(degrees):
        seen = set()
        for t in range(d):
            while True:
                x = int(residues[at + t]) + q * int(rng.integers(0, 360))
                if x not in seen:
                    break
            seen.add(x)
            pairs_r.append((x + j * q) % m)
            pairs_c.append(g * 360 + j)
        at += d
    r = np.concatenate(pairs_r + [np.arange(m), np.arange(1, m)])
    c = np.concatenate(pairs_c + [k + np.arange(m), k + np.arange(m - 1)])
    order = np.lexsort((c, r))
    r, c = r[order], c[order]
    row_ptr = np.zeros(m + 1, np.int32)
    np.add.at(row_ptr, r + 1, 1)
    row_ptr = np.cumsum(row_ptr).astype(np.int32)
    return IraCode(n=n, m=m, k=k, q=q, seed=seed, degrees=degrees, row_ptr=row_ptr,
                   col_ind=c.astype(np.int32), label=label)


def dvbs2_code(name: str, seed: int = IRA_CODE_SEED) -> IraCode:
    """Synthetic code with the DVB-S2 frame size, rate and degree profile ``name`` (see DVBS2_PROFILES)."""
    n, k, profile = DVBS2_PROFILES[name]
    return ira_code(n, k, profile, seed, label=name)


# alist I/O (format read by the reference: uhd_ldpc_ofdm_link.cpp:2722-2770,
# matrix_loader.cpp:13-87) ---------------------------------------------------

def write_alist(path: str, n: int, m: int, row_ptr: np.ndarray, col_ind: np.ndarray) -> None:
    rows = [list(col_ind[row_ptr[r]:row_ptr[r + 1]]) for r in range(m)]
    cols: list[list[int]] = [[] for _ in range(n)]
    for r, row in enumerate(rows):
        for c in row:
            cols[int(c)].append(r)
    max_cw = max(len(c) for c in cols)
    max_rw = max(len(r) for r in rows)
    with open(path, "w") as f:
        f.write(f"{n} {m}\n{max_cw} {max_rw}\n")
        f.write(" ".join(str(len(c)) for c in cols) + "\n")
        f.write(" ".join(str(len(r)) for r in rows) + "\n")
        for c in cols:
            f.write(" ".join(str(r + 1) for r in c + [-1] * (max_cw - len(c))).replace("-1", "0") + "\n")
        for r in rows:
            f.write(" ".join(str(int(c) + 1) for c in r + [-1] * (max_rw - len(r))).replace("-1", "0") + "\n")


def read_alist(path: str) -> tuple[int, int, np.ndarray, np.ndarray]:
    """Parse an alist into CSR with columns sorted and de-duplicated per row."""
    tok = open(path).read().split()
    it = iter(int(t) for t in tok)
    n, m = next(it), next(it)
    max_cw, max_rw = next(it), next(it)
    col_w = [next(it) for _ in range(n)]
    row_w = [next(it) for _ in range(m)]
    for c in range(n):
        for _ in range(max_cw):
            next(it)
    rows = []
    for r in range(m):
        vals = [next(it) for _ in range(max_rw)]
        rows.append(sorted({v - 1 for v in vals[:row_w[r]] if v > 0}))
    del col_w
    row_ptr = np.zeros(m + 1, dtype=np.int32)
    for r in range(m):
        row_ptr[r + 1] = row_ptr[r] + len(rows[r])
    col_ind = np.asarray([c for row in rows for c in row], dtype=np.int32)
    return n, m, row_ptr, col_ind


def unpack_parity_table(table: np.ndarray, n: int, k: int) -> np.ndarray:
    """Unpack a [k][words] uint64 parity table into a dense [k][n-k] uint8 matrix."""
    words = table.shape[1]
    bits = np.unpackbits(np.ascontiguousarray(table).view(np.uint8).reshape(k, words * 8), axis=1,
                         bitorder="little")
    return bits[:, : n - k].astype(np.uint8)


def gf2_parity_matrix(code: QcCode) -> np.ndarray:
    """Dense P [k][n-k] with codeword = [u | u P mod 2], for H = [A | B], P = (B^-1 A)^T.

    Used by the synthetic transmitter to encode random information bits.
    """
    h = code.dense_h().astype(bool)
    k, m = code.k, code.m
    aug = np.concatenate([h[:, k:], h[:, :k]], axis=1)  # [B | A]
    for col in range(m):
        piv = col + int(np.argmax(aug[col:, col]))
        if not aug[piv, col]:
            raise ValueError("parity part of H is singular")
        if piv != col:
            aug[[col, piv]] = aug[[piv, col]]
        rows = np.nonzero(aug[:, col])[0]
        rows = rows[rows != col]
        aug[rows] ^= aug[col]
    return np.ascontiguousarray(aug[:, m:].T.astype(np.uint8))  # (B^-1 A)^T


def encode(p_matrix: np.ndarray, info: np.ndarray) -> np.ndarray:
    """Systematic-front encode of info [B][k] (uint8) with P [k][n-k]."""
    # float32 products are exact here (sums of at most k <= 2^24 ones) and use BLAS
    parity = (info.astype(np.float32) @ p_matrix.astype(np.float32)).astype(np.int64) & 1
    return np.concatenate([info.astype(np.uint8), parity.astype(np.uint8)], axis=1)
