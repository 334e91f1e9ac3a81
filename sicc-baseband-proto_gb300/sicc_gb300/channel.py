"""Seeded synthetic channel inputs for the decoder workloads.

BPSK over AWGN exactly as the reference's decoder benchmark forms its LLRs
(source/cpp_cuda/uhd_cpp/tests/gpu_bp_osd_awgn_bench.cpp:159-172): bit 0 maps
to +1, sigma^2 = 1 / (2 R Eb/N0), y = x + sigma * n, LLR = 2 y / sigma^2
computed in double and stored as float32 (positive LLR favours bit 0).  The
noise comes from a NumPy PCG64 generator so every batch is reproducible from
its seed; information bits are uniform.
"""
from __future__ import annotations

import numpy as np

from .codes import QcCode, encode, gf2_parity_matrix

_P_CACHE: dict[tuple, np.ndarray] = {}


def parity_matrix(code: QcCode) -> np.ndarray:
    key = (code.n, code.k, code.z, code.seed)
    if key not in _P_CACHE:
        _P_CACHE[key] = gf2_parity_matrix(code)
    return _P_CACHE[key]


def sigma2_for(rate: float, ebn0_db: float) -> float:
    return 1.0 / (2.0 * rate * 10.0 ** (ebn0_db / 10.0))


def awgn_llrs(code: QcCode, frames: int, ebn0_db, seed: int, all_zero: bool = False):
    """Return (info uint8 [B,k], codewords uint8 [B,n], llr float32 [B,n]).

    ``ebn0_db`` may be a scalar or a per-frame array.
    """
    rng = np.random.default_rng(seed)
    if all_zero:
        info = np.zeros((frames, code.k), dtype=np.uint8)
    else:
        info = rng.integers(0, 2, size=(frames, code.k), dtype=np.uint8)
    cw = code.encode_bits(info) if hasattr(code, "encode_bits") else encode(parity_matrix(code), info)
    ebn0 = np.broadcast_to(np.asarray(ebn0_db, dtype=np.float64), (frames,))
    sigma2 = 1.0 / (2.0 * code.rate * 10.0 ** (ebn0 / 10.0))
    sigma = np.sqrt(sigma2)[:, None]
    x = 1.0 - 2.0 * cw.astype(np.float64)
    y = x + sigma * rng.standard_normal((frames, code.n))
    llr = ((2.0 / sigma2)[:, None] * y).astype(np.float32)
    return info, cw, llr
