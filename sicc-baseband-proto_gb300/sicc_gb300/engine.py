"""Mixed-code batched decoding (include/sicc_engine.h) and its workloads.

``Engine`` wraps the C ABI.  ``MixedWorkload`` builds the mixed-length,
mixed-rate workload: requests of 1..512 codewords of one code each, the code
drawn per request from the 15 QC codes of ``codes.mixed_codes()``, Eb/N0
uniform in [1, 5] dB per codeword, BP iteration caps of 20 (n <= 256), 25
(n = 512, 1024) and 30 (n = 2048), and an OSD fallback where the OSD kernel
covers the code.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib, channel, codes
from .codes import QcCode


class EngineConfig(C.Structure):
    _fields_ = [("max_codewords", C.c_int), ("max_llr_floats", C.c_longlong), ("max_codes", C.c_int)]


class EngineCode(C.Structure):
    _fields_ = [("n", C.c_int), ("m", C.c_int), ("row_ptr", C.c_void_p), ("col_ind", C.c_void_p),
                ("max_iterations", C.c_int), ("normalization", C.c_float), ("offset", C.c_float),
                ("osd_order", C.c_int), ("osd_max_flip_positions", C.c_int), ("osd_max_tests", C.c_int)]


_SIGS = {
    "sicc_engine_create": (C.c_int, [C.POINTER(EngineConfig), C.POINTER(C.c_ulonglong)]),
    "sicc_engine_destroy": (C.c_int, [C.c_ulonglong]),
    "sicc_engine_add_code": (C.c_int, [C.c_ulonglong, C.POINTER(EngineCode), C.POINTER(C.c_int)]),
    "sicc_engine_set_launch_shape": (C.c_int, [C.c_ulonglong, C.c_int, C.c_int]),
    "sicc_engine_decode_device": (C.c_int, [C.c_ulonglong, C.c_int] + [C.c_void_p] * 9),
    "sicc_engine_decode_device_protected": (C.c_int, [C.c_ulonglong, C.c_int] + [C.c_void_p] * 10),
    "sicc_engine_osd_device": (C.c_int, [C.c_ulonglong, C.c_int] + [C.c_void_p] * 8),
    "sicc_engine_last_ms": (C.c_int, [C.c_ulonglong] + [C.POINTER(C.c_float)] * 3),
}


def _fn(name):
    res, args = _SIGS[name]
    return _lib.bind(name, res, args)


def osd_supported(code: QcCode) -> bool:
    """Codes the warp OSD kernel covers (n <= 256, k <= 128)."""
    return code.n <= 256 and code.k <= 128


def osd_order_for(code: QcCode) -> int:
    """OSD order of the mixed workload: 2 for n <= 256, 1 for longer codes."""
    return 2 if code.n <= 256 else 1


def iteration_cap(n: int) -> int:
    return 20 if n <= 256 else (25 if n <= 1024 else 30)


class Engine:
    def __init__(self, max_codewords: int, max_llr_floats: int, max_codes: int = 64):
        cfg = EngineConfig(max_codewords=max_codewords, max_llr_floats=max_llr_floats, max_codes=max_codes)
        h = C.c_ulonglong(0)
        _lib.check(_fn("sicc_engine_create")(C.byref(cfg), C.byref(h)), "sicc_engine_create")
        self.handle = h.value
        self._keep = []

    def close(self):
        if getattr(self, "handle", 0):
            _lib.check(_fn("sicc_engine_destroy")(self.handle), "sicc_engine_destroy")
            self.handle = 0

    # -- launch shapes (include/sicc_tune.h) --
    def code_warps(self, code_id: int) -> int:
        from . import tune
        return tune.code_warps(self.handle, code_id)

    def set_code_warps(self, code_id: int, warps: int) -> None:
        from . import tune
        tune.set_code_warps(self.handle, code_id, warps)

    def autotune(self, codewords, d_code, d_llr, d_llr_off, d_info, d_info_off, reps: int = 3):
        """Tunes warps per codeword of each code and warps per CTA on this batch (outputs are
        overwritten); returns (default BP ms, tuned BP ms)."""
        from . import tune
        return tune.engine_autotune(self.handle, codewords, d_code, d_llr, d_llr_off, d_info, d_info_off, reps)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_code(self, code: QcCode, max_iter: int, alpha: float = 0.75, beta: float = 0.0, osd_order: int = -1,
                 osd_max_flip: int = 64, osd_max_tests: int = 4096) -> int:
        rp = np.ascontiguousarray(code.row_ptr, np.int32)
        ci = np.ascontiguousarray(code.col_ind, np.int32)
        self._keep += [rp, ci]
        spec = EngineCode(n=code.n, m=code.m, row_ptr=rp.ctypes.data, col_ind=ci.ctypes.data,
                          max_iterations=max_iter, normalization=alpha, offset=beta, osd_order=osd_order,
                          osd_max_flip_positions=osd_max_flip, osd_max_tests=osd_max_tests)
        cid = C.c_int(-1)
        _lib.check(_fn("sicc_engine_add_code")(self.handle, C.byref(spec), C.byref(cid)), "sicc_engine_add_code")
        return cid.value

    def set_launch_shape(self, warps_per_cta: int, ctas: int):
        _lib.check(_fn("sicc_engine_set_launch_shape")(self.handle, warps_per_cta, ctas), "sicc_engine_set_launch_shape")

    def decode_device(self, count, d_code_ids, d_llr, d_llr_off, d_info, d_info_off, d_success=None, d_used=None,
                      d_iter=None, stream=None, d_protection=None):
        """One batch; with d_protection (uint8 per codeword) only codewords marked 1 may fall back to OSD."""
        st = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        p = _lib.ptr
        if d_protection is None:
            _lib.check(_fn("sicc_engine_decode_device")(self.handle, count, p(d_code_ids), p(d_llr), p(d_llr_off),
                                                        p(d_info), p(d_info_off), p(d_success), p(d_used), p(d_iter),
                                                        st), "sicc_engine_decode_device")
        else:
            _lib.check(_fn("sicc_engine_decode_device_protected")(self.handle, count, p(d_code_ids), p(d_protection),
                                                                  p(d_llr), p(d_llr_off), p(d_info), p(d_info_off),
                                                                  p(d_success), p(d_used), p(d_iter), st),
                       "sicc_engine_decode_device_protected")

    def osd_device(self, count, d_code_ids, d_llr, d_llr_off, d_info, d_info_off, d_used=None, d_metric=None,
                   stream=None):
        """OSD alone on the given soft values (codes registered with an OSD order)."""
        st = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        p = _lib.ptr
        _lib.check(_fn("sicc_engine_osd_device")(self.handle, count, p(d_code_ids), p(d_llr), p(d_llr_off), p(d_info),
                                                 p(d_info_off), p(d_used), p(d_metric), st), "sicc_engine_osd_device")

    def last_ms(self):
        a, b, c = C.c_float(), C.c_float(), C.c_float()
        _lib.check(_fn("sicc_engine_last_ms")(self.handle, C.byref(a), C.byref(b), C.byref(c)), "sicc_engine_last_ms")
        return a.value, b.value, c.value


@dataclass
class MixedWorkload:
    codes: list           # the QcCode set
    req_code: np.ndarray  # [R] code index of each request
    req_start: np.ndarray # [R+1] first codeword of each request
    code_of: np.ndarray   # [N] uint8
    llr: np.ndarray       # float32 packed
    llr_off: np.ndarray   # int64 [N]
    info: list            # per codeword true info bits (packed array + offsets)
    info_true: np.ndarray
    info_off: np.ndarray  # int64 [N]
    ebn0: np.ndarray

    @property
    def count(self) -> int:
        return int(self.code_of.shape[0])

    @property
    def info_bits(self) -> int:
        return int(self.info_true.shape[0])


def mixed_workload(total: int = 100_000, seed: int = 4242, max_burst: int = 512, code_set=None,
                   ebn0_range=(1.0, 5.0)) -> MixedWorkload:
    """Requests of U{1..max_burst} codewords of one code until `total` codewords."""
    cs = code_set if code_set is not None else codes.mixed_codes()
    rng = np.random.default_rng(seed)
    req_code, sizes = [], []
    left = total
    while left > 0:
        b = int(min(rng.integers(1, max_burst + 1), left))
        req_code.append(int(rng.integers(0, len(cs))))
        sizes.append(b)
        left -= b
    req_code = np.array(req_code, np.int32)
    req_start = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    code_of = np.repeat(req_code, sizes).astype(np.uint8)
    ebn0 = rng.uniform(ebn0_range[0], ebn0_range[1], size=total)
    ns = np.array([cs[c].n for c in code_of], np.int64)
    ks = np.array([cs[c].k for c in code_of], np.int64)
    llr_off = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    info_off = np.concatenate([[0], np.cumsum(ks)[:-1]]).astype(np.int64)
    llr = np.empty(int(ns.sum()), np.float32)
    info_true = np.empty(int(ks.sum()), np.uint8)
    for r, c in enumerate(req_code):
        a, b = int(req_start[r]), int(req_start[r + 1])
        inf, _, l = channel.awgn_llrs(cs[c], b - a, ebn0[a:b], seed=seed * 7919 + r)
        llr[llr_off[a]: llr_off[a] + (b - a) * cs[c].n] = l.reshape(-1)
        info_true[info_off[a]: info_off[a] + (b - a) * cs[c].k] = inf.reshape(-1)
    return MixedWorkload(codes=cs, req_code=req_code, req_start=req_start, code_of=code_of, llr=llr, llr_off=llr_off,
                         info=[], info_true=info_true, info_off=info_off, ebn0=ebn0)
