"""ctypes front end for the oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg, always as the checker or the timed CPU
baseline, never as a path of the product.

* ``Oracle``    — oracle/liboracle.so, the C restatement (sicc_oracle.c).
* ``Reference`` — oracle/_ref/libref.so, the reference's own CPU receive path
  compiled from its sources (present only where the reference tree was).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")


def ref_root() -> str:
    """Root of the reference tree as the oracle recipe resolves it (REF_ROOT, else its default)."""
    out = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref-root"], check=True,
                         capture_output=True, text=True)
    return out.stdout.strip()


def build_oracle(ref: bool = False) -> None:
    """Compile liboracle.so (and, when asked and the reference exists, _ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _c32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class OraclePhy(C.Structure):
    _fields_ = [
        ("nfft", C.c_int), ("cp", C.c_int), ("num_symbols", C.c_int), ("active_sc", C.c_int),
        ("pre_half_len", C.c_int), ("bits_per_symbol", C.c_int), ("num_pilots", C.c_int),
        ("num_data", C.c_int), ("rate", C.c_double), ("sync_threshold", C.c_double),
        ("used_indices", C.c_void_p), ("pilot_symbols", C.c_void_p), ("data_symbols", C.c_void_p),
        ("preamble", C.c_void_p), ("pilot_grid", C.c_void_p), ("constellation", C.c_void_p),
    ]


class Oracle:
    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        L = C.CDLL(path)
        self.L = L
        L.or_code_create.restype = C.c_void_p
        L.or_code_create.argtypes = [C.c_int, C.c_int, _i32p, _i32p, C.c_int]
        L.or_code_destroy.argtypes = [C.c_void_p]
        for f in ("or_code_n", "or_code_m", "or_code_k", "or_code_is_accumulator"):
            getattr(L, f).argtypes = [C.c_void_p]
            getattr(L, f).restype = C.c_int
        L.or_code_info_cols.argtypes = [C.c_void_p, _i32p, _i32p]
        L.or_encode.argtypes = [C.c_void_p, _u8p, _u8p]
        L.or_syndrome_weight.argtypes = [C.c_void_p, _u8p]
        L.or_syndrome_weight.restype = C.c_int
        L.or_systematic_parity.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
        L.or_systematic_parity.restype = C.c_int
        L.or_greedy_color_order.argtypes = [C.c_void_p, _i32p, _i32p]
        L.or_greedy_color_order.restype = C.c_int
        L.or_nms_flooding_ref.argtypes = [C.c_void_p, _f32p, C.c_int, C.c_double, _u8p, _f32p,
                                          C.POINTER(C.c_int)]
        L.or_nms_flooding_ref.restype = C.c_int
        L.or_nms_flooding_f32.argtypes = [C.c_void_p, _f32p, C.c_int, C.c_float, C.c_float, C.c_float,
                                          _u8p, _f32p, _f32p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.or_nms_flooding_f32.restype = C.c_int
        L.or_nms_layered_f32.argtypes = [C.c_void_p, C.c_void_p, _f32p, C.c_int, C.c_float, C.c_float,
                                         _u8p, _f32p, _f32p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.or_nms_layered_f32.restype = C.c_int
        L.or_nms_layered_f64.argtypes = [C.c_void_p, C.c_void_p, _f32p, C.c_int, C.c_double, C.c_double,
                                         _u8p, _f64p, C.POINTER(C.c_int)]
        L.or_nms_layered_f64.restype = C.c_int
        L.or_osd.argtypes = [C.c_int, C.c_int, _u64p, C.c_int, _f32p, C.c_int, C.c_int, C.c_int, _u8p,
                             C.POINTER(C.c_float), C.POINTER(C.c_int)]
        L.or_osd.restype = C.c_int
        L.or_bp_osd_batch.argtypes = [C.c_void_p, _u64p, C.c_int, _f32p, C.c_int, C.c_int, C.c_int, C.c_float,
                                      C.c_int, C.c_int, C.c_int, _u8p, _u8p]
        L.or_bp_osd_batch.restype = C.c_int
        L.or_fft_shifted.argtypes = [_f32p, C.c_int, _f32p]
        L.or_sync_earliest.argtypes = [C.POINTER(OraclePhy), _f32p, C.c_longlong, C.c_longlong,
                                       C.POINTER(C.c_longlong), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.or_sync_earliest.restype = C.c_int
        L.or_demod_frame.argtypes = [C.POINTER(OraclePhy), _f32p, C.c_double, C.c_double, _f32p]
        L.or_llr_maxlog.argtypes = [C.POINTER(OraclePhy), _f32p, C.c_int, _f64p, _f32p]

    # ---- codes ----
    def code(self, n, m, row_ptr, col_ind, systematic_front=True):
        return OracleCode(self, n, m, row_ptr, col_ind, systematic_front)

    # ---- OSD ----
    def osd(self, parity_table, n, k, llr, order=2, max_flip=64, max_tests=4096):
        table = np.ascontiguousarray(parity_table, dtype=np.uint64)
        out = np.zeros(n, dtype=np.uint8)
        metric = C.c_float()
        best = C.c_int()
        tests = self.L.or_osd(n, k, table, table.shape[1], np.ascontiguousarray(llr, dtype=np.float32),
                              order, max_flip, max_tests, out, C.byref(metric), C.byref(best))
        if tests < 0:
            raise RuntimeError("OSD: rank-deficient generator")
        return out, float(metric.value), int(best.value), int(tests)

    # ---- OFDM ----
    def fft_shifted(self, time_iq: np.ndarray) -> np.ndarray:
        t = np.ascontiguousarray(time_iq, dtype=np.complex64)
        out = np.zeros_like(t)
        self.L.or_fft_shifted(t.view(np.float32), t.shape[0], out.view(np.float32))
        return out

    def phy(self, tables) -> "OraclePhyHandle":
        return OraclePhyHandle(tables)

    def sync_earliest(self, ph, buf: np.ndarray, max_search: int = 0):
        b = np.ascontiguousarray(buf, dtype=np.complex64)
        s, co, fi, cfo = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        r = self.L.or_sync_earliest(C.byref(ph.s), b.view(np.float32), b.shape[0], max_search,
                                    C.byref(s), C.byref(co), C.byref(fi), C.byref(cfo))
        return r, int(s.value), co.value, fi.value, cfo.value

    def demod_frame(self, ph, frame: np.ndarray, cfo_hz: float, noise_var: float) -> np.ndarray:
        f = np.ascontiguousarray(frame, dtype=np.complex64)
        out = np.zeros(ph.coded_bits, dtype=np.float32)
        self.L.or_demod_frame(C.byref(ph.s), f.view(np.float32), cfo_hz, noise_var, out)
        return out

    def llr_maxlog(self, ph, x: np.ndarray, sigma2: np.ndarray) -> np.ndarray:
        xx = np.ascontiguousarray(x, dtype=np.complex64)
        out = np.zeros(xx.shape[0] * ph.s.bits_per_symbol, dtype=np.float32)
        self.L.or_llr_maxlog(C.byref(ph.s), xx.view(np.float32), xx.shape[0],
                             np.ascontiguousarray(sigma2, dtype=np.float64), out)
        return out


class OraclePhyHandle:
    """Keeps the numpy tables alive behind an or_phy struct."""

    def __init__(self, t):
        self.keep = dict(
            used=_c32(t.used_indices), pilots=_c32(t.pilot_symbols), data=_c32(t.data_symbols),
            pre=np.ascontiguousarray(t.preamble, dtype=np.complex64),
            grid=np.ascontiguousarray(t.pilot_grid, dtype=np.complex64),
            const=np.ascontiguousarray(t.constellation, dtype=np.complex64))
        k = self.keep
        self.s = OraclePhy(
            nfft=t.nfft, cp=t.cp, num_symbols=t.num_symbols, active_sc=t.active_sc,
            pre_half_len=t.pre_half_len, bits_per_symbol=t.bits_per_symbol,
            num_pilots=len(k["pilots"]), num_data=len(k["data"]), rate=t.sample_rate,
            sync_threshold=t.sync_threshold,
            used_indices=k["used"].ctypes.data, pilot_symbols=k["pilots"].ctypes.data,
            data_symbols=k["data"].ctypes.data, preamble=k["pre"].ctypes.data,
            pilot_grid=k["grid"].ctypes.data, constellation=k["const"].ctypes.data)
        self.coded_bits = t.active_sc * len(k["data"]) * t.bits_per_symbol


class OracleCode:
    def __init__(self, o: Oracle, n, m, row_ptr, col_ind, systematic_front=True):
        self.o = o
        self.row_ptr = _c32(row_ptr)
        self.col_ind = _c32(col_ind)
        self.h = o.L.or_code_create(n, m, self.row_ptr, self.col_ind, 1 if systematic_front else 0)
        if not self.h:
            raise ValueError("oracle: code construction failed (rank deficient or bad shape)")
        self.n, self.m = n, m
        self.k = o.L.or_code_k(self.h)

    def __del__(self):
        try:
            self.o.L.or_code_destroy(self.h)
        except Exception:
            pass

    def info_cols(self):
        info = np.zeros(self.k, np.int32)
        piv = np.zeros(self.m, np.int32)
        self.o.L.or_code_info_cols(self.h, info, piv)
        return info, piv

    def encode(self, info):
        out = np.zeros(self.n, np.uint8)
        self.o.L.or_encode(self.h, np.ascontiguousarray(info, dtype=np.uint8), out)
        return out

    def syndrome_weight(self, bits):
        return self.o.L.or_syndrome_weight(self.h, np.ascontiguousarray(bits, dtype=np.uint8))

    def systematic_parity(self):
        words = C.c_int()
        if self.o.L.or_systematic_parity(self.h, None, C.byref(words)) != 0:
            raise ValueError("code is not systematic-front")
        t = np.zeros((self.k, words.value), np.uint64)
        self.o.L.or_systematic_parity(self.h, t.ctypes.data, C.byref(words))
        return t

    def color_order(self):
        order = np.zeros(self.m, np.int32)
        color = np.zeros(self.m, np.int32)
        nc = self.o.L.or_greedy_color_order(self.h, order, color)
        return order, color, nc

    def bp_osd_batch(self, llrs, schedule=0, max_iter=20, alpha=0.75, osd_order=2, osd_max_flip=64,
                     osd_max_tests=4096, table=None):
        llrs = np.ascontiguousarray(llrs, np.float32).reshape(-1, self.n)
        table = self.systematic_parity() if table is None else np.ascontiguousarray(table, np.uint64)
        info = np.zeros((llrs.shape[0], self.k), np.uint8)
        used = np.zeros(llrs.shape[0], np.uint8)
        self.o.L.or_bp_osd_batch(self.h, table, table.shape[1], llrs, llrs.shape[0], schedule, max_iter, alpha,
                                 osd_order, osd_max_flip, osd_max_tests, info, used)
        return info, used

    def flooding_ref(self, llr, max_iter, normalization):
        bits = np.zeros(self.n, np.uint8)
        app = np.zeros(self.n, np.float32)
        it = C.c_int()
        ok = self.o.L.or_nms_flooding_ref(self.h, np.ascontiguousarray(llr, np.float32), max_iter,
                                          normalization, bits, app, C.byref(it))
        return bool(ok), bits, app, it.value

    def flooding(self, llr, max_iter, alpha, beta=0.0, damping=0.0):
        bits = np.zeros(self.n, np.uint8)
        app = np.zeros(self.n, np.float32)
        best = np.zeros(self.n, np.float32)
        it, bw = C.c_int(), C.c_int()
        ok = self.o.L.or_nms_flooding_f32(self.h, np.ascontiguousarray(llr, np.float32), max_iter, alpha,
                                          beta, damping, bits, app, best, C.byref(it), C.byref(bw))
        return bool(ok), bits, app, best, it.value, bw.value

    def layered(self, llr, max_iter, alpha, beta=0.0, row_order=None):
        bits = np.zeros(self.n, np.uint8)
        app = np.zeros(self.n, np.float32)
        best = np.zeros(self.n, np.float32)
        it, bw = C.c_int(), C.c_int()
        ro = None if row_order is None else _c32(row_order)
        ok = self.o.L.or_nms_layered_f32(self.h, None if ro is None else ro.ctypes.data,
                                         np.ascontiguousarray(llr, np.float32), max_iter, alpha, beta,
                                         bits, app, best, C.byref(it), C.byref(bw))
        return bool(ok), bits, app, best, it.value, bw.value

    def layered_f64(self, llr, max_iter, alpha, beta=0.0, row_order=None):
        bits = np.zeros(self.n, np.uint8)
        app = np.zeros(self.n, np.float64)
        it = C.c_int()
        ro = None if row_order is None else _c32(row_order)
        ok = self.o.L.or_nms_layered_f64(self.h, None if ro is None else ro.ctypes.data,
                                         np.ascontiguousarray(llr, np.float32), max_iter, alpha, beta,
                                         bits, app, C.byref(it))
        return bool(ok), bits, app, it.value


class Reference:
    """The reference's own CPU receive path (oracle/_ref/libref.so)."""

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_SO)

    def __init__(self, path: str = REF_SO):
        L = C.CDLL(path)
        self.L = L
        L.ref_last_error.restype = C.c_char_p
        L.ref_code_create.restype = C.c_void_p
        L.ref_code_create.argtypes = [C.c_int, C.c_int, _i32p, _i32p, C.c_int]
        L.ref_code_destroy.argtypes = [C.c_void_p]
        L.ref_code_k.argtypes = [C.c_void_p]
        L.ref_code_is_accumulator.argtypes = [C.c_void_p]
        L.ref_code_info_cols.argtypes = [C.c_void_p, _i32p, _i32p]
        L.ref_encode.argtypes = [C.c_void_p, _u8p, _u8p]
        L.ref_check_syndrome.argtypes = [C.c_void_p, _u8p]
        L.ref_systematic_parity.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
        L.ref_decode_min_sum.argtypes = [C.c_void_p, _f32p, C.c_int, C.c_int, C.c_double, _u8p, _u8p, _i32p]
        L.ref_fft_shifted.argtypes = [_f32p, C.c_int, _f32p]
        L.ref_phy_create.restype = C.c_void_p
        L.ref_phy_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_int,
                                     C.c_double, C.c_double, C.c_void_p, C.c_void_p]
        L.ref_phy_destroy.argtypes = [C.c_void_p]
        for f in ("ref_phy_frame_len", "ref_phy_coded_bits", "ref_phy_num_pilots"):
            getattr(L, f).argtypes = [C.c_void_p]
        L.ref_phy_tables.argtypes = [C.c_void_p, _i32p, _i32p, _i32p, _f32p]
        L.ref_llr_maxlog.argtypes = [C.c_void_p, _f32p, C.c_int, _f64p, _f32p]
        L.ref_find_frame_earliest.argtypes = [C.c_void_p, _f32p, C.c_int, C.c_int,
                                              C.POINTER(C.c_longlong), C.POINTER(C.c_double),
                                              C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ref_find_frame_max.argtypes = [C.c_void_p, _f32p, C.c_int, C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ref_decode_frame.argtypes = [C.c_void_p, C.c_void_p, _f32p, C.c_double, C.c_int, C.c_double,
                                       C.c_double, _u8p, C.POINTER(C.c_int)]
        L.ref_build_tx_frame.argtypes = [C.c_void_p, C.c_void_p, _u8p, C.c_int, _f32p]

    def code(self, n, m, row_ptr, col_ind, systematic_front=True):
        rp, ci = _c32(row_ptr), _c32(col_ind)
        h = self.L.ref_code_create(n, m, rp, ci, 1 if systematic_front else 0)
        if not h:
            raise ValueError(self.L.ref_last_error().decode())
        return RefCode(self, h, n, m, (rp, ci))

    def fft_shifted(self, time_iq):
        t = np.ascontiguousarray(time_iq, dtype=np.complex64)
        out = np.zeros_like(t)
        self.L.ref_fft_shifted(t.view(np.float32), t.shape[0], out.view(np.float32))
        return out

    def phy(self, t):
        pre = np.ascontiguousarray(t.preamble, dtype=np.complex64)
        grid = np.ascontiguousarray(t.pilot_grid, dtype=np.complex64)
        h = self.L.ref_phy_create(t.nfft, t.cp, t.num_symbols, t.active_sc, t.pre_half_len,
                                  t.modulation.encode(), t.pilot_period, t.sample_rate, t.sync_threshold,
                                  pre.ctypes.data, grid.ctypes.data)
        if not h:
            raise ValueError(self.L.ref_last_error().decode())
        return RefPhy(self, h, (pre, grid))


class RefCode:
    def __init__(self, r, h, n, m, keep):
        self.r, self.h, self.n, self.m, self.keep = r, h, n, m, keep
        self.k = r.L.ref_code_k(h)

    def __del__(self):
        try:
            self.r.L.ref_code_destroy(self.h)
        except Exception:
            pass

    def info_cols(self):
        info = np.zeros(self.k, np.int32)
        piv = np.zeros(self.m, np.int32)
        self.r.L.ref_code_info_cols(self.h, info, piv)
        return info, piv

    def encode(self, info):
        out = np.zeros(self.n, np.uint8)
        self.r.L.ref_encode(self.h, np.ascontiguousarray(info, np.uint8), out)
        return out

    def syndrome_ok(self, bits):
        return bool(self.r.L.ref_check_syndrome(self.h, np.ascontiguousarray(bits, np.uint8)))

    def systematic_parity(self):
        words = C.c_int()
        if self.r.L.ref_systematic_parity(self.h, None, C.byref(words)) != 0:
            raise ValueError(self.r.L.ref_last_error().decode())
        t = np.zeros((self.k, words.value), np.uint64)
        self.r.L.ref_systematic_parity(self.h, t.ctypes.data, C.byref(words))
        return t

    def decode_min_sum(self, llr, max_iter, normalization):
        llr = np.ascontiguousarray(llr, np.float32).reshape(-1, self.n)
        b = llr.shape[0]
        bits = np.zeros((b, self.n), np.uint8)
        ok = np.zeros(b, np.uint8)
        it = np.zeros(b, np.int32)
        self.r.L.ref_decode_min_sum(self.h, llr, b, max_iter, normalization, bits, ok, it)
        return ok.astype(bool), bits, it


class RefPhy:
    def __init__(self, r, h, keep):
        self.r, self.h, self.keep = r, h, keep
        self.frame_len = r.L.ref_phy_frame_len(h)
        self.coded_bits = r.L.ref_phy_coded_bits(h)

    def __del__(self):
        try:
            self.r.L.ref_phy_destroy(self.h)
        except Exception:
            pass

    def llr_maxlog(self, x, sigma2, bps):
        xx = np.ascontiguousarray(x, np.complex64)
        out = np.zeros(xx.shape[0] * bps, np.float32)
        self.r.L.ref_llr_maxlog(self.h, xx.view(np.float32), xx.shape[0],
                                np.ascontiguousarray(sigma2, np.float64), out)
        return out

    def find_frame_earliest(self, buf, max_search=0):
        b = np.ascontiguousarray(buf, np.complex64)
        s, co, fi, cfo = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        r = self.r.L.ref_find_frame_earliest(self.h, b.view(np.float32), b.shape[0], max_search,
                                             C.byref(s), C.byref(co), C.byref(fi), C.byref(cfo))
        return r, int(s.value), co.value, fi.value, cfo.value

    def decode_frame(self, code: RefCode, frame, cfo_hz, max_iter, normalization, noise_var):
        f = np.ascontiguousarray(frame, np.complex64)
        info = np.zeros(self.coded_bits, np.uint8)
        ok = C.c_int()
        n = self.r.L.ref_decode_frame(self.h, code.h, f.view(np.float32), cfo_hz, max_iter,
                                      normalization, noise_var, info, C.byref(ok))
        if n < 0:
            raise RuntimeError(self.r.L.ref_last_error().decode())
        return info[:n], bool(ok.value)

    def build_tx_frame(self, code: RefCode, info):
        i = np.ascontiguousarray(info, np.uint8)
        out = np.zeros(self.frame_len, np.complex64)
        n = self.r.L.ref_build_tx_frame(self.h, code.h, i, i.shape[0], out.view(np.float32))
        if n < 0:
            raise RuntimeError(self.r.L.ref_last_error().decode())
        return out


# ---- batch decoding on a process pool (the CPU reference run on every host core) ----
def _bp_osd_chunk(args):
    """One worker's share of a batch: BP (+ OSD) through the oracle, with its wall time."""
    import time
    n, m, row_ptr, col_ind, table, llr, kw = args
    oc = Oracle().code(n, m, row_ptr, col_ind)
    t0 = time.perf_counter()
    info, used = oc.bp_osd_batch(llr, table=table, **kw)
    return time.perf_counter() - t0, info, used


def bp_osd_parallel(pool, code, llrs, chunks: int | None = None, **kw):
    """Decodes `llrs` [F][n] with ``OracleCode.bp_osd_batch(**kw)`` split over a process pool.

    `code` needs n, m, row_ptr and col_ind.  The pool must come from a ``spawn``
    context (a forked child of a process that has touched CUDA can hang).
    Returns (wall seconds, info [F][k], used_osd [F]).
    """
    import time
    workers = getattr(pool, "_processes", None) or os.cpu_count() or 1
    parts = np.array_split(np.ascontiguousarray(llrs, np.float32), chunks or 4 * workers)
    table = kw.pop("table", None)
    if table is None:
        table = Oracle().code(code.n, code.m, code.row_ptr, code.col_ind).systematic_parity()
    t0 = time.perf_counter()
    res = pool.map(_bp_osd_chunk, [(code.n, code.m, np.asarray(code.row_ptr), np.asarray(code.col_ind), table, p, kw)
                                   for p in parts if len(p)])
    wall = time.perf_counter() - t0
    return wall, np.concatenate([r[1] for r in res]), np.concatenate([r[2] for r in res])


def _ofdm_chain_chunk(args):
    """The restated CPU receiver on a few frames: earliest-crossing sync, demod with the
    known noise variance, then layered BP of every codeword of the frame."""
    cfg, n, m, row_ptr, col_ind, iq, noise_var, max_iter, alpha = args
    from sicc_gb300 import ofdm  # the package is on the parent's sys.path, passed to spawned workers
    o = Oracle()
    t = ofdm.reference_tables(cfg)
    ph = o.phy(t)
    oc = o.code(n, m, row_ptr, col_ind)
    k = oc.k
    blocks = t.coded_bits // n
    found = np.zeros(len(iq), np.int32)
    start = np.full(len(iq), -1, np.int64)
    cfo = np.zeros(len(iq), np.float64)
    info = np.zeros((len(iq), blocks * k), np.uint8)
    for f, x in enumerate(iq):
        r = o.sync_earliest(ph, x)
        found[f] = r[0]
        if r[0] != 1:
            continue
        start[f], cfo[f] = r[1], r[4]
        llr = o.demod_frame(ph, x[r[1]: r[1] + t.frame_len], r[4], noise_var)
        dec, _ = oc.bp_osd_batch(llr[: blocks * n], schedule=3, max_iter=max_iter, alpha=alpha, osd_order=-1)
        info[f] = dec.reshape(-1)
    return found, start, cfo, info


def ofdm_chain_parallel(pool, cfg, code, iq, noise_var, max_iter, alpha, chunks: int | None = None):
    """Runs ``_ofdm_chain_chunk`` over frames `iq` [F][samples] on a spawn-context pool.

    Returns (found [F], start [F], cfo_hz [F], info [F][blocks*k]).
    """
    workers = getattr(pool, "_processes", None) or os.cpu_count() or 1
    idx = [p for p in np.array_split(np.arange(len(iq)), chunks or 2 * workers) if len(p)]
    res = pool.map(_ofdm_chain_chunk, [(cfg, code.n, code.m, np.asarray(code.row_ptr), np.asarray(code.col_ind),
                                        iq[p], noise_var, max_iter, alpha) for p in idx])
    return tuple(np.concatenate([r[i] for r in res]) for i in range(4))
