"""Host wrapper of the continuous-batching decode service (include/sicc_server.h).

The reference's receive loop has no service form: it runs one decode thread
over a bounded frame queue with fixed batching windows
(source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp:9922-10130).  ``Server``
registers codes and OFDM profiles, then accepts requests (codeword LLRs of one
code, or OFDM IQ frames of one profile) from any thread; ``replay`` drives an
offered-load schedule natively and returns per-request latencies.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .codes import QcCode
from .engine import EngineCode
from .ofdm import Tables
from .pipeline import PipeConfig, PipeTables, pipe_structs

BUSY = 3


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_longlong), ("max_batch_codewords", C.c_int),
                ("max_inflight_batches", C.c_int), ("max_pending_requests", C.c_int), ("max_codes", C.c_int),
                ("max_n", C.c_int)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int), ("code_id", C.c_int), ("phy_id", C.c_int), ("count", C.c_int),
                ("protection", C.c_int), ("host_input", C.c_void_p), ("host_info", C.c_void_p),
                ("tag", C.c_ulonglong)]


class Completion(C.Structure):
    _fields_ = [("request_id", C.c_ulonglong), ("tag", C.c_ulonglong), ("status", C.c_int), ("codewords", C.c_int),
                ("failed_codewords", C.c_int), ("osd_codewords", C.c_int), ("latency_us", C.c_double),
                ("queue_us", C.c_double), ("launch_us", C.c_double), ("batch_gpu_us", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_ulonglong), ("completed", C.c_ulonglong), ("batches", C.c_ulonglong),
                ("codewords", C.c_ulonglong), ("busy_rejections", C.c_ulonglong),
                ("arena_bytes_in_use", C.c_longlong), ("arena_bytes_peak", C.c_longlong),
                ("mean_batch_codewords", C.c_double)]


_SIGS = {
    "sicc_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_ulonglong)]),
    "sicc_server_destroy": (C.c_int, [C.c_ulonglong]),
    "sicc_server_add_code": (C.c_int, [C.c_ulonglong, C.POINTER(EngineCode), C.POINTER(C.c_int)]),
    "sicc_server_add_phy": (C.c_int, [C.c_ulonglong, C.POINTER(PipeConfig), C.POINTER(PipeTables), C.c_int, C.c_int,
                                      C.POINTER(C.c_int)]),
    "sicc_server_start": (C.c_int, [C.c_ulonglong]),
    "sicc_server_submit": (C.c_int, [C.c_ulonglong, C.POINTER(Request), C.POINTER(C.c_ulonglong)]),
    "sicc_server_poll": (C.c_int, [C.c_ulonglong, C.c_int, C.POINTER(Completion), C.POINTER(C.c_int), C.c_int]),
    "sicc_server_get_stats": (C.c_int, [C.c_ulonglong, C.POINTER(ServerStats)]),
    "sicc_server_replay": (C.c_int, [C.c_ulonglong, C.POINTER(Request), C.c_void_p, C.c_int, C.POINTER(Completion),
                                     C.POINTER(C.c_double)]),
}


def _fn(name):
    res, args = _SIGS[name]
    return _lib.bind(name, res, args)


@dataclass
class Done:
    request_id: int
    tag: int
    status: int
    codewords: int
    failed_codewords: int
    osd_codewords: int
    latency_us: float
    queue_us: float
    launch_us: float
    batch_gpu_us: float


def _done(c: Completion) -> Done:
    return Done(c.request_id, c.tag, c.status, c.codewords, c.failed_codewords, c.osd_codewords, c.latency_us,
                c.queue_us, c.launch_us, c.batch_gpu_us)


class Server:
    def __init__(self, hbm_budget_bytes: int, max_batch_codewords: int = 65536, max_inflight_batches: int = 2,
                 max_pending_requests: int = 4096, max_codes: int = 64, max_n: int = 2048):
        cfg = ServerConfig(hbm_budget_bytes=hbm_budget_bytes, max_batch_codewords=max_batch_codewords,
                           max_inflight_batches=max_inflight_batches, max_pending_requests=max_pending_requests,
                           max_codes=max_codes, max_n=max_n)
        h = C.c_ulonglong(0)
        _lib.check(_fn("sicc_server_create")(C.byref(cfg), C.byref(h)), "sicc_server_create")
        self.handle = h.value
        self.codes: list[QcCode] = []
        self.phys: list[dict] = []
        self._inflight: dict[int, tuple] = {}  # request id -> (input, output) kept alive until polled

    def close(self):
        if getattr(self, "handle", 0):
            _lib.check(_fn("sicc_server_destroy")(self.handle), "sicc_server_destroy")
            self.handle = 0
            self._inflight.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_code(self, code: QcCode, max_iter: int, alpha: float = 0.75, osd_order: int = -1,
                 osd_max_flip: int = 64, osd_max_tests: int = 4096) -> int:
        rp = np.ascontiguousarray(code.row_ptr, np.int32)
        ci = np.ascontiguousarray(code.col_ind, np.int32)
        spec = EngineCode(n=code.n, m=code.m, row_ptr=rp.ctypes.data, col_ind=ci.ctypes.data, max_iterations=max_iter,
                          normalization=alpha, offset=0.0, osd_order=osd_order, osd_max_flip_positions=osd_max_flip,
                          osd_max_tests=osd_max_tests)
        cid = C.c_int(-1)
        _lib.check(_fn("sicc_server_add_code")(self.handle, C.byref(spec), C.byref(cid)), "sicc_server_add_code")
        self.codes.append(code)
        return cid.value

    def add_phy(self, tables: Tables, code_id: int, blocks_per_frame: int, noise_var: float, frame_stride: int,
                sync_radius: int = 0) -> int:
        code = self.codes[code_id]
        c, t, keep = pipe_structs(tables, code.n, code.k, blocks_per_frame, noise_var, sync_radius=sync_radius)
        pid = C.c_int(-1)
        _lib.check(_fn("sicc_server_add_phy")(self.handle, C.byref(c), C.byref(t), frame_stride, code_id,
                                              C.byref(pid)), "sicc_server_add_phy")
        self.phys.append(dict(code_id=code_id, blocks=blocks_per_frame, stride=frame_stride))
        return pid.value

    def start(self):
        _lib.check(_fn("sicc_server_start")(self.handle), "sicc_server_start")

    def request(self, kind: int, ident: int, data: np.ndarray, protection: int = 1, tag: int = 0, out=None):
        """(Request, input array, output array) for LLRs [count][n] (kind 0) or IQ [count][stride] (kind 1).

        ``out`` (uint8, C-contiguous, codewords x k) receives the information bits; allocated when None.
        """
        if kind == 0:
            x = np.ascontiguousarray(data, np.float32)
            code = self.codes[ident]
            count = x.shape[0]
            out = np.zeros((count, code.k), np.uint8) if out is None else out
            if out.size != count * code.k or not out.flags.c_contiguous or out.dtype != np.uint8:
                raise ValueError("out must be contiguous uint8 with codewords x k elements")
            req = Request(kind=0, code_id=ident, phy_id=-1, count=count, protection=protection,
                          host_input=x.ctypes.data, host_info=out.ctypes.data, tag=tag)
        else:
            x = np.ascontiguousarray(data, np.complex64)
            p = self.phys[ident]
            code = self.codes[p["code_id"]]
            count = x.shape[0]
            out = np.zeros((count * p["blocks"], code.k), np.uint8) if out is None else out
            if out.size != count * p["blocks"] * code.k or not out.flags.c_contiguous or out.dtype != np.uint8:
                raise ValueError("out must be contiguous uint8 with codewords x k elements")
            req = Request(kind=1, code_id=-1, phy_id=ident, count=count, protection=protection,
                          host_input=x.ctypes.data, host_info=out.ctypes.data, tag=tag)
        return req, x, out

    def submit(self, kind: int, ident: int, data: np.ndarray, protection: int = 1, tag: int = 0):
        """Returns (request id, output array) or (None, None) when the pending queue is full."""
        req, x, out = self.request(kind, ident, data, protection, tag)
        rid = self.submit_request(req, keep=(x, out))
        return (None, None) if rid is None else (rid, out)

    def submit_request(self, req: Request, keep=None):
        """Submits a prepared request; None when the pending queue is full.  ``keep`` is held until polled."""
        rid = C.c_ulonglong(0)
        st = _fn("sicc_server_submit")(self.handle, C.byref(req), C.byref(rid))
        if st == BUSY:
            return None
        _lib.check(st, "sicc_server_submit")
        self._inflight[rid.value] = keep
        return rid.value

    def poll(self, max_count: int = 256, wait_us: int = 1000) -> list[Done]:
        buf = (Completion * max_count)()
        got = C.c_int(0)
        _lib.check(_fn("sicc_server_poll")(self.handle, max_count, buf, C.byref(got), wait_us), "sicc_server_poll")
        res = [_done(buf[i]) for i in range(got.value)]
        for d in res:
            self._inflight.pop(d.request_id, None)
        return res

    def stats(self) -> ServerStats:
        s = ServerStats()
        _lib.check(_fn("sicc_server_get_stats")(self.handle, C.byref(s)), "sicc_server_get_stats")
        return s

    def replay(self, requests: list, arrival_us: np.ndarray):
        """Submit requests[i] (from ``request``) at arrival_us[i]; returns (completions in order, wall us)."""
        n = len(requests)
        arr = (Request * n)(*[r[0] for r in requests])
        t = np.ascontiguousarray(arrival_us, np.float64)
        out = (Completion * n)()
        wall = C.c_double(0.0)
        _lib.check(_fn("sicc_server_replay")(self.handle, arr, t.ctypes.data, n, out, C.byref(wall)),
                   "sicc_server_replay")
        return [_done(out[i]) for i in range(n)], wall.value
