"""Host wrapper of the device-resident request loop (include/sicc_devloop.h).

The loop is one or more lanes, each a CUDA graph repeated on the GPU by a
conditional node, sharing one request ring and one completion ring in pinned
host memory.  Each lane iteration admits requests (within the lane's codeword,
LLR, frame and IQ budgets, while no other lane is admitting), lays them out,
demodulates the OFDM IQ requests, decodes every codeword with the lane's
mixed-code engine (BP, then OSD for failures of requests with protection 1),
copies the information bits back to the requests' pinned host buffers and
publishes completions -- the requests that are final after BP while OSD runs,
the others after it; an iteration that admits nothing skips straight to
publication.  The host only appends requests and drains completions (which
arrive in any order).

Request buffers must be page-locked (e.g. ``torch.empty(..., pin_memory=True)``
viewed as NumPy); ``pinned`` allocates such arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .codes import QcCode
from .engine import EngineCode
from .ofdm import Tables
from .pipeline import PipeConfig, PipeTables, pipe_structs
from .server import BUSY, Completion, Request, _done


class DevLoopConfig(C.Structure):
    _fields_ = [("max_batch_codewords", C.c_int), ("max_batch_llr_floats", C.c_longlong), ("max_codes", C.c_int),
                ("ring_requests", C.c_int), ("idle_timeout_ms", C.c_int), ("max_batch_frames", C.c_int),
                ("max_batch_iq_samples", C.c_longlong), ("lanes", C.c_int)]


class DevLoopStats(C.Structure):
    _fields_ = [("submitted", C.c_ulonglong), ("completed", C.c_ulonglong), ("iterations", C.c_ulonglong),
                ("busy_rejections", C.c_ulonglong), ("launches", C.c_ulonglong), ("codewords", C.c_ulonglong),
                ("running", C.c_int), ("busy_iterations", C.c_ulonglong), ("lanes", C.c_int)]


_SIGS = {
    "sicc_devloop_create": (C.c_int, [C.POINTER(DevLoopConfig), C.POINTER(C.c_ulonglong)]),
    "sicc_devloop_destroy": (C.c_int, [C.c_ulonglong]),
    "sicc_devloop_add_code": (C.c_int, [C.c_ulonglong, C.POINTER(EngineCode), C.POINTER(C.c_int)]),
    "sicc_devloop_add_phy": (C.c_int, [C.c_ulonglong, C.POINTER(PipeConfig), C.POINTER(PipeTables), C.c_int, C.c_int,
                                       C.POINTER(C.c_int)]),
    "sicc_devloop_start": (C.c_int, [C.c_ulonglong]),
    "sicc_devloop_submit": (C.c_int, [C.c_ulonglong, C.POINTER(Request), C.POINTER(C.c_ulonglong)]),
    "sicc_devloop_poll": (C.c_int, [C.c_ulonglong, C.c_int, C.POINTER(Completion), C.POINTER(C.c_int), C.c_int]),
    "sicc_devloop_stop": (C.c_int, [C.c_ulonglong, C.c_int]),
    "sicc_devloop_get_stats": (C.c_int, [C.c_ulonglong, C.POINTER(DevLoopStats)]),
    "sicc_devloop_replay": (C.c_int, [C.c_ulonglong, C.POINTER(Request), C.c_void_p, C.c_int, C.POINTER(Completion),
                                      C.POINTER(C.c_double)]),
}


def _fn(name):
    res, args = _SIGS[name]
    return _lib.bind(name, res, args)


def pinned(shape, dtype) -> np.ndarray:
    """A page-locked NumPy array the GPU can address (through torch's pinned allocator)."""
    import torch
    tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.uint8): torch.uint8,
           np.dtype(np.complex64): torch.complex64}[np.dtype(dtype)]
    return torch.empty(shape, dtype=tdt, pin_memory=True).numpy()


class DevLoop:
    def __init__(self, max_batch_codewords: int, max_batch_llr_floats: int, max_codes: int = 64,
                 ring_requests: int = 4096, idle_timeout_ms: int = 2000, max_batch_frames: int = 0,
                 max_batch_iq_samples: int = 0, lanes: int = 1):
        cfg = DevLoopConfig(max_batch_codewords=max_batch_codewords, max_batch_llr_floats=max_batch_llr_floats,
                            max_codes=max_codes, ring_requests=ring_requests, idle_timeout_ms=idle_timeout_ms,
                            max_batch_frames=max_batch_frames, max_batch_iq_samples=max_batch_iq_samples,
                            lanes=lanes)
        h = C.c_ulonglong(0)
        _lib.check(_fn("sicc_devloop_create")(C.byref(cfg), C.byref(h)), "sicc_devloop_create")
        self.handle = h.value
        self.codes: list[QcCode] = []
        self.phys: list[dict] = []
        self._inflight: dict[int, tuple] = {}

    def close(self):
        if getattr(self, "handle", 0):
            _lib.check(_fn("sicc_devloop_destroy")(self.handle), "sicc_devloop_destroy")
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
        _lib.check(_fn("sicc_devloop_add_code")(self.handle, C.byref(spec), C.byref(cid)), "sicc_devloop_add_code")
        self.codes.append(code)
        return cid.value

    def add_phy(self, tables: Tables, code_id: int, blocks_per_frame: int, noise_var: float, frame_stride: int,
                sync_radius: int = 0) -> int:
        code = self.codes[code_id]
        c, t, keep = pipe_structs(tables, code.n, code.k, blocks_per_frame, noise_var, sync_radius=sync_radius)
        pid = C.c_int(-1)
        _lib.check(_fn("sicc_devloop_add_phy")(self.handle, C.byref(c), C.byref(t), frame_stride, code_id,
                                               C.byref(pid)), "sicc_devloop_add_phy")
        self.phys.append(dict(code_id=code_id, blocks=blocks_per_frame, stride=frame_stride))
        return pid.value

    def start(self):
        _lib.check(_fn("sicc_devloop_start")(self.handle), "sicc_devloop_start")

    def stop(self, wait_ms: int = 10000):
        _lib.check(_fn("sicc_devloop_stop")(self.handle, wait_ms), "sicc_devloop_stop")

    def request(self, code_id: int, llr: np.ndarray, protection: int = 1, tag: int = 0, out=None):
        """(Request, input, output) for pinned LLRs [count][n]; ``out`` pinned uint8 [count][k] (made if None)."""
        code = self.codes[code_id]
        count = llr.shape[0]
        if out is None:
            out = pinned((count, code.k), np.uint8)
        req = Request(kind=0, code_id=code_id, phy_id=-1, count=count, protection=protection,
                      host_input=llr.ctypes.data, host_info=out.ctypes.data, tag=tag)
        return req, llr, out

    def iq_request(self, phy_id: int, iq: np.ndarray, protection: int = 1, tag: int = 0, out=None):
        """(Request, input, output) for pinned IQ frames [count][frame_stride] (complex64); ``out`` pinned uint8
        [count * blocks][k] (made if None)."""
        p = self.phys[phy_id]
        code = self.codes[p["code_id"]]
        count = iq.shape[0]
        if out is None:
            out = pinned((count * p["blocks"], code.k), np.uint8)
        req = Request(kind=1, code_id=-1, phy_id=phy_id, count=count, protection=protection,
                      host_input=iq.ctypes.data, host_info=out.ctypes.data, tag=tag)
        return req, iq, out

    def submit_request(self, req: Request, keep=None):
        """Submits a prepared request; None when the ring is full.  ``keep`` is held until polled."""
        rid = C.c_ulonglong(0)
        st = _fn("sicc_devloop_submit")(self.handle, C.byref(req), C.byref(rid))
        if st == BUSY:
            return None
        _lib.check(st, "sicc_devloop_submit")
        self._inflight[rid.value] = keep
        return rid.value

    def poll(self, max_count: int = 256, wait_us: int = 1000):
        buf = (Completion * max_count)()
        got = C.c_int(0)
        _lib.check(_fn("sicc_devloop_poll")(self.handle, max_count, buf, C.byref(got), wait_us), "sicc_devloop_poll")
        res = [_done(buf[i]) for i in range(got.value)]
        for d in res:
            self._inflight.pop(d.request_id, None)
        return res

    def stats(self) -> DevLoopStats:
        s = DevLoopStats()
        _lib.check(_fn("sicc_devloop_get_stats")(self.handle, C.byref(s)), "sicc_devloop_get_stats")
        return s

    def replay(self, requests: list, arrival_us: np.ndarray):
        """Submit requests[i] (from ``request``) at arrival_us[i]; returns (completions in order, wall us)."""
        n = len(requests)
        arr = (Request * n)(*[r[0] for r in requests])
        t = np.ascontiguousarray(arrival_us, np.float64)
        out = (Completion * n)()
        wall = C.c_double(0.0)
        _lib.check(_fn("sicc_devloop_replay")(self.handle, arr, t.ctypes.data, n, out, C.byref(wall)),
                   "sicc_devloop_replay")
        return [_done(out[i]) for i in range(n)], wall.value
