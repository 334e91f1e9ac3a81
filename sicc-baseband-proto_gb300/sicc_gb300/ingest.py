"""Host wrapper of the real-time receive ingest (include/sicc_ingest.h).

Stands where the reference's GpuOnlineIqBuffer, DeviceFramePool and
GpuRxSyncExtractor::extract_device are driven by its RX loop
(source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp:5666-5744, 6901-6979,
7565-7847, 8480-8567): push samples as they arrive, step to extract the frames
found, demodulate them from the pool, release their slots.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .pipeline import RxPipeline


class IngestConfig(C.Structure):
    _fields_ = [("ring_samples", C.c_longlong), ("pool_frames", C.c_int), ("max_buffered_frames", C.c_int),
                ("sync_tracking_window", C.c_int), ("sync_late_peak_threshold", C.c_float),
                ("buffered_min", C.c_int), ("buffered_max", C.c_int)]


class IngestFrame(C.Structure):
    _fields_ = [("slot", C.c_int), ("peak", C.c_float), ("cfo_hz", C.c_float), ("pad", C.c_int),
                ("position", C.c_longlong)]


class IngestStats(C.Structure):
    _fields_ = [(name, C.c_ulonglong) for name in ("found", "miss", "tracking_miss", "incomplete", "skipped_samples",
                                                   "max_start", "dropped_samples", "pool_exhausted")] + \
               [("buffered", C.c_longlong), ("tracking", C.c_int), ("free_slots", C.c_int)]


_SIGS = {
    "sicc_ingest_create": (C.c_int, [C.c_ulonglong, C.POINTER(IngestConfig), C.POINTER(C.c_ulonglong)]),
    "sicc_ingest_destroy": (C.c_int, [C.c_ulonglong]),
    "sicc_ingest_push": (C.c_int, [C.c_ulonglong, C.c_void_p, C.c_longlong]),
    "sicc_ingest_step": (C.c_int, [C.c_ulonglong, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_int)]),
    "sicc_ingest_frame_ptr": (C.c_int, [C.c_ulonglong, C.c_int, C.POINTER(C.c_void_p)]),
    "sicc_ingest_pool": (C.c_int, [C.c_ulonglong, C.POINTER(C.c_void_p), C.POINTER(C.c_int)]),
    "sicc_ingest_release": (C.c_int, [C.c_ulonglong, C.c_int]),
    "sicc_ingest_stats": (C.c_int, [C.c_ulonglong, C.POINTER(IngestStats)]),
    "sicc_ingest_close": (C.c_int, [C.c_ulonglong]),
}


def _fn(name):
    res, args = _SIGS[name]
    return _lib.bind(name, res, args)


class Ingest:
    def __init__(self, pipe: RxPipeline, ring_samples: int, pool_frames: int = 16, max_buffered_frames: int = 2,
                 tracking_window: int = 256, late_threshold: float = 0.0, buffered_min: int | None = None,
                 buffered_max: int | None = None):
        fl = pipe.frame_samples
        self.pipe = pipe
        self.cfg = IngestConfig(ring_samples=ring_samples, pool_frames=pool_frames,
                                max_buffered_frames=max_buffered_frames, sync_tracking_window=tracking_window,
                                sync_late_peak_threshold=late_threshold,
                                buffered_min=fl if buffered_min is None else buffered_min,
                                buffered_max=max_buffered_frames * fl if buffered_max is None else buffered_max)
        h = C.c_ulonglong(0)
        _lib.check(_fn("sicc_ingest_create")(pipe.handle, C.byref(self.cfg), C.byref(h)), "sicc_ingest_create")
        self.handle = h.value
        self._frames = (IngestFrame * max(pool_frames, 4))()

    def close(self):
        if getattr(self, "handle", 0):
            _lib.check(_fn("sicc_ingest_destroy")(self.handle), "sicc_ingest_destroy")
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def push(self, iq):
        x = iq if hasattr(iq, "data_ptr") else np.ascontiguousarray(iq, np.complex64)
        n = int(x.shape[0])
        _lib.check(_fn("sicc_ingest_push")(self.handle, _lib.ptr(x), n), "sicc_ingest_push")

    def step(self, max_frames: int | None = None, timeout_ms: int = 0):
        """[(slot, position, peak, cfo_hz)] of the frames extracted by one step."""
        m = len(self._frames) if max_frames is None else max_frames
        cnt = C.c_int(0)
        _lib.check(_fn("sicc_ingest_step")(self.handle, m, timeout_ms, C.cast(self._frames, C.c_void_p),
                                           C.byref(cnt)), "sicc_ingest_step")
        return [(f.slot, f.position, f.peak, f.cfo_hz) for f in self._frames[: cnt.value]]

    def frame_ptr(self, slot: int) -> int:
        d = C.c_void_p()
        _lib.check(_fn("sicc_ingest_frame_ptr")(self.handle, slot, C.byref(d)), "sicc_ingest_frame_ptr")
        return d.value

    def pool(self):
        d, fs = C.c_void_p(), C.c_int()
        _lib.check(_fn("sicc_ingest_pool")(self.handle, C.byref(d), C.byref(fs)), "sicc_ingest_pool")
        return d.value, fs.value

    def release(self, slot: int):
        _lib.check(_fn("sicc_ingest_release")(self.handle, slot), "sicc_ingest_release")

    def stats(self) -> dict:
        s = IngestStats()
        _lib.check(_fn("sicc_ingest_stats")(self.handle, C.byref(s)), "sicc_ingest_stats")
        return {name: getattr(s, name) for name, _ in IngestStats._fields_}

    def close_input(self):
        _lib.check(_fn("sicc_ingest_close")(self.handle), "sicc_ingest_close")
