"""ctypes binding of libsicc_gb300.so (the C ABI declared in include/*.h).

The shared library is the only implementation: when it is missing this module
raises instead of falling back to anything else.  Build it with
``sicc-baseband-proto_gb300/build.py`` (``__graft_entry__.build()`` does).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libsicc_gb300.so")
REPO_ROOT = os.path.dirname(PKG_ROOT)
INCLUDE_DIR = os.path.join(REPO_ROOT, "include")

OK, INVALID_ARGUMENT, INTERNAL_ERROR = 0, 1, 2

u64 = C.c_ulonglong
vp = C.c_void_p


class StreamConfig(C.Structure):
    _fields_ = [("n", C.c_int), ("k", C.c_int), ("m", C.c_int), ("max_batch_size", C.c_int),
                ("min_batch_size", C.c_int), ("max_latency_us", u64), ("arrival_ewma_alpha", C.c_double),
                ("default_interarrival_us", u64), ("bp_max_iterations", C.c_int), ("bp_normalization", C.c_float),
                ("bp_offset", C.c_float), ("bp_damping", C.c_float), ("bp_min_abs_llr_accept", C.c_float),
                ("osd_threads", C.c_int)]


class OsdConfig(C.Structure):
    _fields_ = [("n", C.c_int), ("k", C.c_int), ("max_batch_size", C.c_int), ("osd_threads", C.c_int)]


class BpCsrConfig(C.Structure):
    _fields_ = [("n", C.c_int), ("m", C.c_int), ("max_batch_size", C.c_int), ("max_iterations", C.c_int),
                ("normalization", C.c_float), ("offset", C.c_float), ("damping", C.c_float),
                ("min_abs_llr_accept", C.c_float), ("nnz", C.c_int), ("schedule", C.c_int)]


class StreamStats(C.Structure):
    _fields_ = [("submitted_codewords", u64), ("decoded_codewords", u64), ("bp_success_codewords", u64),
                ("osd_fallback_codewords", u64), ("decoded_batches", u64), ("current_pending_codewords", u64),
                ("max_pending_codewords", u64), ("last_submit_timestamp_us", u64),
                ("ewma_interarrival_us", C.c_double), ("average_batch_size", C.c_double),
                ("total_decode_ms", C.c_double)]


class SiccError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where} failed (status {status}): {message}")
        self.status = status


_SIGS = {
    # name: (restype, argtypes)
    "cuda_osd_get_last_error": (C.c_char_p, []),
    "cuda_osd_create_stream_decoder": (C.c_int, [C.POINTER(StreamConfig), C.POINTER(u64)]),
    "cuda_osd_create_stream_decoder_with_matrices": (C.c_int, [C.POINTER(StreamConfig), vp, vp, C.c_int,
                                                               C.POINTER(u64)]),
    "cuda_osd_destroy_stream_decoder": (C.c_int, [u64]),
    "cuda_osd_create_osd_decoder": (C.c_int, [C.POINTER(OsdConfig), C.POINTER(u64)]),
    "cuda_osd_destroy_osd_decoder": (C.c_int, [u64]),
    "cuda_osd_create_bp_csr_decoder": (C.c_int, [C.POINTER(BpCsrConfig), vp, vp, C.POINTER(u64)]),
    "cuda_osd_destroy_bp_csr_decoder": (C.c_int, [u64]),
    "cuda_osd_decode_bp_csr_batch": (C.c_int, [u64, vp, C.c_int, vp, vp, C.POINTER(C.c_double)]),
    "cuda_osd_decode_bp_csr_device_batch": (C.c_int, [u64, vp, C.c_int, vp, vp, C.POINTER(C.c_double)]),
    "cuda_osd_decode_osd_batch": (C.c_int, [u64, vp, C.c_int, vp, vp, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]),
    "cuda_osd_submit_codewords": (C.c_int, [u64, vp, C.c_int, vp, vp, vp]),
    "cuda_osd_submit_device_codewords": (C.c_int, [u64, vp, C.c_int, vp, vp, vp]),
    "cuda_osd_poll_ready": (C.c_int, [u64, C.c_int, vp, vp, vp, vp, vp, C.POINTER(C.c_int)]),
    "cuda_osd_flush": (C.c_int, [u64]),
    "cuda_osd_get_stats": (C.c_int, [u64, C.POINTER(StreamStats)]),
    "cuda_osd_get_decoded_codewords": (u64, [u64]),
    "cuda_osd_get_total_decode_ms": (C.c_double, [u64]),
    "cuda_osd_find_frame": (C.c_int, [vp, vp, C.c_int, vp, vp, C.c_int, C.c_int, C.c_double, C.c_double,
                                      C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "sicc_fec_set_schedule": (C.c_int, [u64, C.c_int]),
    "sicc_fec_set_osd_params": (C.c_int, [u64, C.c_int, C.c_int, C.c_int]),
    "sicc_fec_set_osd_enabled": (C.c_int, [u64, C.c_int]),
    "sicc_fec_set_launch_shape": (C.c_int, [u64, C.c_int, C.c_int]),
    "sicc_fec_set_timing": (C.c_int, [u64, C.c_int]),
    "sicc_fec_get_kernel_ms": (C.c_int, [u64, C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                         C.POINTER(C.c_longlong)]),
    "sicc_fec_decode_device": (C.c_int, [u64, vp, C.c_int, vp, vp, vp, vp, vp]),
    "sicc_bp_csr_decode_device": (C.c_int, [u64, vp, C.c_int, vp, vp, vp, vp, vp]),
    "sicc_osd_decode_device": (C.c_int, [u64, vp, C.c_int, vp, vp, vp, vp]),
}

_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return LIB_PATH


def load() -> C.CDLL:
    """Load libsicc_gb300.so; raises when it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: the CUDA library must be built "
                               "(python sicc-baseband-proto_gb300/build.py); there is no fallback path")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue  # optional symbols are resolved on use
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def bind(name: str, restype, argtypes):
    """Declare the signature of an additional symbol and return it."""
    L = load()
    fn = getattr(L, name)
    fn.restype = restype
    fn.argtypes = argtypes
    return fn


def last_error() -> str:
    msg = load().cuda_osd_get_last_error()
    return msg.decode() if msg else ""


def check(status: int, where: str) -> None:
    if status != OK:
        raise SiccError(status, where, last_error())


def ptr(x) -> int | None:
    """Address of a numpy array or torch tensor (None and raw addresses pass through)."""
    if x is None or isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data
