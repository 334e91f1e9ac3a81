"""Host-side decoder wrappers over the C ABI.

These mirror the reference link driver's wrappers around its decoder library
(source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp): ``CudaBpOsdDecoder``
(:3162-3629: stream BP->OSD with submit/flush/poll and the asynchronous
device-frame window) and ``CudaBpDecoder`` (:3631-3786: generic CSR BP), with
the same argument meaning and the same failure behaviour (a non-zero status
raises with the library's last error).  They add device-resident entry points
used by the batched paths.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib
from .codes import QcCode

FLOODING, NODE_PARALLEL, COLORED_LAYERED, FLAT_LAYERED = 0, 1, 2, 3


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


def dense_h(n: int, m: int, row_ptr, col_ind) -> np.ndarray:
    h = np.zeros((m, n), dtype=np.uint8)
    for r in range(m):
        h[r, col_ind[row_ptr[r]:row_ptr[r + 1]]] = 1
    return h


def systematic_parity_table(n: int, k: int, p_matrix: np.ndarray) -> np.ndarray:
    """[k][ceil((n-k)/64)] uint64 table (bit p of row i = parity bit p of encode(e_i))."""
    words = (n - k + 63) // 64
    padded = np.zeros((k, words * 64), dtype=np.uint8)
    padded[:, : n - k] = p_matrix
    return np.packbits(padded, axis=1, bitorder="little").view(np.uint64).reshape(k, words).copy()


class _Shaped:
    """Launch shape and autotuner of a stream or CSR decoder (include/sicc_tune.h)."""

    def shape(self) -> dict:
        from . import tune
        return tune.get_shape(self.handle)

    def set_shape(self, **fields) -> None:
        from . import tune
        tune.set_shape(self.handle, **fields)

    def autotune(self, d_llr, codewords: int | None = None, reps: int = 5):
        """Times candidate shapes on device LLRs, applies the fastest and caches it per code and
        device; returns a tune.TuneResult (the best shape and every trial)."""
        from . import tune
        return tune.autotune(self.handle, d_llr, codewords, reps)


class StreamBpOsdDecoder(_Shaped):
    """Stream BP -> OSD decoder (the reference's CudaBpOsdDecoder)."""

    def __init__(self, code: QcCode | None = None, *, max_batch: int = 4096, min_batch: int = 30,
                 latency_us: int = 2000, max_iter: int = 20, normalization: float = 0.80, offset: float = 0.15,
                 damping: float = 0.15, min_abs_llr_accept: float = 1.5, p_matrix: np.ndarray | None = None,
                 schedule: int | None = None, osd_order: int | None = None, osd_max_flip: int | None = None,
                 osd_max_tests: int | None = None):
        L = _lib.load()
        cfg = _lib.StreamConfig()
        if code is None:
            cfg.n, cfg.k, cfg.m = 128, 64, 64
        else:
            cfg.n, cfg.k, cfg.m = code.n, code.k, code.m
        cfg.max_batch_size = max_batch
        cfg.min_batch_size = min_batch
        cfg.max_latency_us = max(latency_us, 1)
        cfg.arrival_ewma_alpha = 0.15
        cfg.default_interarrival_us = 150
        cfg.bp_max_iterations = max_iter
        cfg.bp_normalization = normalization
        cfg.bp_offset = offset
        cfg.bp_damping = damping
        cfg.bp_min_abs_llr_accept = min_abs_llr_accept
        cfg.osd_threads = 256
        self.n, self.k, self.max_batch = cfg.n, cfg.k, max_batch
        h = _lib.u64(0)
        if code is None:
            _lib.check(L.cuda_osd_create_stream_decoder(C.byref(cfg), C.byref(h)), "cuda_osd_create_stream_decoder")
        else:
            if p_matrix is None:
                from .channel import parity_matrix
                p_matrix = parity_matrix(code)
            self._h_dense = dense_h(code.n, code.m, code.row_ptr, code.col_ind)
            self._parity = systematic_parity_table(code.n, code.k, p_matrix)
            _lib.check(L.cuda_osd_create_stream_decoder_with_matrices(
                C.byref(cfg), self._h_dense.ctypes.data, self._parity.ctypes.data, self._parity.shape[1],
                C.byref(h)), "cuda_osd_create_stream_decoder_with_matrices")
        self.handle = h.value
        self.frame_sequence = 0
        if schedule is not None:
            _lib.check(L.sicc_fec_set_schedule(self.handle, schedule), "sicc_fec_set_schedule")
        if osd_order is not None or osd_max_flip is not None or osd_max_tests is not None:
            self.set_osd_params(2 if osd_order is None else osd_order,
                                min(self.k, 64) if osd_max_flip is None else osd_max_flip,
                                4096 if osd_max_tests is None else osd_max_tests)

    def close(self):
        if getattr(self, "handle", 0):
            _lib.check(_lib.load().cuda_osd_destroy_stream_decoder(self.handle), "cuda_osd_destroy_stream_decoder")
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_osd_params(self, order: int, max_flip: int, max_tests: int):
        _lib.check(_lib.load().sicc_fec_set_osd_params(self.handle, order, max_flip, max_tests),
                   "sicc_fec_set_osd_params")

    def set_osd_enabled(self, enabled: bool):
        _lib.check(_lib.load().sicc_fec_set_osd_enabled(self.handle, 1 if enabled else 0), "sicc_fec_set_osd_enabled")

    def set_launch_shape(self, slots_per_cta: int, ctas: int):
        _lib.check(_lib.load().sicc_fec_set_launch_shape(self.handle, slots_per_cta, ctas), "sicc_fec_set_launch_shape")

    def set_timing(self, enabled: bool):
        _lib.check(_lib.load().sicc_fec_set_timing(self.handle, 1 if enabled else 0), "sicc_fec_set_timing")

    def kernel_ms(self):
        """(calls, bp_ms, osd_ms, osd_codewords) summed over the decode calls since the last query."""
        n, a, b, c = C.c_int(), C.c_float(), C.c_float(), C.c_longlong()
        _lib.check(_lib.load().sicc_fec_get_kernel_ms(self.handle, C.byref(n), C.byref(a), C.byref(b), C.byref(c)),
                   "sicc_fec_get_kernel_ms")
        return n.value, a.value, b.value, c.value

    # -- the reference wrapper's synchronous decode (L:3428-3539) --
    def decode(self, llrs: np.ndarray, device: bool = False):
        """Decode one frame of codewords; returns (info [blocks,k] uint8, used_osd count)."""
        L = _lib.load()
        blocks = int(llrs.shape[0])
        if blocks <= 0:
            raise ValueError("CUDA BP-OSD decoder received an empty frame")
        now = int(time.monotonic() * 1e6)
        ts = np.full(blocks, now, dtype=np.uint64)
        ids = np.full(blocks, self.frame_sequence, dtype=np.uint64)
        self.frame_sequence += 1
        bidx = np.arange(blocks, dtype=np.uint32)
        submit = L.cuda_osd_submit_device_codewords if device else L.cuda_osd_submit_codewords
        if not device:
            llrs = np.ascontiguousarray(llrs, dtype=np.float32)
        _lib.check(submit(self.handle, _lib.ptr(llrs), blocks, ts.ctypes.data, ids.ctypes.data, bidx.ctypes.data),
                   "cuda_osd_submit_codewords")
        _lib.check(L.cuda_osd_flush(self.handle), "cuda_osd_flush")
        info = np.zeros((blocks, self.k), dtype=np.uint8)
        tmp = np.zeros((blocks, self.k), dtype=np.uint8)
        o_ts = np.zeros(blocks, np.uint64)
        o_ids = np.zeros(blocks, np.uint64)
        o_blk = np.zeros(blocks, np.uint32)
        o_used = np.zeros(blocks, np.uint8)
        decoded = used = 0
        while decoded < blocks:
            ready = C.c_int(0)
            _lib.check(L.cuda_osd_poll_ready(self.handle, blocks, tmp.ctypes.data, o_ts.ctypes.data, o_ids.ctypes.data,
                                             o_blk.ctypes.data, o_used.ctypes.data, C.byref(ready)),
                       "cuda_osd_poll_ready")
            if ready.value <= 0:
                raise RuntimeError("CUDA BP-OSD flush returned no ready codewords")
            r = ready.value
            if np.any(o_blk[:r] >= blocks):
                raise RuntimeError("CUDA BP-OSD returned an invalid block index")
            info[o_blk[:r]] = tmp[:r]
            used += int(o_used[:r].sum())
            decoded += r
        return info, used

    # -- asynchronous window (L:3309-3426) --
    def submit(self, llrs, frame_ids, block_indices, device: bool = False, timestamps=None):
        L = _lib.load()
        cnt = int(len(block_indices))
        ts = np.asarray(timestamps if timestamps is not None else
                        np.full(cnt, int(time.monotonic() * 1e6)), dtype=np.uint64)
        ids = np.ascontiguousarray(frame_ids, dtype=np.uint64)
        bidx = np.ascontiguousarray(block_indices, dtype=np.uint32)
        fn = L.cuda_osd_submit_device_codewords if device else L.cuda_osd_submit_codewords
        if not device:
            llrs = np.ascontiguousarray(llrs, dtype=np.float32)
        _lib.check(fn(self.handle, _lib.ptr(llrs), cnt, ts.ctypes.data, ids.ctypes.data, bidx.ctypes.data),
                   "cuda_osd_submit_codewords")

    def flush(self):
        _lib.check(_lib.load().cuda_osd_flush(self.handle), "cuda_osd_flush")

    def poll_buffers(self, max_codewords: int):
        """Output arrays for ``poll`` (info, timestamps, frame_ids, block_indices, used_osd)."""
        return (np.zeros((max_codewords, self.k), np.uint8), np.zeros(max_codewords, np.uint64),
                np.zeros(max_codewords, np.uint64), np.zeros(max_codewords, np.uint32),
                np.zeros(max_codewords, np.uint8))

    def poll(self, max_codewords: int, bufs=None):
        """Returns (info [r,k], timestamps, frame_ids, block_indices, used_osd) for r ready codewords.

        ``bufs`` (from ``poll_buffers``, at least max_codewords long) avoids allocating per call.
        """
        L = _lib.load()
        tmp, o_ts, o_ids, o_blk, o_used = bufs if bufs is not None else self.poll_buffers(max_codewords)
        ready = C.c_int(0)
        _lib.check(L.cuda_osd_poll_ready(self.handle, max_codewords, tmp.ctypes.data, o_ts.ctypes.data,
                                         o_ids.ctypes.data, o_blk.ctypes.data, o_used.ctypes.data, C.byref(ready)),
                   "cuda_osd_poll_ready")
        r = ready.value
        return tmp[:r], o_ts[:r], o_ids[:r], o_blk[:r], o_used[:r]

    def stats(self) -> dict:
        s = _lib.StreamStats()
        _lib.check(_lib.load().cuda_osd_get_stats(self.handle, C.byref(s)), "cuda_osd_get_stats")
        return {f: getattr(s, f) for f, _ in _lib.StreamStats._fields_}

    # -- device-resident batch (extension) --
    def decode_device_batch(self, d_llr, d_info, d_success=None, d_used_osd=None, d_iter=None, stream=None,
                            count: int | None = None):
        cnt = int(d_llr.shape[0]) if count is None else count
        _lib.check(_lib.load().sicc_fec_decode_device(
            self.handle, _lib.ptr(d_llr), cnt, _lib.ptr(d_info), _lib.ptr(d_success), _lib.ptr(d_used_osd),
            _lib.ptr(d_iter), _stream_ptr(stream)), "sicc_fec_decode_device")


class CsrBpDecoder(_Shaped):
    """Generic CSR BP decoder (the reference's CudaBpDecoder)."""

    def __init__(self, n: int, m: int, row_ptr, col_ind, *, max_batch: int = 4096, max_iter: int = 20,
                 normalization: float = 0.75, offset: float = 0.0, damping: float = 0.0,
                 min_abs_llr_accept: float = 0.0, schedule: int = FLAT_LAYERED):
        L = _lib.load()
        self.row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
        self.col_ind = np.ascontiguousarray(col_ind, dtype=np.int32)
        cfg = _lib.BpCsrConfig(n=n, m=m, max_batch_size=max_batch, max_iterations=max_iter,
                               normalization=normalization, offset=offset, damping=damping,
                               min_abs_llr_accept=min_abs_llr_accept, nnz=int(self.row_ptr[-1]), schedule=schedule)
        h = _lib.u64(0)
        _lib.check(L.cuda_osd_create_bp_csr_decoder(C.byref(cfg), self.row_ptr.ctypes.data, self.col_ind.ctypes.data,
                                                    C.byref(h)), "cuda_osd_create_bp_csr_decoder")
        self.handle = h.value
        self.n, self.m, self.k = n, m, n - m

    @classmethod
    def for_code(cls, code: QcCode, **kw):
        return cls(code.n, code.m, code.row_ptr, code.col_ind, **kw)

    def close(self):
        if getattr(self, "handle", 0):
            _lib.check(_lib.load().cuda_osd_destroy_bp_csr_decoder(self.handle), "cuda_osd_destroy_bp_csr_decoder")
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_launch_shape(self, slots_per_cta: int, ctas: int):
        _lib.check(_lib.load().sicc_fec_set_launch_shape(self.handle, slots_per_cta, ctas), "sicc_fec_set_launch_shape")

    def decode(self, llrs, device: bool = False):
        """Returns (code_bits [B,n] uint8, success [B] uint8, total_decode_ms)."""
        L = _lib.load()
        blocks = int(llrs.shape[0])
        bits = np.zeros((blocks, self.n), np.uint8)
        ok = np.zeros(blocks, np.uint8)
        ms = C.c_double(0.0)
        if device:
            _lib.check(L.cuda_osd_decode_bp_csr_device_batch(self.handle, _lib.ptr(llrs), blocks, bits.ctypes.data,
                                                             ok.ctypes.data, C.byref(ms)),
                       "cuda_osd_decode_bp_csr_device_batch")
        else:
            llrs = np.ascontiguousarray(llrs, dtype=np.float32)
            _lib.check(L.cuda_osd_decode_bp_csr_batch(self.handle, llrs.ctypes.data, blocks, bits.ctypes.data,
                                                      ok.ctypes.data, C.byref(ms)), "cuda_osd_decode_bp_csr_batch")
        return bits, ok, ms.value

    def decode_device_batch(self, d_llr, d_bits=None, d_success=None, d_app=None, d_iter=None, stream=None,
                            count: int | None = None):
        cnt = int(d_llr.shape[0]) if count is None else count
        _lib.check(_lib.load().sicc_bp_csr_decode_device(
            self.handle, _lib.ptr(d_llr), cnt, _lib.ptr(d_bits), _lib.ptr(d_success), _lib.ptr(d_app),
            _lib.ptr(d_iter), _stream_ptr(stream)), "sicc_bp_csr_decode_device")


class OsdOnlyDecoder:
    """OSD-only batch decoder over the built-in CCSDS (128,64) code."""

    def __init__(self, max_batch: int = 4096):
        L = _lib.load()
        cfg = _lib.OsdConfig(n=128, k=64, max_batch_size=max_batch, osd_threads=256)
        h = _lib.u64(0)
        _lib.check(L.cuda_osd_create_osd_decoder(C.byref(cfg), C.byref(h)), "cuda_osd_create_osd_decoder")
        self.handle = h.value
        self.n, self.k = 128, 64

    def close(self):
        if getattr(self, "handle", 0):
            _lib.check(_lib.load().cuda_osd_destroy_osd_decoder(self.handle), "cuda_osd_destroy_osd_decoder")
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_osd_params(self, order: int, max_flip: int, max_tests: int):
        _lib.check(_lib.load().sicc_fec_set_osd_params(self.handle, order, max_flip, max_tests),
                   "sicc_fec_set_osd_params")

    def decode(self, llrs):
        L = _lib.load()
        llrs = np.ascontiguousarray(llrs, dtype=np.float32)
        b = llrs.shape[0]
        info = np.zeros((b, self.k), np.uint8)
        dist = np.zeros(b, np.float32)
        ms, mbps = C.c_double(0), C.c_double(0)
        _lib.check(L.cuda_osd_decode_osd_batch(self.handle, llrs.ctypes.data, b, info.ctypes.data, dist.ctypes.data,
                                               C.byref(ms), C.byref(mbps)), "cuda_osd_decode_osd_batch")
        return info, dist, ms.value, mbps.value

    def decode_device(self, d_llr, d_info, d_code=None, d_dist=None, stream=None):
        _lib.check(_lib.load().sicc_osd_decode_device(self.handle, _lib.ptr(d_llr), int(d_llr.shape[0]),
                                                      _lib.ptr(d_info), _lib.ptr(d_code), _lib.ptr(d_dist),
                                                      _stream_ptr(stream)), "sicc_osd_decode_device")


def find_frame(signal: np.ndarray, preamble: np.ndarray, pre_half_len: int, threshold: float, fs: float):
    """cuda_osd_find_frame: returns (start index 1-based or 0, peak, cfo_hz)."""
    L = _lib.load()
    sr = np.ascontiguousarray(signal.real, dtype=np.float64)
    si = np.ascontiguousarray(signal.imag, dtype=np.float64)
    pr = np.ascontiguousarray(preamble.real, dtype=np.float64)
    pi = np.ascontiguousarray(preamble.imag, dtype=np.float64)
    start, peak, cfo = C.c_int(0), C.c_double(0), C.c_double(0)
    _lib.check(L.cuda_osd_find_frame(sr.ctypes.data, si.ctypes.data, len(sr), pr.ctypes.data, pi.ctypes.data, len(pr),
                                     pre_half_len, threshold, fs, C.byref(start), C.byref(peak), C.byref(cfo)),
               "cuda_osd_find_frame")
    return start.value, peak.value, cfo.value
