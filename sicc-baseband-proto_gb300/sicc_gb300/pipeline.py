"""Host wrapper of the OFDM receive pipeline (include/sicc_pipe.h).

Mirrors the reference bridge class usrp_gpu_pipeline_bridge::Pipeline
(source/cpp_cuda/uhd_cpp/src/gpu_ofdm_pipeline.hpp:65-93): constructor with a
Config and a slot count, upload_static_tables, find_frame[_device],
demod_frame_to_device_llr, demod_frame_device_to_device_llr,
demod_frame_to_host_llr, and the transmit members submit_tx_frame_async,
submit_tx_frame_device_async, synchronize_tx; plus the batched device
extensions (receive and transmit).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .ofdm import Tables


class PipeConfig(C.Structure):
    _fields_ = [("nfft", C.c_int), ("cp", C.c_int), ("preamble_len", C.c_int), ("pre_half_len", C.c_int),
                ("num_symbols", C.c_int), ("active_sc", C.c_int), ("bits_per_symbol", C.c_int), ("code_n", C.c_int),
                ("code_k", C.c_int), ("blocks_per_frame", C.c_int), ("max_rx_search_samples", C.c_int),
                ("sample_rate", C.c_float), ("sync_threshold", C.c_float), ("tx_amplitude", C.c_float),
                ("demod_noise_var", C.c_float), ("use_pilot_channel_est", C.c_int), ("sync_radius", C.c_int),
                ("max_batch_frames", C.c_int)]


class PipeTables(C.Structure):
    _fields_ = [("used_indices", C.c_void_p), ("pilot_symbols", C.c_void_p), ("pilot_count", C.c_int),
                ("data_symbols", C.c_void_p), ("data_count", C.c_int), ("interp_p0", C.c_void_p),
                ("interp_p1", C.c_void_p), ("interp_alpha", C.c_void_p), ("pilot_grid", C.c_void_p),
                ("preamble", C.c_void_p)]


class PipeTxTables(C.Structure):
    _fields_ = [("generator_kn", C.c_void_p), ("dvb_s2_accumulator", C.c_int), ("row_info_offsets", C.c_void_p),
                ("row_info_cols", C.c_void_p), ("precomp_h", C.c_void_p), ("actual_h", C.c_void_p)]


class PipeSync(C.Structure):
    _fields_ = [("start", C.c_int), ("metric", C.c_float), ("cfo_hz", C.c_float)]


#: dtype of one device search record (sicc_pipe_sync_record_t)
SYNC_RECORD = np.dtype([("found", np.int32), ("start", np.int32), ("coarse", np.float32), ("fine", np.float32),
                        ("cfo_hz", np.float32), ("coarse_start", np.int32)])

_SIGS = {
    "sicc_pipe_create": (C.c_int, [C.POINTER(PipeConfig), C.c_int, C.POINTER(C.c_ulonglong)]),
    "sicc_pipe_destroy": (C.c_int, [C.c_ulonglong]),
    "sicc_pipe_upload_static_tables": (C.c_int, [C.c_ulonglong, C.POINTER(PipeTables)]),
    "sicc_pipe_find_frame": (C.c_int, [C.c_ulonglong, C.c_int, C.c_void_p, C.c_int, C.POINTER(PipeSync)]),
    "sicc_pipe_find_frame_device": (C.c_int, [C.c_ulonglong, C.c_int, C.c_void_p, C.c_int, C.POINTER(PipeSync)]),
    "sicc_pipe_demod_to_device": (C.c_int, [C.c_ulonglong, C.c_int, C.c_void_p, C.POINTER(PipeSync),
                                            C.POINTER(C.c_void_p)]),
    "sicc_pipe_demod_device_to_device": (C.c_int, [C.c_ulonglong, C.c_int, C.c_void_p, C.POINTER(PipeSync),
                                                   C.POINTER(C.c_void_p)]),
    "sicc_pipe_demod_to_host": (C.c_int, [C.c_ulonglong, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(PipeSync)]),
    "sicc_pipe_demod_batch": (C.c_int, [C.c_ulonglong, C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p,
                                        C.c_void_p, C.c_void_p]),
    "sicc_pipe_demod_gather": (C.c_int, [C.c_ulonglong, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p]),
    "sicc_pipe_last_batch_ms": (C.c_int, [C.c_ulonglong, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "sicc_pipe_upload_tx_tables": (C.c_int, [C.c_ulonglong, C.POINTER(PipeTxTables)]),
    "sicc_pipe_tx_frame_device": (C.c_int, [C.c_ulonglong, C.c_int, C.c_void_p, C.c_float, C.c_ulonglong, C.c_int,
                                            C.POINTER(C.c_void_p)]),
    "sicc_pipe_tx_frame": (C.c_int, [C.c_ulonglong, C.c_int, C.c_void_p, C.c_void_p]),
    "sicc_pipe_tx_synchronize": (C.c_int, [C.c_ulonglong, C.c_int]),
    "sicc_pipe_tx_batch": (C.c_int, [C.c_ulonglong, C.c_void_p, C.c_int, C.c_void_p, C.c_float, C.c_ulonglong,
                                     C.c_void_p]),
}


def wait_timeouts() -> int:
    """Demodulator waits on staged-sample copies that hit their iteration limit (expected 0)."""
    out = C.c_uint(0)
    _lib.check(_lib.bind("sicc_pipe_wait_timeouts", C.c_int, [C.POINTER(C.c_uint)])(C.byref(out)),
               "sicc_pipe_wait_timeouts")
    return out.value


def _fn(name):
    res, args = _SIGS[name]
    return _lib.bind(name, res, args)


def _sync_tuple(s: PipeSync):
    return s.start, s.metric, s.cfo_hz


def pipe_structs(tables: Tables, code_n: int, code_k: int, blocks_per_frame: int, noise_var: float,
                 max_rx_search_samples: int = 0, max_batch_frames: int = 256, sync_radius: int = 0,
                 use_pilot_channel_est: bool = True):
    """(PipeConfig, PipeTables, arrays the tables point into) for one PHY profile."""
    cfg = tables.cfg
    c = PipeConfig(nfft=cfg.nfft, cp=cfg.cp, preamble_len=2 * cfg.pre_half_len, pre_half_len=cfg.pre_half_len,
                   num_symbols=cfg.num_symbols, active_sc=cfg.active_sc, bits_per_symbol=cfg.bits_per_symbol,
                   code_n=code_n, code_k=code_k, blocks_per_frame=blocks_per_frame,
                   max_rx_search_samples=max_rx_search_samples, sample_rate=cfg.sample_rate,
                   sync_threshold=cfg.sync_threshold, tx_amplitude=cfg.amplitude, demod_noise_var=noise_var,
                   use_pilot_channel_est=1 if use_pilot_channel_est else 0, sync_radius=sync_radius,
                   max_batch_frames=max_batch_frames)
    keep = dict(used=np.ascontiguousarray(tables.used_indices, np.int32),
                pil=np.ascontiguousarray(tables.pilot_symbols, np.int32),
                dat=np.ascontiguousarray(tables.data_symbols, np.int32),
                p0=np.ascontiguousarray(tables.interp_p0, np.int32),
                p1=np.ascontiguousarray(tables.interp_p1, np.int32),
                al=np.ascontiguousarray(tables.interp_alpha, np.float32),
                grid=np.ascontiguousarray(tables.pilot_grid, np.complex64),
                pre=np.ascontiguousarray(tables.preamble, np.complex64))
    t = PipeTables(used_indices=keep["used"].ctypes.data, pilot_symbols=keep["pil"].ctypes.data,
                   pilot_count=len(keep["pil"]), data_symbols=keep["dat"].ctypes.data,
                   data_count=len(keep["dat"]), interp_p0=keep["p0"].ctypes.data,
                   interp_p1=keep["p1"].ctypes.data, interp_alpha=keep["al"].ctypes.data,
                   pilot_grid=keep["grid"].ctypes.data, preamble=keep["pre"].ctypes.data)
    return c, t, keep


class RxPipeline:
    def __init__(self, tables: Tables, code_n: int, code_k: int, blocks_per_frame: int, noise_var: float,
                 slots: int = 3, max_rx_search_samples: int = 0, max_batch_frames: int = 256, sync_radius: int = 0,
                 use_pilot_channel_est: bool = True):
        c, t, keep = pipe_structs(tables, code_n, code_k, blocks_per_frame, noise_var, max_rx_search_samples,
                                  max_batch_frames, sync_radius, use_pilot_channel_est)
        h = C.c_ulonglong(0)
        _lib.check(_fn("sicc_pipe_create")(C.byref(c), slots, C.byref(h)), "sicc_pipe_create")
        self.handle = h.value
        self.tables = tables
        self.coded_bits = blocks_per_frame * code_n
        self.frame_samples = tables.frame_len
        _lib.check(_fn("sicc_pipe_upload_static_tables")(self.handle, C.byref(t)), "upload_static_tables")

    def close(self):
        if getattr(self, "handle", 0):
            _lib.check(_fn("sicc_pipe_destroy")(self.handle), "sicc_pipe_destroy")
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def find_frame(self, slot: int, iq: np.ndarray):
        x = np.ascontiguousarray(iq, np.complex64)
        s = PipeSync()
        _lib.check(_fn("sicc_pipe_find_frame")(self.handle, slot, x.ctypes.data, x.shape[0], C.byref(s)), "find_frame")
        return _sync_tuple(s)

    def find_frame_device(self, slot: int, d_iq, count: int):
        s = PipeSync()
        _lib.check(_fn("sicc_pipe_find_frame_device")(self.handle, slot, _lib.ptr(d_iq), count, C.byref(s)),
                   "find_frame_device")
        return _sync_tuple(s)

    def demod_to_device(self, slot: int, frame: np.ndarray):
        x = np.ascontiguousarray(frame, np.complex64)
        s = PipeSync()
        d = C.c_void_p()
        _lib.check(_fn("sicc_pipe_demod_to_device")(self.handle, slot, x.ctypes.data, C.byref(s), C.byref(d)),
                   "demod_frame_to_device_llr")
        return d.value, _sync_tuple(s)

    def demod_device_to_device(self, slot: int, d_frame, cfo_hz: float, metric: float = 1.0):
        s = PipeSync(start=0, metric=metric, cfo_hz=cfo_hz)
        d = C.c_void_p()
        _lib.check(_fn("sicc_pipe_demod_device_to_device")(self.handle, slot, _lib.ptr(d_frame), C.byref(s),
                                                           C.byref(d)), "demod_frame_device_to_device_llr")
        return d.value

    def demod_to_host(self, slot: int, frame: np.ndarray):
        x = np.ascontiguousarray(frame, np.complex64)
        out = np.zeros(self.coded_bits, np.float32)
        s = PipeSync()
        _lib.check(_fn("sicc_pipe_demod_to_host")(self.handle, slot, x.ctypes.data, out.ctypes.data, C.byref(s)),
                   "demod_frame_to_host_llr")
        return out, _sync_tuple(s)

    def demod_batch(self, d_iq, stride: int, sample_count: int, frames: int, d_llr, d_sync=None, stream=None):
        st = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        _lib.check(_fn("sicc_pipe_demod_batch")(self.handle, _lib.ptr(d_iq), stride, sample_count, frames,
                                                _lib.ptr(d_llr), _lib.ptr(d_sync), st), "sicc_pipe_demod_batch")

    def demod_gather(self, d_iq, d_frame_off, sample_count: int, frames: int, d_llr, d_llr_off, d_sync, stream=None):
        """Frames at d_iq + frame_off[f] (complex samples) -> LLRs at d_llr + llr_off[f] (floats)."""
        st = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        p = _lib.ptr
        _lib.check(_fn("sicc_pipe_demod_gather")(self.handle, p(d_iq), p(d_frame_off), sample_count, frames, p(d_llr),
                                                 p(d_llr_off), p(d_sync), st), "sicc_pipe_demod_gather")

    def set_demod_shape(self, symbols_per_cta: int):
        """Data symbols per demodulator CTA (results do not depend on it)."""
        fn = _lib.bind("sicc_pipe_set_demod_shape", C.c_int, [_lib.u64, C.c_int])
        _lib.check(fn(self.handle, symbols_per_cta), "sicc_pipe_set_demod_shape")

    def last_batch_ms(self):
        a, b = C.c_float(), C.c_float()
        _lib.check(_fn("sicc_pipe_last_batch_ms")(self.handle, C.byref(a), C.byref(b)), "sicc_pipe_last_batch_ms")
        return a.value, b.value

    # ---- transmit (gpu_ofdm_pipeline.cu:854-1075) ----
    def upload_tx_tables(self, generator_kn=None, accumulator=None, precomp_h=None, actual_h=None):
        """generator_kn: [k][n] 0/1; or accumulator=(row_info_offsets [m+1], row_info_cols)."""
        keep = {}
        t = PipeTxTables()
        if accumulator is not None:
            keep["off"] = np.ascontiguousarray(accumulator[0], np.int32)
            keep["cols"] = np.ascontiguousarray(accumulator[1], np.int32)
            t.dvb_s2_accumulator = 1
            t.row_info_offsets = keep["off"].ctypes.data
            t.row_info_cols = keep["cols"].ctypes.data if keep["cols"].size else None
        else:
            keep["gen"] = np.ascontiguousarray(generator_kn, np.uint8)
            t.generator_kn = keep["gen"].ctypes.data
        for name, arr in (("precomp_h", precomp_h), ("actual_h", actual_h)):
            if arr is not None:
                keep[name] = np.ascontiguousarray(arr, np.complex64)
                setattr(t, name, keep[name].ctypes.data)
        _lib.check(_fn("sicc_pipe_upload_tx_tables")(self.handle, C.byref(t)), "upload_static_tables (TX)")

    def tx_frame(self, slot: int, info_bits: np.ndarray) -> np.ndarray:
        """submit_tx_frame_async + synchronize_tx: one frame of info bits -> complex64 frame."""
        u = np.ascontiguousarray(info_bits, np.uint8)
        out = np.zeros(self.frame_samples, np.complex64)
        _lib.check(_fn("sicc_pipe_tx_frame")(self.handle, slot, u.ctypes.data, out.ctypes.data), "submit_tx_frame_async")
        self.tx_synchronize(slot)
        return out

    def tx_frame_device(self, slot: int, info_bits: np.ndarray, noise_var: float = 0.0, seed: int = 0,
                        add_noise: bool = False) -> int:
        """submit_tx_frame_device_async: the device address of the slot's frame."""
        u = np.ascontiguousarray(info_bits, np.uint8)
        d = C.c_void_p()
        _lib.check(_fn("sicc_pipe_tx_frame_device")(self.handle, slot, u.ctypes.data, noise_var, seed,
                                                    1 if add_noise else 0, C.byref(d)), "submit_tx_frame_device_async")
        return d.value

    def tx_synchronize(self, slot: int):
        _lib.check(_fn("sicc_pipe_tx_synchronize")(self.handle, slot), "synchronize_tx")

    def tx_batch(self, d_info, frames: int, d_frames, noise_var: float = 0.0, seed: int = 0, stream=None):
        st = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        _lib.check(_fn("sicc_pipe_tx_batch")(self.handle, _lib.ptr(d_info), frames, _lib.ptr(d_frames), noise_var,
                                             seed, st), "sicc_pipe_tx_batch")


#: The bridge class name of the reference: one pipeline object serves both directions.
Pipeline = RxPipeline
