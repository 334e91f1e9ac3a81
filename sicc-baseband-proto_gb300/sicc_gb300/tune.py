"""Launch shapes and the autotuner (include/sicc_tune.h).

The stream and CSR decoders and the mixed-code engine expose their kernel
shapes here: lanes per codeword and codewords per CTA of the layered BP
kernel, the OSD warp's candidate rounds between best-metric exchanges, the
grids, and the mixed engine's warps per codeword of each code.  ``autotune``
times candidates on a caller's batch and applies the fastest; the library
remembers it per (code, settings, device) for decoders made later, and
``save`` / ``load`` carry that cache across processes.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import _lib


class FecShape(C.Structure):
    _fields_ = [("lanes_per_codeword", C.c_int), ("slots_per_cta", C.c_int), ("ctas", C.c_int),
                ("osd_share_rounds", C.c_int), ("osd_ctas", C.c_int)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class TuneTrial(C.Structure):
    _fields_ = [("shape", FecShape), ("ms", C.c_float)]


_SIGS = {
    "sicc_fec_get_shape": (C.c_int, [_lib.u64, C.POINTER(FecShape)]),
    "sicc_fec_set_shape": (C.c_int, [_lib.u64, C.POINTER(FecShape)]),
    "sicc_fec_autotune": (C.c_int, [_lib.u64, _lib.vp, C.c_int, C.c_int, C.POINTER(FecShape), C.POINTER(TuneTrial),
                                    C.c_int, C.POINTER(C.c_int)]),
    "sicc_engine_set_code_warps": (C.c_int, [_lib.u64, C.c_int, C.c_int]),
    "sicc_engine_get_code_warps": (C.c_int, [_lib.u64, C.c_int, C.POINTER(C.c_int)]),
    "sicc_engine_autotune": (C.c_int, [_lib.u64, C.c_int, _lib.vp, _lib.vp, _lib.vp, _lib.vp, _lib.vp, C.c_int,
                                       C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "sicc_tune_save": (C.c_int, [C.c_char_p]),
    "sicc_tune_load": (C.c_int, [C.c_char_p]),
    "sicc_tune_clear": (C.c_int, []),
    "sicc_tune_entries": (C.c_int, []),
}


def _fn(name):
    res, args = _SIGS[name]
    return _lib.bind(name, res, args)


@dataclass
class TuneResult:
    best: dict
    trials: list  # [(shape dict, median ms)]

    @property
    def best_ms(self) -> float:
        return min(ms for _, ms in self.trials)

    @property
    def default_ms(self) -> float:
        return self.trials[0][1]


def get_shape(handle: int) -> dict:
    s = FecShape()
    _lib.check(_fn("sicc_fec_get_shape")(handle, C.byref(s)), "sicc_fec_get_shape")
    return s.as_dict()


def set_shape(handle: int, **fields) -> None:
    s = FecShape(**{**get_shape(handle), **fields})
    _lib.check(_fn("sicc_fec_set_shape")(handle, C.byref(s)), "sicc_fec_set_shape")


def autotune(handle: int, d_llr, codewords: int | None = None, reps: int = 5) -> TuneResult:
    """Sweeps shapes of a stream or CSR decoder on device LLRs; applies and caches the fastest."""
    cnt = int(d_llr.shape[0]) if codewords is None else codewords
    best = FecShape()
    trials = (TuneTrial * 256)()
    count = C.c_int(0)
    _lib.check(_fn("sicc_fec_autotune")(handle, _lib.ptr(d_llr), cnt, reps, C.byref(best), trials, 256,
                                        C.byref(count)), "sicc_fec_autotune")
    return TuneResult(best.as_dict(), [(trials[i].shape.as_dict(), float(trials[i].ms))
                                       for i in range(min(count.value, 256))])


def set_code_warps(engine_handle: int, code_id: int, warps: int) -> None:
    _lib.check(_fn("sicc_engine_set_code_warps")(engine_handle, code_id, warps), "sicc_engine_set_code_warps")


def code_warps(engine_handle: int, code_id: int) -> int:
    w = C.c_int(0)
    _lib.check(_fn("sicc_engine_get_code_warps")(engine_handle, code_id, C.byref(w)), "sicc_engine_get_code_warps")
    return w.value


def engine_autotune(engine_handle: int, codewords: int, d_code, d_llr, d_llr_off, d_info, d_info_off,
                    reps: int = 3) -> tuple[float, float]:
    """Tunes an engine's warps per codeword of each code and warps per CTA; returns
    (default BP ms, tuned BP ms) on the given batch."""
    a, b = C.c_float(0), C.c_float(0)
    _lib.check(_fn("sicc_engine_autotune")(engine_handle, codewords, _lib.ptr(d_code), _lib.ptr(d_llr),
                                           _lib.ptr(d_llr_off), _lib.ptr(d_info), _lib.ptr(d_info_off), reps,
                                           C.byref(a), C.byref(b)), "sicc_engine_autotune")
    return a.value, b.value


def save(path: str) -> None:
    _lib.check(_fn("sicc_tune_save")(path.encode()), "sicc_tune_save")


def load(path: str) -> None:
    _lib.check(_fn("sicc_tune_load")(path.encode()), "sicc_tune_load")


def clear() -> None:
    _fn("sicc_tune_clear")()


def entries() -> int:
    return int(_fn("sicc_tune_entries")())
