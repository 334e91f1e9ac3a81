"""Receive-decoder routing and the GB300 decoder each route maps to.

``make_plan`` restates the reference's ``RxDecoderRouter::make_plan``
(source/cpp_cuda/uhd_cpp/src/rx_decoder_router.cpp:43-116): block lengths
above 1000 are forced to GPU BP whatever was requested (with the CSR / NR
lifting-factor checks of :20-40), explicit requests are honoured, a short
Polar code goes to SCL and any other short code to the CPU min-sum decoder.
Names, reasons and errors are the reference's (``std::runtime_error`` becomes
``RuntimeError``).

``build_decoder`` instantiates the GB300 decoder of a GPU plan: the CSR BP
decoder for ``gpu-bp`` and the stream BP->OSD decoder for ``gpu-bp-osd``
(the reference decoder library's limits, n <= 256 and k <= 128; longer codes
get a one-code engine with the large-code OSD).  CPU and Polar plans stay
with the reference's own host decoders: this library has no CPU path.
"""
from __future__ import annotations

from dataclasses import dataclass
from enum import Enum


class RxDecoderKind(Enum):
    GPU_BP = "gpu-bp"
    GPU_BP_OSD = "gpu-bp-osd"
    CPU_MIN_SUM = "cpu-min-sum"
    POLAR_SCL = "polar-scl"


@dataclass
class FecParams:
    """The parts of the reference's FecConfig (fec_config.hpp) that routing reads."""
    family: str                 # "ldpc" (CSR-defined, DvbS2LdpcParams), "nr" (NrLdpcParams) or "polar"
    block_length: int
    information_length: int
    csr_nonempty: bool = True   # ldpc: row_ptr, col_ind and val all present
    lifting_factor_zc: int = 0  # nr


@dataclass
class RxDecoderPlan:
    kind: RxDecoderKind
    fec: FecParams
    reason: str
    requires_gpu: bool


def to_string(kind: RxDecoderKind) -> str:
    return kind.value


def _validate_gpu_bp_input(fec: FecParams) -> None:
    if fec.family == "ldpc" and not fec.csr_nonempty:
        raise RuntimeError("GPU BP routing requires non-empty CSR matrix")
    if fec.family == "nr" and fec.lifting_factor_zc <= 0:
        raise RuntimeError("GPU BP routing requires a valid NR lifting factor")


def make_plan(fec: FecParams | None, requested: str = "auto") -> RxDecoderPlan:
    if fec is None:
        raise RuntimeError("RX decoder routing received a null FEC config")
    if fec.block_length <= 0 or fec.information_length <= 0:
        raise RuntimeError("RX decoder routing received invalid FEC dimensions")
    req = requested.lower()
    if fec.block_length > 1000:  # strict rule: long codes always go to GPU BP
        _validate_gpu_bp_input(fec)
        return RxDecoderPlan(RxDecoderKind.GPU_BP, fec, "block_length > 1000: forced GPU BP decoder", True)
    if req in ("cuda-bp-osd", "gpu-bp-osd"):
        return RxDecoderPlan(RxDecoderKind.GPU_BP_OSD, fec, "explicit short-code CUDA BP-OSD request", True)
    if req in ("cuda-osd", "gpu-osd", "osd-only"):
        return RxDecoderPlan(RxDecoderKind.GPU_BP_OSD, fec, "explicit short-code CUDA OSD-only request", True)
    if req in ("polar-scl", "scl"):
        if fec.family != "polar":
            raise RuntimeError("polar-scl requested for a non-Polar FEC config")
        return RxDecoderPlan(RxDecoderKind.POLAR_SCL, fec, "explicit short Polar SCL request", False)
    if req in ("cuda-bp", "gpu-bp"):
        _validate_gpu_bp_input(fec)
        return RxDecoderPlan(RxDecoderKind.GPU_BP, fec, "explicit GPU BP request", True)
    if fec.family == "polar":
        return RxDecoderPlan(RxDecoderKind.POLAR_SCL, fec, "auto: short Polar code routes to SCL", False)
    return RxDecoderPlan(RxDecoderKind.CPU_MIN_SUM, fec, "auto: short LDPC code routes to CPU min-sum", False)


def build_decoder(plan: RxDecoderPlan, code, *, max_batch: int = 4096, min_batch: int = 30, max_iter: int = 20,
                  normalization: float = 0.80, osd_order: int = 2):
    """The GB300 decoder for a GPU plan (defaults: the reference's RxDecoderRuntimeOptions)."""
    from . import engine, fec
    if plan.kind is RxDecoderKind.GPU_BP:
        return fec.CsrBpDecoder.for_code(code, max_batch=max_batch, max_iter=max_iter, normalization=normalization)
    if plan.kind is RxDecoderKind.GPU_BP_OSD:
        if engine.osd_supported(code):
            return fec.StreamBpOsdDecoder(code, max_batch=max_batch, min_batch=min_batch, max_iter=max_iter,
                                          normalization=normalization, osd_order=osd_order)
        eng = engine.Engine(max_codewords=max_batch, max_llr_floats=max_batch * code.n, max_codes=1)
        eng.add_code(code, max_iter, normalization, 0.0, osd_order)
        return eng
    raise RuntimeError(f"{to_string(plan.kind)} plans run on the host decoders of the link; "
                       "the GB300 library decodes gpu-bp and gpu-bp-osd plans")
