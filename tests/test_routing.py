"""Receive-decoder routing, pinned to the reference's own known answers.

tests/fec_offline_validation.cpp:70-107 (the reference's FEC test) fixes the
automatic routes: CCSDS (512,256) -> CPU min-sum, DVB-S2 (64800,32400) and NR
(25344, lifting 384) -> GPU BP requiring a GPU, Polar (16,8) -> SCL.  The
remaining cases follow rx_decoder_router.cpp:43-116 branch by branch.
"""
import pytest

from sicc_gb300 import routing
from sicc_gb300.routing import FecParams, RxDecoderKind, make_plan


def test_reference_known_answers():
    assert make_plan(FecParams("ldpc", 512, 256)).kind is RxDecoderKind.CPU_MIN_SUM
    dvbs2 = make_plan(FecParams("ldpc", 64800, 32400))
    assert dvbs2.kind is RxDecoderKind.GPU_BP and dvbs2.requires_gpu
    nr = make_plan(FecParams("nr", 25344, 8448, lifting_factor_zc=384))
    assert nr.kind is RxDecoderKind.GPU_BP
    assert make_plan(FecParams("polar", 16, 8)).kind is RxDecoderKind.POLAR_SCL


def test_long_codes_are_forced_to_gpu_bp_whatever_was_requested():
    for req in ("auto", "cuda-bp-osd", "osd-only", "cpu", "polar-scl"):
        p = make_plan(FecParams("ldpc", 1001, 500), req)
        assert p.kind is RxDecoderKind.GPU_BP and p.reason == "block_length > 1000: forced GPU BP decoder"
    assert make_plan(FecParams("ldpc", 1000, 500), "auto").kind is RxDecoderKind.CPU_MIN_SUM  # 1000 is short
    with pytest.raises(RuntimeError, match="non-empty CSR"):
        make_plan(FecParams("ldpc", 2048, 1024, csr_nonempty=False))
    with pytest.raises(RuntimeError, match="NR lifting factor"):
        make_plan(FecParams("nr", 25344, 8448, lifting_factor_zc=0))


@pytest.mark.parametrize("req,kind,reason", [
    ("cuda-bp-osd", RxDecoderKind.GPU_BP_OSD, "explicit short-code CUDA BP-OSD request"),
    ("GPU-BP-OSD", RxDecoderKind.GPU_BP_OSD, "explicit short-code CUDA BP-OSD request"),
    ("cuda-osd", RxDecoderKind.GPU_BP_OSD, "explicit short-code CUDA OSD-only request"),
    ("osd-only", RxDecoderKind.GPU_BP_OSD, "explicit short-code CUDA OSD-only request"),
    ("cuda-bp", RxDecoderKind.GPU_BP, "explicit GPU BP request"),
    ("gpu-bp", RxDecoderKind.GPU_BP, "explicit GPU BP request"),
    ("auto", RxDecoderKind.CPU_MIN_SUM, "auto: short LDPC code routes to CPU min-sum"),
    ("cpu", RxDecoderKind.CPU_MIN_SUM, "auto: short LDPC code routes to CPU min-sum"),
])
def test_short_ldpc_requests(req, kind, reason):
    p = make_plan(FecParams("ldpc", 128, 64), req)
    assert p.kind is kind and p.reason == reason
    assert p.requires_gpu == (kind in (RxDecoderKind.GPU_BP, RxDecoderKind.GPU_BP_OSD))


def test_polar_and_invalid_configs():
    assert make_plan(FecParams("polar", 64, 32), "scl").reason == "explicit short Polar SCL request"
    with pytest.raises(RuntimeError, match="non-Polar"):
        make_plan(FecParams("ldpc", 128, 64), "polar-scl")
    with pytest.raises(RuntimeError, match="null FEC config"):
        make_plan(None)
    with pytest.raises(RuntimeError, match="invalid FEC dimensions"):
        make_plan(FecParams("ldpc", 0, 64))
    assert [routing.to_string(k) for k in RxDecoderKind] == ["gpu-bp", "gpu-bp-osd", "cpu-min-sum", "polar-scl"]


def test_cpu_plans_are_not_built_here():
    with pytest.raises(RuntimeError, match="host decoders"):
        routing.build_decoder(make_plan(FecParams("ldpc", 128, 64)), code=None)


@pytest.mark.gpu
def test_gpu_plans_build_gb300_decoders(cuda):
    from sicc_gb300 import codes, engine, fec
    short = codes.short_code()
    d = routing.build_decoder(make_plan(FecParams("ldpc", short.n, short.k), "cuda-bp-osd"), short)
    assert isinstance(d, fec.StreamBpOsdDecoder)
    d = routing.build_decoder(make_plan(FecParams("ldpc", short.n, short.k), "cuda-bp"), short)
    assert isinstance(d, fec.CsrBpDecoder)
    big = [c for c in codes.mixed_codes() if c.n == 512][0]
    d = routing.build_decoder(make_plan(FecParams("ldpc", big.n, big.k), "cuda-bp-osd"), big)
    assert isinstance(d, engine.Engine)
