"""Launch shapes and the autotuner keep the decoders bit-exact.

Every shape the autotuner may pick must decode exactly as the default shape
does: the lanes that update one codeword's rows of a check-node layer
(rows of a layer share no variable), the codewords per CTA and the grid of
the layered BP kernel, the OSD warp's candidate rounds between best-metric
exchanges (pruning only drops candidates that cannot win), and the mixed
engine's warps per codeword of each code.  The tests force shapes across the
range, run the autotuner, and compare outputs with the defaults; a decoder
made after tuning starts from the tuned shape.
"""
import numpy as np
import pytest

from sicc_gb300 import channel, codes, engine, fec, tune

pytestmark = pytest.mark.gpu


def _stream(code, B):
    return fec.StreamBpOsdDecoder(code, max_batch=B, max_iter=20, normalization=0.75, offset=0.0, damping=0.0,
                                  min_abs_llr_accept=0.0, osd_order=2, osd_max_flip=64, osd_max_tests=4096)


def _run_stream(torch, dec, d_llr):
    B = d_llr.shape[0]
    out = [torch.full((B, dec.k), 0xAA, dtype=torch.uint8, device="cuda")] + \
          [torch.full((B,), 0xAA, dtype=torch.uint8, device="cuda") for _ in range(3)]
    dec.decode_device_batch(d_llr, *out, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in out]


def test_stream_decoder_shapes_are_bit_exact(cuda):
    torch = cuda
    tune.clear()
    code = codes.short_code()
    _, _, llr = channel.awgn_llrs(code, 8192, 2.0, seed=515)
    d_llr = torch.from_numpy(llr).cuda()
    dec = _stream(code, 8192)
    ref = _run_stream(torch, dec, d_llr)
    assert ref[2].sum() > 500  # plenty of OSD work at 2 dB
    shapes = [dict(lanes_per_codeword=16, slots_per_cta=8), dict(lanes_per_codeword=8),
              dict(lanes_per_codeword=8, slots_per_cta=32, ctas=152), dict(lanes_per_codeword=4, slots_per_cta=16),
              dict(lanes_per_codeword=2), dict(osd_share_rounds=1), dict(osd_share_rounds=8, osd_ctas=300)]
    for sh in shapes:
        dec.set_shape(**{**dict(lanes_per_codeword=0, slots_per_cta=0, ctas=0, osd_share_rounds=0, osd_ctas=0), **sh})
        got = _run_stream(torch, dec, d_llr)
        for a, b in zip(ref, got):
            assert np.array_equal(a, b), sh
    res = dec.autotune(d_llr, reps=2)
    assert len(res.trials) > 10 and res.best_ms <= res.default_ms
    assert dec.shape() == res.best
    got = _run_stream(torch, dec, d_llr)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b), res.best
    # a decoder made afterwards for the same code and settings starts from the tuned shape
    again = _stream(code, 8192)
    assert again.shape() == res.best
    assert tune.entries() >= 1
    tune.clear()


def test_invalid_shapes_are_rejected(cuda):
    from sicc_gb300 import _lib
    dec = _stream(codes.short_code(), 256)
    for bad in (dict(lanes_per_codeword=3), dict(lanes_per_codeword=64), dict(slots_per_cta=3),
                dict(lanes_per_codeword=16, slots_per_cta=32), dict(osd_share_rounds=65), dict(ctas=-1)):
        with pytest.raises(_lib.SiccError):
            dec.set_shape(**bad)


def test_csr_decoder_lanes_per_codeword_bit_exact(cuda):
    """The (1024,512) code of the OFDM workload (64-row layers: 32 lanes, 2 rows each, by default)."""
    torch = cuda
    code = codes.ofdm_code()
    _, _, llr = channel.awgn_llrs(code, 960, 1.6, seed=77)
    d_llr = torch.from_numpy(llr).cuda()
    dec = fec.CsrBpDecoder.for_code(code, max_batch=960, max_iter=25, normalization=0.75)

    def run():
        bits = torch.zeros((960, code.n), dtype=torch.uint8, device="cuda")
        ok = torch.zeros(960, dtype=torch.uint8, device="cuda")
        app = torch.zeros((960, code.n), dtype=torch.float32, device="cuda")
        it = torch.zeros(960, dtype=torch.uint8, device="cuda")
        dec.decode_device_batch(d_llr, bits, ok, app, it, stream=torch.cuda.current_stream())
        torch.cuda.synchronize()
        return bits.cpu().numpy(), ok.cpu().numpy(), app.cpu().numpy().view(np.uint32), it.cpu().numpy()

    ref = run()
    for lanes, slots in ((16, 4), (8, 8), (32, 2)):
        dec.set_shape(lanes_per_codeword=lanes, slots_per_cta=slots, ctas=0)
        got = run()
        for a, b in zip(ref, got):
            assert np.array_equal(a, b), (lanes, slots)
    tune.clear()
    res = dec.autotune(d_llr, reps=1)
    got = run()
    for a, b in zip(ref, got):
        assert np.array_equal(a, b), res.best
    tune.clear()


def test_engine_code_warps_and_autotune_bit_exact(cuda):
    torch = cuda
    tune.clear()
    cs = codes.mixed_codes()
    w = engine.mixed_workload(total=6000, seed=21, max_burst=64, code_set=cs)
    eng = engine.Engine(max_codewords=w.count, max_llr_floats=w.llr.size)
    for c in cs:
        eng.add_code(c, engine.iteration_cap(c.n), 0.75, 0.0, engine.osd_order_for(c), 64, 4096)
    d = dict(code=torch.from_numpy(w.code_of).cuda(), llr=torch.from_numpy(w.llr).cuda(),
             llr_off=torch.from_numpy(w.llr_off).cuda(), info_off=torch.from_numpy(w.info_off).cuda())

    def run():
        info = torch.full((w.info_bits,), 0xAA, dtype=torch.uint8, device="cuda")
        ok = torch.full((w.count,), 0xAA, dtype=torch.uint8, device="cuda")
        used = torch.full((w.count,), 0xAA, dtype=torch.uint8, device="cuda")
        it = torch.zeros(w.count, dtype=torch.uint8, device="cuda")
        eng.decode_device(w.count, d["code"], d["llr"], d["llr_off"], info, d["info_off"], ok, used, it,
                          stream=torch.cuda.current_stream())
        torch.cuda.synchronize()
        return info.cpu().numpy(), ok.cpu().numpy(), used.cpu().numpy(), it.cpu().numpy()

    ref = run()
    wide = [i for i, c in enumerate(cs) if eng.code_warps(i) == 4]
    assert wide, "the mix has codes with 128-row layers"
    for warps in (2, 1):
        for i in wide:
            eng.set_code_warps(i, warps)
        got = run()
        for a, b in zip(ref, got):
            assert np.array_equal(a, b), warps
    for i in wide:
        eng.set_code_warps(i, 4)
    scratch = torch.zeros(w.info_bits, dtype=torch.uint8, device="cuda")
    base_ms, tuned_ms = eng.autotune(w.count, d["code"], d["llr"], d["llr_off"], scratch, d["info_off"], reps=2)
    assert tuned_ms <= base_ms
    got = run()
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    # an engine made afterwards starts its codes from the tuned warps
    eng2 = engine.Engine(max_codewords=w.count, max_llr_floats=w.llr.size)
    for c in cs:
        eng2.add_code(c, engine.iteration_cap(c.n), 0.75, 0.0, engine.osd_order_for(c), 64, 4096)
    assert [eng2.code_warps(i) for i in range(len(cs))] == [eng.code_warps(i) for i in range(len(cs))]
    tune.clear()
