"""The allocation-free BP->OSD entry point checked against the allocating one.

Some callers cannot allocate device memory when they decode: a receiver whose
device memory is fixed once it starts, or a receive loop with a sample
deadline, where a cudaMalloc may wait on work already queued on the GPU.  They
call sicc_fec_decode_device_static, which keeps the BP->OSD hand-off scratch in
a static device array of the library instead of per-decoder memory.  On the same
inputs its outputs must equal those of sicc_fec_decode_device bit for bit, on
every call: the array keeps the previous call's contents, so a second call in
a row checks that what must start at zero is cleared.

This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from sicc_gb300 import _lib, channel, codes, fec

pytestmark = pytest.mark.gpu


def _static_entry():
    return _lib.bind("sicc_fec_decode_device_static", C.c_int,
                     [_lib.u64, _lib.vp, C.c_int, _lib.vp, _lib.vp, _lib.vp, _lib.vp, _lib.vp])


def _outputs(torch, count, k, fill):
    return [torch.full((count, k), fill, dtype=torch.uint8, device="cuda"),
            torch.full((count,), fill, dtype=torch.uint8, device="cuda"),
            torch.full((count,), fill, dtype=torch.uint8, device="cuda"),
            torch.full((count,), fill, dtype=torch.uint8, device="cuda")]


def _decode_static(fn, dec, d_llr, outs, stream):
    info, ok, used, it = outs
    _lib.check(fn(dec.handle, d_llr.data_ptr(), int(d_llr.shape[0]), info.data_ptr(), ok.data_ptr(),
                  used.data_ptr(), it.data_ptr(), stream.cuda_stream), "sicc_fec_decode_device_static")


def test_static_scratch_entry_matches_allocating_entry(cuda):
    torch = cuda
    fn = _static_entry()
    code = codes.short_code()
    stream = torch.cuda.current_stream()
    # 2 dB: about a fifth of the frames fail BP and go through the scratch to OSD
    _, _, llr = channel.awgn_llrs(code, 6000, 2.0, seed=2024)
    d_llr = torch.from_numpy(llr).cuda()
    kw = dict(max_iter=20, normalization=0.75, offset=0.0, damping=0.0, min_abs_llr_accept=0.0)
    ref_dec = fec.StreamBpOsdDecoder(code, max_batch=8192, **kw)
    ref = _outputs(torch, 6000, code.k, 0)
    ref_dec.decode_device_batch(d_llr, ref[0], ref[1], ref[2], ref[3], stream=stream)
    torch.cuda.synchronize()
    assert int(ref[2].sum()) > 500  # the hand-off path is exercised

    # a decoder created with a small max_batch_size: the static entry is not bound by it
    dec = fec.StreamBpOsdDecoder(code, max_batch=64, min_batch=1, **kw)
    for call in range(2):
        outs = _outputs(torch, 6000, code.k, 0xAA)
        _decode_static(fn, dec, d_llr, outs, stream)
        torch.cuda.synchronize()
        for got, exp in zip(outs, ref):
            assert torch.equal(got, exp), f"call {call}"


def test_static_scratch_entry_rejects_oversized_batches(cuda):
    torch = cuda
    fn = _static_entry()
    code = codes.short_code()
    dec = fec.StreamBpOsdDecoder(code, max_batch=64, min_batch=1, max_iter=20, normalization=0.75, offset=0.0,
                                 damping=0.0, min_abs_llr_accept=0.0)
    cap = 8192
    d_llr = torch.zeros((cap + 1, code.n), dtype=torch.float32, device="cuda")
    outs = _outputs(torch, cap + 1, code.k, 0)
    st = fn(dec.handle, d_llr.data_ptr(), cap + 1, outs[0].data_ptr(), None, None, None, None)
    assert st == _lib.INVALID_ARGUMENT
    assert "8192" in _lib.last_error()
    # the largest batch is accepted
    _decode_static(fn, dec, d_llr[:cap], [o[:cap] for o in outs], torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert np.all(outs[0][:cap].cpu().numpy() == 0)  # all-zero LLRs decode to the all-zero word
