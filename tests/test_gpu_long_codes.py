"""GPU parity of the long-code BP path (codes too large for one CTA's shared memory).

DVB-S2-sized IRA codes (N16200, N64800) through the reference-facing CSR BP
decoder (cuda_osd_create_bp_csr_decoder / decode_bp_csr_device_batch), which
hands them to the CTA-per-codeword kernels of csrc/bp_wide.cu.  Bar, as for
the short codes: hard decisions, success flags, iteration counts and the
posterior LLRs bit for bit against the single-precision oracle of the same
schedule.
"""
import numpy as np
import pytest

from sicc_gb300 import channel, codes

pytestmark = pytest.mark.gpu


def _run(torch, dec, llr, n):
    b = llr.shape[0]
    d_llr = torch.from_numpy(np.ascontiguousarray(llr)).cuda()
    d_bits = torch.zeros((b, n), dtype=torch.uint8, device="cuda")
    d_ok = torch.zeros(b, dtype=torch.uint8, device="cuda")
    d_app = torch.zeros((b, n), dtype=torch.float32, device="cuda")
    d_it = torch.zeros(b, dtype=torch.uint8, device="cuda")
    dec.decode_device_batch(d_llr, d_bits, d_ok, d_app, d_it, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    return d_bits.cpu().numpy(), d_ok.cpu().numpy(), d_app.cpu().numpy(), d_it.cpu().numpy()


def _llrs(code, ebn0, frames, seed):
    return channel.awgn_llrs(code, frames, ebn0, seed)[2]


def _check(o, bits, ok, app, it):
    assert bool(ok) == o[0]
    assert int(it) == o[4]
    assert np.array_equal(bits, o[1])
    assert np.array_equal(app.view(np.uint32), o[2].view(np.uint32))


@pytest.mark.parametrize("name,ebn0,frames", [("N16200_R1/2", (1.2, 1.8, 2.2), 3), ("N64800_R1/2", (1.5, 2.2), 3)])
def test_colored_layered_long_code(cuda, oracle, name, ebn0, frames):
    from sicc_gb300 import fec
    code = codes.dvbs2_code(name)
    oc = oracle.code(code.n, code.m, code.row_ptr, code.col_ind)
    order, _, _ = oc.color_order()
    llr = np.concatenate([_llrs(code, e, frames, 40 + i) for i, e in enumerate(ebn0)])
    dec = fec.CsrBpDecoder(code.n, code.m, code.row_ptr, code.col_ind, max_batch=llr.shape[0], max_iter=25,
                           normalization=0.75, schedule=fec.COLORED_LAYERED)
    bits, ok, app, it = _run(cuda, dec, llr, code.n)
    for i, x in enumerate(llr):
        _check(oc.layered(x, 25, 0.75, row_order=order), bits[i], ok[i], app[i], it[i])
    assert ok.any() and not ok.all()  # both outcomes covered


def test_flat_layered_long_code(cuda, oracle):
    """Row-by-row layers (the accumulator chain joins consecutive rows): one barrier per row."""
    from sicc_gb300 import fec
    code = codes.dvbs2_code("N16200_R1/4")
    oc = oracle.code(code.n, code.m, code.row_ptr, code.col_ind)
    llr = _llrs(code, 0.5, 3, 60)
    dec = fec.CsrBpDecoder(code.n, code.m, code.row_ptr, code.col_ind, max_batch=3, max_iter=4,
                           normalization=0.8, offset=0.1, schedule=fec.FLAT_LAYERED)
    bits, ok, app, it = _run(cuda, dec, llr, code.n)
    for i, x in enumerate(llr):
        _check(oc.layered(x, 4, 0.8, 0.1), bits[i], ok[i], app[i], it[i])


@pytest.mark.parametrize("damping", [0.0, 0.15])
def test_flooding_long_code(cuda, oracle, damping):
    from sicc_gb300 import fec
    code = codes.dvbs2_code("N16200_R1/2")
    oc = oracle.code(code.n, code.m, code.row_ptr, code.col_ind)
    llr = np.concatenate([_llrs(code, 1.2, 3, 70), _llrs(code, 1.8, 3, 71)])
    dec = fec.CsrBpDecoder(code.n, code.m, code.row_ptr, code.col_ind, max_batch=llr.shape[0], max_iter=30,
                           normalization=0.8, offset=0.15, damping=damping, schedule=fec.FLOODING)
    bits, ok, app, it = _run(cuda, dec, llr, code.n)
    for i, x in enumerate(llr):
        _check(oc.flooding(x, 30, 0.8, 0.15, damping), bits[i], ok[i], app[i], it[i])


def test_host_batches_in_chunks(cuda):
    """The host entry point (cuda_osd_decode_bp_csr_batch) splits a batch larger than max_batch."""
    from sicc_gb300 import fec
    code = codes.dvbs2_code("N64800_R1/2")
    llr = _llrs(code, 2.5, 5, 80)
    dec = fec.CsrBpDecoder(code.n, code.m, code.row_ptr, code.col_ind, max_batch=2, max_iter=25,
                           normalization=0.75, schedule=fec.COLORED_LAYERED)
    bits, ok, _ = dec.decode(llr)
    full = fec.CsrBpDecoder(code.n, code.m, code.row_ptr, code.col_ind, max_batch=5, max_iter=25,
                            normalization=0.75, schedule=fec.COLORED_LAYERED)
    bits2, ok2, _, _ = _run(cuda, full, llr, code.n)
    assert np.array_equal(bits, bits2) and np.array_equal(ok, ok2)
    info, _, _ = channel.awgn_llrs(code, 5, 2.5, 80)
    assert ok.all() and np.array_equal(bits[:, : code.k], info)
