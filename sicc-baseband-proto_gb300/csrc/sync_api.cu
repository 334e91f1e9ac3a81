// cuda_osd_find_frame: the decoder library's host-IQ frame search, on the sync kernel.
#include "../../include/sicc_fec.h"
#include "ofdm_kernels.h"

#include <vector>

namespace sicc {
namespace {

template <class F>
int guarded_sync(F&& f)
{
    try {
        return f();
    } catch (const InvalidArgument& e) {
        set_last_error(e.what());
        return CUDA_OSD_STATUS_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return CUDA_OSD_STATUS_INTERNAL_ERROR;
    }
}

struct DevMem {
    void* p = nullptr;
    explicit DevMem(size_t bytes) { check_cuda(cudaMalloc(&p, bytes), "cudaMalloc(find_frame)"); }
    ~DevMem() { cudaFree(p); }
};

}  // namespace
}  // namespace sicc

using namespace sicc;

extern "C" int cuda_osd_find_frame(const double* signal_real, const double* signal_imag, int signal_length,
                                   const double* preamble_real, const double* preamble_imag, int preamble_length,
                                   int pre_half_len, double sync_peak_thresh, double fs, int* out_start_idx_1based,
                                   double* out_peak, double* out_cfo_hz)
{
    return guarded_sync([&] {
        if (!signal_real || !signal_imag || !preamble_real || !preamble_imag || !out_start_idx_1based)
            throw InvalidArgument("null argument");
        if (pre_half_len <= 0 || preamble_length != 2 * pre_half_len)
            throw InvalidArgument("preamble_length must equal 2 * pre_half_len");
        if (signal_length < preamble_length) throw InvalidArgument("signal shorter than the preamble");
        std::vector<float2> sig(static_cast<size_t>(signal_length)), pre(static_cast<size_t>(preamble_length));
        float pre_energy = 0.0f;
        for (int i = 0; i < signal_length; ++i)
            sig[i] = make_float2(static_cast<float>(signal_real[i]), static_cast<float>(signal_imag[i]));
        for (int i = 0; i < preamble_length; ++i) {
            pre[i] = make_float2(static_cast<float>(preamble_real[i]), static_cast<float>(preamble_imag[i]));
            pre_energy += pre[i].x * pre[i].x + pre[i].y * pre[i].y;
        }
        DevMem d_sig(sig.size() * sizeof(float2)), d_pre(pre.size() * sizeof(float2)), d_out(sizeof(SyncOut));
        check_cuda(cudaMemcpy(d_sig.p, sig.data(), sig.size() * sizeof(float2), cudaMemcpyHostToDevice), "copy signal");
        check_cuda(cudaMemcpy(d_pre.p, pre.data(), pre.size() * sizeof(float2), cudaMemcpyHostToDevice), "copy preamble");
        SyncParams p{};
        p.half_len = pre_half_len;
        p.pre_len = preamble_length;
        p.radius = 16;
        p.threshold = static_cast<float>(sync_peak_thresh);
        p.sample_rate = static_cast<float>(fs);
        p.mode = 1;
        p.max_search = 0;
        p.frame_len = 0;
        p.pre_energy = pre_energy;
        launch_sync(static_cast<const float2*>(d_sig.p), 0, nullptr, signal_length, 1,
                    static_cast<const float2*>(d_pre.p), p, static_cast<SyncOut*>(d_out.p), nullptr);
        SyncOut r{};
        check_cuda(cudaMemcpy(&r, d_out.p, sizeof(SyncOut), cudaMemcpyDeviceToHost), "copy sync result");
        *out_start_idx_1based = (r.found == 1) ? r.start + 1 : 0;
        if (out_peak) *out_peak = r.fine;
        if (out_cfo_hz) *out_cfo_hz = (r.found == 1) ? r.cfo_hz : 0.0;
        return CUDA_OSD_STATUS_OK;
    });
}
