// usrp_gpu_pipeline_bridge::Pipeline (include/gpu_ofdm_pipeline.hpp) over the
// C ABI of include/sicc_pipe.h: each member maps to one sicc_pipe_* call and
// turns a non-zero status into std::runtime_error with the library's message.
#include "../../include/gpu_ofdm_pipeline.hpp"
#include "../../include/sicc_pipe.h"

#include <stdexcept>
#include <string>

namespace usrp_gpu_pipeline_bridge {

namespace {

void check(int status, const char* what)
{
    if (status != CUDA_OSD_STATUS_OK) throw std::runtime_error(std::string(what) + ": " + cuda_osd_get_last_error());
}

SyncResult from_c(const sicc_pipe_sync_t& s)
{
    SyncResult r;
    r.start = s.start;
    r.metric = s.metric;
    r.cfo_hz = s.cfo_hz;
    return r;
}

void require_size(size_t actual, size_t expected, const char* name)
{
    if (actual != expected)
        throw std::runtime_error(std::string(name) + " has wrong size; expected " + std::to_string(expected) +
                                 ", got " + std::to_string(actual));
}

}  // namespace

struct Pipeline::Impl {
    Config cfg;
    unsigned long long handle = 0;
};

Pipeline::Pipeline(const Config& cfg, int slots) : impl_(new Impl)
{
    impl_->cfg = cfg;
    sicc_pipe_config_t c{};
    c.nfft = cfg.nfft;
    c.cp = cfg.cp;
    c.preamble_len = cfg.preamble_len;
    c.pre_half_len = cfg.pre_half_len;
    c.num_symbols = cfg.num_symbols;
    c.active_sc = cfg.active_sc;
    c.bits_per_symbol = cfg.bits_per_symbol;
    c.code_n = cfg.code_n;
    c.code_k = cfg.code_k;
    c.blocks_per_frame = cfg.blocks_per_frame;
    c.max_rx_search_samples = cfg.max_rx_search_samples;
    c.sample_rate = cfg.sample_rate;
    c.sync_threshold = cfg.sync_threshold;
    c.tx_amplitude = cfg.tx_amplitude;
    c.demod_noise_var = cfg.demod_noise_var;
    c.use_pilot_channel_est = cfg.use_pilot_channel_est ? 1 : 0;
    check(sicc_pipe_create(&c, slots, &impl_->handle), "GpuOfdmPipeline");
}

Pipeline::~Pipeline()
{
    if (impl_ && impl_->handle) sicc_pipe_destroy(impl_->handle);
}

void Pipeline::upload_static_tables(const StaticTables& t)
{
    const Config& c = impl_->cfg;
    require_size(t.used_indices.size(), static_cast<size_t>(c.active_sc), "used_indices");
    require_size(t.preamble.size(), static_cast<size_t>(c.preamble_len), "preamble");
    require_size(t.interp_p0.size(), t.data_symbols.size(), "interp_p0");
    require_size(t.interp_p1.size(), t.data_symbols.size(), "interp_p1");
    require_size(t.interp_alpha.size(), t.data_symbols.size(), "interp_alpha");
    require_size(t.pilot_grid.size(), t.pilot_symbols.size() * static_cast<size_t>(c.active_sc), "pilot_grid");
    sicc_pipe_tables_t ct{};
    ct.used_indices = t.used_indices.data();
    ct.pilot_symbols = t.pilot_symbols.data();
    ct.pilot_count = static_cast<int>(t.pilot_symbols.size());
    ct.data_symbols = t.data_symbols.data();
    ct.data_count = static_cast<int>(t.data_symbols.size());
    ct.interp_p0 = t.interp_p0.data();
    ct.interp_p1 = t.interp_p1.data();
    ct.interp_alpha = t.interp_alpha.data();
    ct.pilot_grid = reinterpret_cast<const float*>(t.pilot_grid.data());
    ct.preamble = reinterpret_cast<const float*>(t.preamble.data());
    check(sicc_pipe_upload_static_tables(impl_->handle, &ct), "upload_static_tables");
    // transmit-side members (gpu_ofdm_pipeline.cu:854-920)
    if (!t.generator_kn.empty() || t.dvb_s2_accumulator) {
        const size_t re = static_cast<size_t>(c.num_symbols) * c.active_sc;
        if (!t.generator_kn.empty())
            require_size(t.generator_kn.size(), static_cast<size_t>(c.code_k) * c.code_n, "generator_kn");
        if (t.dvb_s2_accumulator)
            require_size(t.row_info_offsets.size(), static_cast<size_t>(c.code_n - c.code_k) + 1, "row_info_offsets");
        if (!t.precomp_h.empty()) require_size(t.precomp_h.size(), re, "precomp_h");
        if (!t.actual_h.empty()) require_size(t.actual_h.size(), re, "actual_h");
        sicc_pipe_tx_tables_t tx{};
        tx.generator_kn = t.generator_kn.empty() ? nullptr : t.generator_kn.data();
        tx.dvb_s2_accumulator = t.dvb_s2_accumulator ? 1 : 0;
        tx.row_info_offsets = t.row_info_offsets.empty() ? nullptr : t.row_info_offsets.data();
        tx.row_info_cols = t.row_info_cols.empty() ? nullptr : t.row_info_cols.data();
        tx.precomp_h = t.precomp_h.empty() ? nullptr : reinterpret_cast<const float*>(t.precomp_h.data());
        tx.actual_h = t.actual_h.empty() ? nullptr : reinterpret_cast<const float*>(t.actual_h.data());
        check(sicc_pipe_upload_tx_tables(impl_->handle, &tx), "upload_static_tables");
    }
}

void Pipeline::submit_tx_frame_async(int slot, const uint8_t* h_info_bits, Complex32* h_tx_frame)
{
    check(sicc_pipe_tx_frame(impl_->handle, slot, h_info_bits, reinterpret_cast<float*>(h_tx_frame)),
          "submit_tx_frame_async");
}

const Complex32* Pipeline::submit_tx_frame_device_async(int slot, const uint8_t* h_info_bits, float frequency_noise_var,
                                                        uint64_t noise_seed, bool add_frequency_noise)
{
    const float* d = nullptr;
    check(sicc_pipe_tx_frame_device(impl_->handle, slot, h_info_bits, frequency_noise_var, noise_seed,
                                    add_frequency_noise ? 1 : 0, &d),
          "submit_tx_frame_device_async");
    return reinterpret_cast<const Complex32*>(d);
}

void Pipeline::synchronize_tx(int slot)
{
    check(sicc_pipe_tx_synchronize(impl_->handle, slot), "synchronize_tx");
}

SyncResult Pipeline::find_frame(int slot, const Complex32* h_samples, int sample_count)
{
    sicc_pipe_sync_t s{};
    check(sicc_pipe_find_frame(impl_->handle, slot, reinterpret_cast<const float*>(h_samples), sample_count, &s),
          "find_frame");
    return from_c(s);
}

SyncResult Pipeline::find_frame_device(int slot, const Complex32* d_samples, int sample_count)
{
    sicc_pipe_sync_t s{};
    check(sicc_pipe_find_frame_device(impl_->handle, slot, reinterpret_cast<const float*>(d_samples), sample_count, &s),
          "find_frame_device");
    return from_c(s);
}

const float* Pipeline::demod_frame_to_device_llr(int slot, const Complex32* h_frame, SyncResult* sync_result)
{
    sicc_pipe_sync_t s{};
    const float* d = nullptr;
    check(sicc_pipe_demod_to_device(impl_->handle, slot, reinterpret_cast<const float*>(h_frame), &s, &d),
          "demod_frame_to_device_llr");
    if (sync_result) *sync_result = from_c(s);
    return d;
}

const float* Pipeline::demod_frame_device_to_device_llr(int slot, const Complex32* d_frame,
                                                        const SyncResult& sync_result)
{
    sicc_pipe_sync_t s{};
    s.start = 0;
    s.metric = sync_result.metric;
    s.cfo_hz = sync_result.cfo_hz;
    const float* d = nullptr;
    check(sicc_pipe_demod_device_to_device(impl_->handle, slot, reinterpret_cast<const float*>(d_frame), &s, &d),
          "demod_frame_device_to_device_llr");
    return d;
}

SyncResult Pipeline::demod_frame_to_host_llr(int slot, const Complex32* h_frame, float* h_llr)
{
    sicc_pipe_sync_t s{};
    check(sicc_pipe_demod_to_host(impl_->handle, slot, reinterpret_cast<const float*>(h_frame), h_llr, &s),
          "demod_frame_to_host_llr");
    return from_c(s);
}

}  // namespace usrp_gpu_pipeline_bridge
