// C ABI of the OFDM receive pipeline (include/sicc_pipe.h): per-slot device
// buffers and streams around the sync and demod kernels.  The slot model
// follows the reference bridge (gpu_ofdm_pipeline.cu:1077-1247, 1472-1668):
// a caller-managed ring of slots; every synchronous call waits for its slot's
// stream before returning; returned device LLRs stay valid until the slot is
// reused.
#include "../../include/sicc_ingest.h"
#include "../../include/sicc_pipe.h"
#include "ofdm_kernels.h"
#include "pipe_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

namespace sicc {
namespace {

static_assert(sizeof(sicc_pipe_sync_record_t) == sizeof(SyncOut), "sync record layout");

template <class T>
struct Buf {
    T* p = nullptr;
    void alloc(size_t n)
    {
        release();
        if (n) check_cuda(cudaMalloc(&p, n * sizeof(T)), "cudaMalloc(pipeline)");
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
    }
    ~Buf() { release(); }
};

template <class T>
void upload(Buf<T>& b, const T* src, size_t n)
{
    b.alloc(n);
    if (n) check_cuda(cudaMemcpy(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice), "upload pipeline table");
}

struct Slot {
    Buf<float2> samples;
    Buf<SyncOut> sync;
    Buf<float> llr;
    Buf<uint8_t> tx_info;  // TX: one frame's info bits
    Buf<float2> tx_frame;
    cudaStream_t stream = nullptr;
    cudaEvent_t tx_done = nullptr;
    ~Slot()
    {
        if (tx_done) cudaEventDestroy(tx_done);
        if (stream) cudaStreamDestroy(stream);
    }
};

struct Pipe {
    sicc_pipe_config_t cfg{};
    int device = 0;
    int frame_samples = 0;
    int coded_bits = 0;     // blocks_per_frame * code_n: LLRs kept per frame
    int capacity_bits = 0;  // data REs * bits per symbol
    int max_rx = 0;
    int batch_frames = 256;
    int symbols_per_cta = 0;  // data symbols per demod CTA; their pilots span at most 4
    std::vector<int> h_p0, h_p1;  // interpolation pilots of each data symbol (host copies)
    bool tables = false;
    float pre_energy = 0.0f;
    DemodView view{};
    Buf<int> used_bins, pilot_syms, data_syms, p0, p1;
    Buf<float> alpha, axis;
    Buf<float2> pilot_grid, preamble, twiddle;
    std::vector<std::unique_ptr<Slot>> slots;
    Buf<SyncOut> batch_sync;
    // transmitter
    bool tx_tables = false;
    TxView txv{};
    Buf<int> pilot_of_sym, data_of_sym;
    Buf<uint32_t> gen, gen_tab;
    Buf<int> acc_off, acc_cols;
    Buf<float2> precomp, actual;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    bool batch_timed = false;
    std::mutex mu;
    ~Pipe()
    {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }

    SyncParams sync_params(int mode) const
    {
        SyncParams p{};
        p.half_len = cfg.pre_half_len;
        p.pre_len = cfg.preamble_len;
        p.radius = cfg.sync_radius > 0 ? cfg.sync_radius : std::min(16, cfg.cp);
        p.threshold = cfg.sync_threshold;
        p.sample_rate = cfg.sample_rate;
        p.mode = mode;
        p.max_search = 0;
        p.frame_len = frame_samples;
        p.pre_energy = pre_energy;
        return p;
    }
};

std::mutex g_mu;
std::map<unsigned long long, std::shared_ptr<Pipe>> g_pipes;
unsigned long long g_next = 0x7100;

std::shared_ptr<Pipe> get(unsigned long long h)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_pipes.find(h);
    if (it == g_pipes.end()) throw InvalidArgument("invalid pipeline handle");
    return it->second;
}

Slot& slot_of(Pipe& p, int slot)
{
    if (slot < 0 || slot >= static_cast<int>(p.slots.size())) throw InvalidArgument("invalid GPU pipeline slot");
    return *p.slots[slot];
}

template <class F>
int guarded(F&& f)
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

void require_tables(const Pipe& p)
{
    if (!p.tables) throw InvalidArgument("upload_static_tables must run before receiving");
}

void require_tx(const Pipe& p)
{
    if (!p.tables) throw InvalidArgument("upload_static_tables must run before transmitting");
    if (!p.tx_tables) throw InvalidArgument("GPU TX requested before uploading a generator matrix");
}

// One frame of device info bits -> a device frame, on the slot's stream.
void tx_one(Pipe& p, Slot& s, float noise_var, unsigned long long seed)
{
    launch_tx(p.txv, s.tx_info.p, 1, s.tx_frame.p, noise_var, seed, s.stream);
}

sicc_pipe_sync_t to_public(const SyncOut& s)
{
    sicc_pipe_sync_t r{};
    r.start = (s.found == 1) ? s.start : -1;
    r.metric = s.fine;
    r.cfo_hz = (s.found == 1) ? s.cfo_hz : 0.0f;
    return r;
}

// Search `count` samples already in device memory (slot stream); returns the result.
// The most pilot symbols one demodulator CTA needs when it takes `spc` data symbols
// (0 without pilot channel estimation).
int pilot_span(const Pipe& p, int spc)
{
    if (!p.cfg.use_pilot_channel_est) return 0;
    const int nd = static_cast<int>(p.h_p0.size());
    int worst = 0;
    for (int d0 = 0; d0 < nd; d0 += std::max(spc, 1)) {
        int lo = 1 << 30, hi = -1;
        for (int d = d0; d < std::min(nd, d0 + spc); ++d) {
            lo = std::min(lo, std::min(p.h_p0[d], p.h_p1[d]));
            hi = std::max(hi, std::max(p.h_p0[d], p.h_p1[d]));
        }
        worst = std::max(worst, hi - lo + 1);
    }
    return worst;
}

SyncOut run_sync(Pipe& p, Slot& s, const float2* d_iq, int count)
{
    if (count < p.cfg.preamble_len) throw InvalidArgument("RX sample_count is shorter than the preamble");
    const SyncParams sp = p.sync_params(0);
    launch_sync(d_iq, 0, nullptr, count, 1, p.preamble.p, sp, s.sync.p, s.stream);
    SyncOut out{};
    check_cuda(cudaMemcpyAsync(&out, s.sync.p, sizeof(SyncOut), cudaMemcpyDeviceToHost, s.stream), "copy sync result");
    check_cuda(cudaStreamSynchronize(s.stream), "synchronize sync");
    return out;
}

}  // namespace
}  // namespace sicc

using namespace sicc;

extern "C" {

int sicc_pipe_create(const sicc_pipe_config_t* config, int slots, unsigned long long* out_handle)
{
    return guarded([&] {
        if (!config || !out_handle) throw InvalidArgument("null argument");
        *out_handle = 0;
        const sicc_pipe_config_t& c = *config;
        if (c.blocks_per_frame <= 0) throw InvalidArgument("blocks_per_frame must be set before constructing the pipeline");
        if (c.nfft < 4 || (c.nfft & (c.nfft - 1))) throw InvalidArgument("nfft must be a power of two");
        if (c.cp < 0 || c.cp >= c.nfft) throw InvalidArgument("cp must be in [0, nfft)");
        if (c.active_sc <= 0 || c.active_sc >= c.nfft) throw InvalidArgument("active_sc must be in (0, nfft)");
        if (c.preamble_len != 2 * c.pre_half_len || c.pre_half_len <= 0)
            throw InvalidArgument("preamble_len must equal 2 * pre_half_len");
        if (c.bits_per_symbol != 1 && c.bits_per_symbol != 2 && c.bits_per_symbol != 4 && c.bits_per_symbol != 6)
            throw InvalidArgument("bits_per_symbol must be 1, 2, 4, or 6");
        auto p = std::make_shared<Pipe>();
        p->cfg = c;
        check_cuda(cudaGetDevice(&p->device), "cudaGetDevice");
        p->frame_samples = c.preamble_len + c.num_symbols * (c.nfft + c.cp);
        p->coded_bits = c.blocks_per_frame * c.code_n;
        p->max_rx = c.max_rx_search_samples > 0 ? c.max_rx_search_samples : p->frame_samples;
        p->batch_frames = c.max_batch_frames > 0 ? c.max_batch_frames : 256;
        const int n_slots = std::max(slots, 1);
        for (int i = 0; i < n_slots; ++i) {
            auto s = std::make_unique<Slot>();
            check_cuda(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate(slot)");
            // twice the longest buffer, zero-filled: a frame found near the end of a one-frame
            // buffer ("incomplete") is demodulated from defined memory (zeros past the samples)
            const size_t cap = 2 * static_cast<size_t>(std::max(p->max_rx, p->frame_samples));
            s->samples.alloc(cap);
            check_cuda(cudaMemset(s->samples.p, 0, cap * sizeof(float2)), "zero slot samples");
            s->sync.alloc(1);
            s->llr.alloc(static_cast<size_t>(p->coded_bits));
            p->slots.push_back(std::move(s));
        }
        p->batch_sync.alloc(static_cast<size_t>(p->batch_frames));
        for (auto& e : p->ev) check_cuda(cudaEventCreate(&e), "cudaEventCreate(pipeline)");
        std::lock_guard<std::mutex> lock(g_mu);
        *out_handle = ++g_next;
        g_pipes[*out_handle] = p;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_destroy(unsigned long long handle)
{
    return guarded([&] {
        std::shared_ptr<Pipe> p;
        {
            std::lock_guard<std::mutex> lock(g_mu);
            auto it = g_pipes.find(handle);
            if (it == g_pipes.end()) throw InvalidArgument("invalid pipeline handle");
            p = it->second;
            g_pipes.erase(it);
        }
        cudaSetDevice(p->device);
        for (auto& s : p->slots) cudaStreamSynchronize(s->stream);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_upload_static_tables(unsigned long long handle, const sicc_pipe_tables_t* t)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        if (!t || !t->used_indices || !t->data_symbols || !t->interp_p0 || !t->interp_p1 || !t->interp_alpha ||
            !t->preamble)
            throw InvalidArgument("null table");
        const auto& c = p->cfg;
        if (t->data_count <= 0 || t->data_count > c.num_symbols) throw InvalidArgument("data_symbols has wrong size");
        p->capacity_bits = t->data_count * c.active_sc * c.bits_per_symbol;
        if (p->coded_bits > p->capacity_bits)
            throw InvalidArgument("coded bits per frame exceed the data resource elements");
        if (p->coded_bits % c.bits_per_symbol)
            throw InvalidArgument("coded bits per frame must be a multiple of bits_per_symbol");
        if (c.use_pilot_channel_est && (t->pilot_count <= 0 || !t->pilot_symbols || !t->pilot_grid))
            throw InvalidArgument("pilot tables are required for pilot channel estimation");
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        std::vector<int> bins(c.active_sc);
        for (int sc = 0; sc < c.active_sc; ++sc) {
            const int u = t->used_indices[sc];
            if (u < 0 || u >= c.nfft) throw InvalidArgument("used_indices out of range");
            bins[sc] = (u + c.nfft / 2) % c.nfft;  // shifted grid -> natural bin (gpu_ofdm_pipeline.cu:124-127)
        }
        for (int d = 0; d < t->data_count; ++d) {
            if (t->data_symbols[d] < 0 || t->data_symbols[d] >= c.num_symbols) throw InvalidArgument("data symbol index");
            if (c.use_pilot_channel_est &&
                (t->interp_p0[d] < 0 || t->interp_p0[d] >= t->pilot_count || t->interp_p1[d] < 0 ||
                 t->interp_p1[d] >= t->pilot_count || std::abs(t->interp_p1[d] - t->interp_p0[d]) > 3))
                throw InvalidArgument("interpolation pilot indices out of range");
        }
        // data symbols per CTA: about three (measured on the 16-QAM workload: 3 per CTA 54.7 us, 2
        // 57.4, 4 59.0, 13 83.4 per 256 frames), fewer when their interpolation pilots would span
        // more than four
        p->h_p0.assign(t->interp_p0, t->interp_p0 + t->data_count);
        p->h_p1.assign(t->interp_p1, t->interp_p1 + t->data_count);
        {
            const int groups = (t->data_count + 2) / 3;
            int spc = (t->data_count + groups - 1) / groups;
            while (spc > 1 && pilot_span(*p, spc) > kDemodMaxPilots) --spc;
            p->symbols_per_cta = spc;
        }
        upload(p->used_bins, bins.data(), bins.size());
        upload(p->data_syms, t->data_symbols, t->data_count);
        upload(p->p0, t->interp_p0, t->data_count);
        upload(p->p1, t->interp_p1, t->data_count);
        upload(p->alpha, t->interp_alpha, t->data_count);
        if (t->pilot_count > 0) {
            for (int q = 0; q < t->pilot_count; ++q)
                if (t->pilot_symbols[q] < 0 || t->pilot_symbols[q] >= c.num_symbols) throw InvalidArgument("pilot symbol index");
            upload(p->pilot_syms, t->pilot_symbols, t->pilot_count);
            upload(p->pilot_grid, reinterpret_cast<const float2*>(t->pilot_grid),
                   static_cast<size_t>(t->pilot_count) * c.active_sc);
        }
        upload(p->preamble, reinterpret_cast<const float2*>(t->preamble), c.preamble_len);
        float e = 0.0f;
        for (int i = 0; i < c.preamble_len; ++i)
            e += t->preamble[2 * i] * t->preamble[2 * i] + t->preamble[2 * i + 1] * t->preamble[2 * i + 1];
        p->pre_energy = e;
        // twiddles exp(-2 pi i j / N), computed in double
        std::vector<float2> tw(c.nfft);
        for (int j = 0; j < c.nfft; ++j) {
            const double a = -2.0 * 3.141592653589793238462643383279502884 * j / c.nfft;
            tw[j] = make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a)));
        }
        upload(p->twiddle, tw.data(), tw.size());
        // axis amplitudes of Gray square QAM, scaled to unit average power as the
        // reference constellation (uhd_ldpc_ofdm_link.cpp:2362-2414)
        std::vector<float> lv;
        const int bps = c.bits_per_symbol;
        if (bps == 1) {
            lv = {1.0f, -1.0f};
        } else if (bps == 2) {
            const float s = static_cast<float>(1.0 / std::sqrt(2.0));
            lv = {s, -s};
        } else {
            const int ab = bps / 2, levels = 1 << ab;
            double avg = 0.0;
            auto g2b = [](int g) {
                int b = 0;
                for (; g; g >>= 1) b ^= g;
                return b;
            };
            for (int i = 0; i < levels; ++i)
                for (int q = 0; q < levels; ++q) {
                    const double a = (levels - 1) - 2 * g2b(i), b = (levels - 1) - 2 * g2b(q);
                    avg += a * a + b * b;
                }
            const float scale = static_cast<float>(1.0 / std::sqrt(avg / (levels * levels)));
            for (int g = 0; g < levels; ++g) lv.push_back(static_cast<float>((levels - 1) - 2 * g2b(g)) * scale);
        }
        upload(p->axis, lv.data(), lv.size());
        DemodView& v = p->view;
        v.nfft = c.nfft;
        v.cp = c.cp;
        v.num_symbols = c.num_symbols;
        v.active_sc = c.active_sc;
        v.bits_per_symbol = c.bits_per_symbol;
        v.pre_len = c.preamble_len;
        v.num_pilots = t->pilot_count;
        v.num_data = t->data_count;
        v.sample_rate = c.sample_rate;
        v.noise_var = c.demod_noise_var;
        v.use_pilot_est = c.use_pilot_channel_est ? 1 : 0;
        v.kept_bits = p->coded_bits;
        v.used_bins = p->used_bins.p;
        v.pilot_symbols = p->pilot_syms.p;
        v.data_symbols = p->data_syms.p;
        v.interp_p0 = p->p0.p;
        v.interp_p1 = p->p1.p;
        v.interp_alpha = p->alpha.p;
        v.pilot_grid = p->pilot_grid.p;
        v.twiddle = p->twiddle.p;
        v.axis_levels = p->axis.p;
        v.max_pilots_per_cta = pilot_span(*p, p->symbols_per_cta);
        // per-symbol pilot / data indices for the transmitter's resource grid
        std::vector<int> pos(c.num_symbols, -1), dos(c.num_symbols, -1);
        for (int q = 0; q < t->pilot_count; ++q) pos[t->pilot_symbols[q]] = q;
        for (int d = 0; d < t->data_count; ++d) dos[t->data_symbols[d]] = d;
        upload(p->pilot_of_sym, pos.data(), pos.size());
        upload(p->data_of_sym, dos.data(), dos.size());
        TxView& x = p->txv;
        x.nfft = c.nfft;
        x.cp = c.cp;
        x.num_symbols = c.num_symbols;
        x.active_sc = c.active_sc;
        x.bits_per_symbol = c.bits_per_symbol;
        x.pre_len = c.preamble_len;
        x.code_n = c.code_n;
        x.code_k = c.code_k;
        x.blocks = c.blocks_per_frame;
        x.frame_samples = p->frame_samples;
        x.amplitude = c.tx_amplitude;
        x.used_bins = p->used_bins.p;
        x.pilot_of_symbol = p->pilot_of_sym.p;
        x.data_of_symbol = p->data_of_sym.p;
        x.pilot_grid = p->pilot_grid.p;
        x.preamble = p->preamble.p;
        x.twiddle = p->twiddle.p;
        p->tables = true;
        return CUDA_OSD_STATUS_OK;
    });
}

static int find_frame_impl(unsigned long long handle, int slot, const float* iq, bool device, int count,
                           sicc_pipe_sync_t* out)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tables(*p);
        if (!iq || !out) throw InvalidArgument("null argument");
        Slot& s = slot_of(*p, slot);
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        if (count > p->max_rx) throw InvalidArgument("RX sample_count exceeds slot allocation");
        const float2* d = reinterpret_cast<const float2*>(iq);
        if (!device) {
            check_cuda(cudaMemcpyAsync(s.samples.p, iq, static_cast<size_t>(count) * sizeof(float2),
                                       cudaMemcpyHostToDevice, s.stream),
                       "copy RX samples");
            d = s.samples.p;
        }
        *out = to_public(run_sync(*p, s, d, count));
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_find_frame(unsigned long long handle, int slot, const float* host_iq, int sample_count,
                         sicc_pipe_sync_t* out_sync)
{
    return find_frame_impl(handle, slot, host_iq, false, sample_count, out_sync);
}

int sicc_pipe_find_frame_device(unsigned long long handle, int slot, const float* device_iq, int sample_count,
                                sicc_pipe_sync_t* out_sync)
{
    return find_frame_impl(handle, slot, device_iq, true, sample_count, out_sync);
}

int sicc_pipe_demod_to_device(unsigned long long handle, int slot, const float* host_frame, sicc_pipe_sync_t* out_sync,
                              const float** out_device_llr)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tables(*p);
        if (!host_frame || !out_device_llr) throw InvalidArgument("null argument");
        Slot& s = slot_of(*p, slot);
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        const int count = p->frame_samples;
        check_cuda(cudaMemcpyAsync(s.samples.p, host_frame, static_cast<size_t>(count) * sizeof(float2),
                                   cudaMemcpyHostToDevice, s.stream),
                   "copy RX frame");
        const SyncOut so = run_sync(*p, s, s.samples.p, count);
        // frames that run past the buffer are demodulated as found (the buffer is one frame long)
        SyncOut use = so;
        if (so.found == 2) {
            use.found = 1;
            check_cuda(cudaMemcpyAsync(s.sync.p, &use, sizeof(SyncOut), cudaMemcpyHostToDevice, s.stream), "sync");
        }
        launch_demod(p->view, s.samples.p, 0, s.sync.p, 1, s.llr.p, p->coded_bits, s.stream, p->symbols_per_cta);
        check_cuda(cudaStreamSynchronize(s.stream), "synchronize RX demod device LLR");
        if (out_sync) *out_sync = to_public(so);
        *out_device_llr = s.llr.p;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_demod_device_to_device(unsigned long long handle, int slot, const float* device_frame,
                                     const sicc_pipe_sync_t* sync, const float** out_device_llr)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tables(*p);
        if (!device_frame || !sync || !out_device_llr) throw InvalidArgument("null argument");
        Slot& s = slot_of(*p, slot);
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        SyncOut so{};
        so.found = 1;
        so.start = 0;  // the device frame starts at its first sample (gpu_ofdm_pipeline.cu:1230-1236)
        so.fine = sync->metric;
        so.cfo_hz = sync->cfo_hz;
        check_cuda(cudaMemcpyAsync(s.sync.p, &so, sizeof(SyncOut), cudaMemcpyHostToDevice, s.stream), "copy sync");
        launch_demod(p->view, reinterpret_cast<const float2*>(device_frame), 0, s.sync.p, 1, s.llr.p, p->coded_bits,
                     s.stream, p->symbols_per_cta);
        check_cuda(cudaStreamSynchronize(s.stream), "synchronize RX device-frame demod LLR");
        *out_device_llr = s.llr.p;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_demod_to_host(unsigned long long handle, int slot, const float* host_frame, float* host_llr,
                            sicc_pipe_sync_t* out_sync)
{
    const float* d_llr = nullptr;
    sicc_pipe_sync_t so{};
    int st = sicc_pipe_demod_to_device(handle, slot, host_frame, &so, &d_llr);
    if (st != CUDA_OSD_STATUS_OK) return st;
    return guarded([&] {
        auto p = get(handle);
        if (!host_llr) throw InvalidArgument("null host_llr");
        Slot& s = slot_of(*p, slot);
        check_cuda(cudaMemcpyAsync(host_llr, d_llr, static_cast<size_t>(p->coded_bits) * sizeof(float),
                                   cudaMemcpyDeviceToHost, s.stream),
                   "copy RX LLRs to host");
        check_cuda(cudaStreamSynchronize(s.stream), "synchronize RX demod LLR copy");
        if (out_sync) *out_sync = so;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_demod_batch(unsigned long long handle, const float* device_iq, long long stride, int sample_count,
                          int frames, float* device_llr, sicc_pipe_sync_record_t* device_sync, void* cuda_stream)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tables(*p);
        if (!device_iq || !device_llr) throw InvalidArgument("null device pointer");
        if (frames <= 0 || frames > p->batch_frames) throw InvalidArgument("frames must be in 1..max_batch_frames");
        if (sample_count < p->cfg.preamble_len || stride < sample_count)
            throw InvalidArgument("sample_count must cover the preamble and fit the stride");
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
        SyncOut* so = device_sync ? reinterpret_cast<SyncOut*>(device_sync) : p->batch_sync.p;
        check_cuda(cudaEventRecord(p->ev[0], st), "cudaEventRecord");
        launch_sync(reinterpret_cast<const float2*>(device_iq), stride, nullptr, sample_count, frames, p->preamble.p,
                    p->sync_params(0), so, st);
        check_cuda(cudaEventRecord(p->ev[1], st), "cudaEventRecord");
        launch_demod(p->view, reinterpret_cast<const float2*>(device_iq), stride, so, frames, device_llr, p->coded_bits,
                     st, p->symbols_per_cta);
        check_cuda(cudaEventRecord(p->ev[2], st), "cudaEventRecord");
        p->batch_timed = true;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_demod_gather(unsigned long long handle, const float* device_iq, const long long* device_frame_offsets,
                           int sample_count, int frames, float* device_llr, const long long* device_llr_offsets,
                           sicc_pipe_sync_record_t* device_sync, void* cuda_stream)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tables(*p);
        if (!device_iq || !device_frame_offsets || !device_llr || !device_llr_offsets || !device_sync)
            throw InvalidArgument("null device pointer");
        if (frames <= 0 || frames > p->batch_frames) throw InvalidArgument("frames must be in 1..max_batch_frames");
        if (sample_count < p->cfg.preamble_len) throw InvalidArgument("sample_count must cover the preamble");
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
        SyncOut* so = reinterpret_cast<SyncOut*>(device_sync);
        const float2* iq = reinterpret_cast<const float2*>(device_iq);
        check_cuda(cudaEventRecord(p->ev[0], st), "cudaEventRecord");
        launch_sync(iq, sample_count, nullptr, sample_count, frames, p->preamble.p, p->sync_params(0), so, st,
                    device_frame_offsets);
        check_cuda(cudaEventRecord(p->ev[1], st), "cudaEventRecord");
        launch_demod(p->view, iq, 0, so, frames, device_llr, 0, st, p->symbols_per_cta, device_frame_offsets,
                     device_llr_offsets);
        check_cuda(cudaEventRecord(p->ev[2], st), "cudaEventRecord");
        p->batch_timed = true;
        return CUDA_OSD_STATUS_OK;
    });
}

}  // extern "C"

namespace sicc {

int pipe_dims(unsigned long long handle, PipeDims* out)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tables(*p);
        if (!out) throw InvalidArgument("null argument");
        out->frame_samples = p->frame_samples;
        out->coded_bits = p->coded_bits;
        out->code_n = p->cfg.code_n;
        out->code_k = p->cfg.code_k;
        out->blocks = p->cfg.blocks_per_frame;
        out->preamble_len = p->cfg.preamble_len;
        out->max_frames = p->batch_frames;
        return CUDA_OSD_STATUS_OK;
    });
}

int pipe_gather_scratch(unsigned long long handle, int sample_count, int frames, size_t* out_bytes,
                        size_t* out_ticket_offset, size_t* out_ticket_bytes)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tables(*p);
        const SyncScratchLayout l = sync_scratch_layout(sample_count, nullptr, sample_count, frames, p->sync_params(0));
        if (out_bytes) *out_bytes = l.bytes;
        if (out_ticket_offset) *out_ticket_offset = l.ticket_offset;
        if (out_ticket_bytes) *out_ticket_bytes = l.ticket_bytes;
        return CUDA_OSD_STATUS_OK;
    });
}

int pipe_gather_counted(unsigned long long handle, const float* device_iq, const long long* device_frame_offsets,
                        int sample_count, int max_frames, const int* frames_ptr, float* device_llr,
                        const long long* device_llr_offsets, void* device_sync, void* scratch, size_t scratch_bytes,
                        cudaStream_t st)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tables(*p);
        if (!device_iq || !device_frame_offsets || !device_llr || !device_llr_offsets || !device_sync || !frames_ptr ||
            !scratch)
            throw InvalidArgument("null device pointer");
        if (max_frames <= 0) throw InvalidArgument("max_frames must be positive");
        if (sample_count < p->cfg.preamble_len) throw InvalidArgument("sample_count must cover the preamble");
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        SyncOut* so = static_cast<SyncOut*>(device_sync);
        const float2* iq = reinterpret_cast<const float2*>(device_iq);
        launch_sync(iq, sample_count, nullptr, sample_count, max_frames, p->preamble.p, p->sync_params(0), so, st,
                    device_frame_offsets, frames_ptr, scratch, scratch_bytes);
        launch_demod(p->view, iq, 0, so, max_frames, device_llr, 0, st, p->symbols_per_cta, device_frame_offsets,
                     device_llr_offsets, frames_ptr);
        return CUDA_OSD_STATUS_OK;
    });
}

}  // namespace sicc

extern "C" {

int sicc_pipe_upload_tx_tables(unsigned long long handle, const sicc_pipe_tx_tables_t* t)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        if (!t) throw InvalidArgument("null table");
        const auto& c = p->cfg;
        const int n = c.code_n, k = c.code_k, m = n - k;
        if (k <= 0 || m <= 0) throw InvalidArgument("code dimensions must satisfy 0 < code_k < code_n");
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        TxView& x = p->txv;
        if (t->dvb_s2_accumulator) {
            if (!t->row_info_offsets) throw InvalidArgument("row_info_offsets has wrong size");
            const int nnz = t->row_info_offsets[m];
            if (t->row_info_offsets[0] != 0 || nnz < 0 || (nnz > 0 && !t->row_info_cols))
                throw InvalidArgument("row_info_offsets has wrong size");
            for (int r = 0; r < m; ++r)
                if (t->row_info_offsets[r + 1] < t->row_info_offsets[r]) throw InvalidArgument("row_info_offsets must not decrease");
            for (int q = 0; q < nnz; ++q)
                if (t->row_info_cols[q] < 0 || t->row_info_cols[q] >= k) throw InvalidArgument("row_info_cols out of range");
            upload(p->acc_off, t->row_info_offsets, static_cast<size_t>(m) + 1);
            if (nnz > 0) upload(p->acc_cols, t->row_info_cols, static_cast<size_t>(nnz));
            else p->acc_cols.alloc(1);
            p->gen.release();
            p->gen_tab.release();
            x.gen_tab = nullptr;
            x.acc_offsets = p->acc_off.p;
            x.acc_cols = p->acc_cols.p;
            x.gen_words = nullptr;
            x.gen_stride = 0;
        } else {
            if (!t->generator_kn) throw InvalidArgument("GPU TX requested before uploading a generator matrix");
            const int gw = (n + 31) / 32;
            std::vector<uint32_t> words(static_cast<size_t>(k) * gw, 0u);  // bit-packed rows
            for (int r = 0; r < k; ++r)
                for (int j = 0; j < n; ++j)
                    if (t->generator_kn[static_cast<size_t>(r) * n + j] & 1u) words[static_cast<size_t>(r) * gw + j / 32] |= 1u << (j % 32);
            upload(p->gen, words.data(), words.size());
            // byte tables: entry (g, e) = XOR of rows 8g + b for the set bits b of e (when they fit in 256 MB)
            const int groups = (k + 7) / 8;
            const size_t tab_words = static_cast<size_t>(groups) * 256 * gw;
            if (tab_words * 4 <= (static_cast<size_t>(256) << 20)) {
                std::vector<uint32_t> tab(tab_words, 0u);
                for (int g = 0; g < groups; ++g)
                    for (int e = 1; e < 256; ++e) {
                        const int b = __builtin_ctz(static_cast<unsigned>(e));
                        uint32_t* dst = &tab[(static_cast<size_t>(g) * 256 + e) * gw];
                        const uint32_t* prev = &tab[(static_cast<size_t>(g) * 256 + (e & (e - 1))) * gw];
                        const int row = 8 * g + b;
                        for (int w = 0; w < gw; ++w)
                            dst[w] = prev[w] ^ (row < k ? words[static_cast<size_t>(row) * gw + w] : 0u);
                    }
                upload(p->gen_tab, tab.data(), tab.size());
            } else {
                p->gen_tab.release();
            }
            p->acc_off.release();
            p->acc_cols.release();
            x.gen_words = p->gen.p;
            x.gen_tab = p->gen_tab.p;
            x.gen_stride = gw;
            x.acc_offsets = nullptr;
            x.acc_cols = nullptr;
        }
        const size_t re = static_cast<size_t>(c.num_symbols) * c.active_sc;
        if (t->precomp_h) upload(p->precomp, reinterpret_cast<const float2*>(t->precomp_h), re);
        else p->precomp.release();
        if (t->actual_h) upload(p->actual, reinterpret_cast<const float2*>(t->actual_h), re);
        else p->actual.release();
        x.precomp_h = p->precomp.p;
        x.actual_h = p->actual.p;
        const size_t info_bits = static_cast<size_t>(c.blocks_per_frame) * k;
        for (auto& sl : p->slots) {
            if (!sl->tx_info.p) {
                sl->tx_info.alloc(info_bits);
                sl->tx_frame.alloc(static_cast<size_t>(p->frame_samples));
                check_cuda(cudaEventCreateWithFlags(&sl->tx_done, cudaEventDisableTiming), "cudaEventCreate(tx)");
            }
        }
        p->tx_tables = true;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_tx_frame_device(unsigned long long handle, int slot, const unsigned char* host_info_bits,
                              float frequency_noise_var, unsigned long long noise_seed, int add_frequency_noise,
                              const float** out_device_frame)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tx(*p);
        if (!host_info_bits || !out_device_frame) throw InvalidArgument("null argument");
        Slot& s = slot_of(*p, slot);
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        const size_t info_bits = static_cast<size_t>(p->cfg.blocks_per_frame) * p->cfg.code_k;
        check_cuda(cudaMemcpyAsync(s.tx_info.p, host_info_bits, info_bits, cudaMemcpyHostToDevice, s.stream),
                   "copy TX info bits");
        tx_one(*p, s, add_frequency_noise ? frequency_noise_var : 0.0f, noise_seed);
        check_cuda(cudaEventRecord(s.tx_done, s.stream), "record tx_done");
        *out_device_frame = reinterpret_cast<const float*>(s.tx_frame.p);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_tx_frame(unsigned long long handle, int slot, const unsigned char* host_info_bits, float* host_frame)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tx(*p);
        if (!host_info_bits || !host_frame) throw InvalidArgument("null argument");
        Slot& s = slot_of(*p, slot);
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        const size_t info_bits = static_cast<size_t>(p->cfg.blocks_per_frame) * p->cfg.code_k;
        check_cuda(cudaMemcpyAsync(s.tx_info.p, host_info_bits, info_bits, cudaMemcpyHostToDevice, s.stream),
                   "copy TX info bits");
        tx_one(*p, s, 0.0f, 0ull);
        check_cuda(cudaMemcpyAsync(host_frame, s.tx_frame.p, static_cast<size_t>(p->frame_samples) * sizeof(float2),
                                   cudaMemcpyDeviceToHost, s.stream),
                   "copy TX frame to host");
        check_cuda(cudaEventRecord(s.tx_done, s.stream), "record tx_done");
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_tx_synchronize(unsigned long long handle, int slot)
{
    return guarded([&] {
        auto p = get(handle);
        Slot* s = nullptr;
        {
            std::lock_guard<std::mutex> lock(p->mu);
            s = &slot_of(*p, slot);
        }
        if (s->tx_done) check_cuda(cudaEventSynchronize(s->tx_done), "synchronize tx_done");  // no TX yet: nothing to wait for
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_tx_batch(unsigned long long handle, const unsigned char* device_info_bits, int frames,
                       float* device_frames, float frequency_noise_var, unsigned long long noise_seed, void* cuda_stream)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tx(*p);
        if (!device_info_bits || !device_frames) throw InvalidArgument("null device pointer");
        if (frames <= 0 || frames > p->batch_frames) throw InvalidArgument("frames must be in 1..max_batch_frames");
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
        launch_tx(p->txv, device_info_bits, frames, reinterpret_cast<float2*>(device_frames), frequency_noise_var,
                  noise_seed, st);
        return CUDA_OSD_STATUS_OK;
    });
}

}  // extern "C"

namespace sicc {
namespace {

// Real-time ingest: device IQ ring (mirrored tail of `mirror` samples, so any
// window of up to `mirror` samples from any read position is contiguous), a
// leased frame pool, and the extraction loop of the receive path.
struct Ingest {
    std::shared_ptr<Pipe> pipe;
    sicc_ingest_config_t cfg{};
    int frame_samples = 0;
    long long cap = 0, mirror = 0;
    Buf<float2> ring;  // [cap + mirror]
    Buf<float2> pool;  // [pool_frames][frame_samples]
    Buf<int> d_slots;
    Buf<unsigned char> d_out;        // IngestState, then [pool_frames] IngestRecord: one readback
    unsigned char* h_out = nullptr;  // pinned copy of d_out
    IngestState* h_state = nullptr;  // in h_out
    IngestRecord* h_rec = nullptr;   // in h_out
    int* h_slots = nullptr;          // pinned
    cudaStream_t copy_stream = nullptr, stream = nullptr;
    cudaEvent_t pushed = nullptr;
    long long read_pos = 0, size = 0, pos_index = 0;  // pos_index: stream index of ring[read_pos]
    unsigned long long dropped = 0;
    bool busy = false, tracking = false, closed = false;
    std::deque<int> free_slots;
    std::vector<char> leased;
    IngestState acc{};
    std::mutex mu, step_mu;
    std::condition_variable cv;
    ~Ingest()
    {
        if (stream) cudaStreamSynchronize(stream);
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        if (h_out) cudaFreeHost(h_out);
        if (h_slots) cudaFreeHost(h_slots);
        if (pushed) cudaEventDestroy(pushed);
        if (stream) cudaStreamDestroy(stream);
        if (copy_stream) cudaStreamDestroy(copy_stream);
    }
    void consume(long long c)  // under mu
    {
        c = std::min(c, size);
        read_pos = (read_pos + c) % cap;
        size -= c;
        pos_index += c;
    }
};

std::map<unsigned long long, std::shared_ptr<Ingest>> g_ingests;
unsigned long long g_next_ingest = 0x9100;

std::shared_ptr<Ingest> get_ingest(unsigned long long h)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_ingests.find(h);
    if (it == g_ingests.end()) throw InvalidArgument("invalid ingest handle");
    return it->second;
}

}  // namespace
}  // namespace sicc

extern "C" {

int sicc_ingest_create(unsigned long long pipe_handle, const sicc_ingest_config_t* config, unsigned long long* out_handle)
{
    return guarded([&] {
        if (!config || !out_handle) throw InvalidArgument("null argument");
        *out_handle = 0;
        auto p = get(pipe_handle);
        std::lock_guard<std::mutex> plock(p->mu);
        require_tables(*p);
        const sicc_ingest_config_t& c = *config;
        if (c.buffered_max <= 0 || c.buffered_min < 0) throw InvalidArgument("buffered_max must be positive");
        if (c.max_buffered_frames < 0 || c.sync_tracking_window < 0) throw InvalidArgument("invalid search windows");
        auto g = std::make_shared<Ingest>();
        g->pipe = p;
        g->cfg = c;
        g->cfg.pool_frames = std::max(c.pool_frames, 4);
        g->frame_samples = p->frame_samples;
        g->mirror = std::max<long long>(std::max(c.buffered_min, c.buffered_max), p->cfg.preamble_len);
        g->cap = std::max<long long>(std::max<long long>(c.ring_samples, 4096), g->mirror);
        check_cuda(cudaSetDevice(p->device), "cudaSetDevice");
        g->ring.alloc(static_cast<size_t>(g->cap + g->mirror));
        check_cuda(cudaMemset(g->ring.p, 0, static_cast<size_t>(g->cap + g->mirror) * sizeof(float2)), "zero ring");
        g->pool.alloc(static_cast<size_t>(g->cfg.pool_frames) * g->frame_samples);
        g->d_slots.alloc(static_cast<size_t>(g->cfg.pool_frames));
        const size_t out_bytes = sizeof(IngestState) + sizeof(IngestRecord) * g->cfg.pool_frames;
        g->d_out.alloc(out_bytes);
        check_cuda(cudaMallocHost(&g->h_out, out_bytes), "cudaMallocHost(ingest)");
        g->h_state = reinterpret_cast<IngestState*>(g->h_out);
        g->h_rec = reinterpret_cast<IngestRecord*>(g->h_out + sizeof(IngestState));
        check_cuda(cudaMallocHost(&g->h_slots, sizeof(int) * g->cfg.pool_frames), "cudaMallocHost(ingest)");
        check_cuda(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate(ingest)");
        check_cuda(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking), "cudaStreamCreate(ingest)");
        check_cuda(cudaEventCreateWithFlags(&g->pushed, cudaEventDisableTiming), "cudaEventCreate(ingest)");
        g->leased.assign(static_cast<size_t>(g->cfg.pool_frames), 0);
        for (int i = 0; i < g->cfg.pool_frames; ++i) g->free_slots.push_back(i);
        std::lock_guard<std::mutex> lock(g_mu);
        *out_handle = ++g_next_ingest;
        g_ingests[*out_handle] = g;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_ingest_destroy(unsigned long long handle)
{
    return guarded([&] {
        std::shared_ptr<Ingest> g;
        {
            std::lock_guard<std::mutex> lock(g_mu);
            auto it = g_ingests.find(handle);
            if (it == g_ingests.end()) throw InvalidArgument("invalid ingest handle");
            g = it->second;
            g_ingests.erase(it);
        }
        {
            std::lock_guard<std::mutex> lock(g->mu);
            g->closed = true;
        }
        g->cv.notify_all();
        std::lock_guard<std::mutex> step(g->step_mu);  // a running step finishes first
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_ingest_push(unsigned long long handle, const float* host_iq, long long count)
{
    return guarded([&] {
        auto g = get_ingest(handle);
        if (count < 0) throw InvalidArgument("count must be >= 0");
        if (!host_iq || count == 0) return CUDA_OSD_STATUS_OK;
        const float2* src = reinterpret_cast<const float2*>(host_iq);
        {
            std::lock_guard<std::mutex> lock(g->mu);
            if (g->closed) return CUDA_OSD_STATUS_OK;
            check_cuda(cudaSetDevice(g->pipe->device), "cudaSetDevice");
            if (count > g->cap) {  // only the newest cap samples can be kept
                const long long skip = count - g->cap;
                src += skip;
                count = g->cap;
                g->dropped += static_cast<unsigned long long>(skip);
            }
            if (g->size + count > g->cap) {
                if (g->busy) {  // the oldest samples are being searched: the new ones that do not fit are lost
                    const long long room = g->cap - g->size;
                    g->dropped += static_cast<unsigned long long>(count - room);
                    count = room;
                } else {  // drop the oldest, as GpuOnlineIqBuffer::push
                    const long long drop = g->size + count - g->cap;
                    g->consume(drop);
                    g->dropped += static_cast<unsigned long long>(drop);
                }
            }
            long long write_pos = (g->read_pos + g->size) % g->cap;
            long long remaining = count;
            const float2* s2 = src;
            while (remaining > 0) {
                const long long n = std::min(remaining, g->cap - write_pos);
                check_cuda(cudaMemcpyAsync(g->ring.p + write_pos, s2, static_cast<size_t>(n) * sizeof(float2),
                                           cudaMemcpyHostToDevice, g->copy_stream),
                           "copy RX samples to the device ring");
                if (write_pos < g->mirror) {  // the mirrored tail repeats the ring's first samples
                    const long long m = std::min(n, g->mirror - write_pos);
                    check_cuda(cudaMemcpyAsync(g->ring.p + g->cap + write_pos, s2, static_cast<size_t>(m) * sizeof(float2),
                                               cudaMemcpyHostToDevice, g->copy_stream),
                               "copy RX samples to the ring tail");
                }
                s2 += n;
                remaining -= n;
                write_pos = (write_pos + n) % g->cap;
            }
            check_cuda(cudaEventRecord(g->pushed, g->copy_stream), "cudaEventRecord(ingest push)");
            g->size += count;
        }
        g->cv.notify_one();
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_ingest_step(unsigned long long handle, int max_frames, int timeout_ms, sicc_ingest_frame_t* out_frames,
                     int* out_count)
{
    return guarded([&] {
        auto g = get_ingest(handle);
        if (!out_count || (max_frames > 0 && !out_frames)) throw InvalidArgument("null argument");
        *out_count = 0;
        std::lock_guard<std::mutex> step(g->step_mu);
        Pipe& p = *g->pipe;
        const int F = g->frame_samples;
        long long window = 0, n = 0, w_index = 0;
        bool latest = false;
        int nslots = 0;
        IngestState st{};
        {
            std::unique_lock<std::mutex> lock(g->mu);
            latest = g->size > g->cap * 3 / 4;
            if (latest) {  // pop_latest_device (L:7754-7766): keep the newest buffered_max, restart acquisition
                if (g->size > g->cfg.buffered_max) {
                    const long long drop = g->size - g->cfg.buffered_max;
                    g->consume(drop);
                    g->dropped += static_cast<unsigned long long>(drop);
                }
                g->tracking = false;
                n = g->size;
            } else {  // peek_batch_device (L:7721-7739)
                g->cv.wait_for(lock, std::chrono::milliseconds(std::max(timeout_ms, 0)),
                               [&] { return g->closed || g->size >= g->cfg.buffered_min; });
                n = std::min<long long>(g->size, std::max(g->cfg.buffered_min, g->cfg.buffered_max));
            }
            if (n == 0) return CUDA_OSD_STATUS_OK;
            window = g->read_pos;
            w_index = g->pos_index;
            g->busy = true;
            nslots = std::min(static_cast<int>(g->free_slots.size()), std::max(max_frames, 0));
            for (int i = 0; i < nslots; ++i) g->h_slots[i] = g->free_slots[static_cast<size_t>(i)];
            st.tracking = g->tracking ? 1 : 0;
        }
        *g->h_state = st;
        IngestParams ip{};
        ip.frame_len = F;
        ip.acq_window = std::max(F, g->cfg.max_buffered_frames * F);
        ip.track_window = p.cfg.preamble_len + std::max(256, g->cfg.sync_tracking_window);
        ip.strict_window = std::max(256, 4 * p.cfg.cp);
        ip.late_threshold = g->cfg.sync_late_peak_threshold;
        ip.max_frames = std::max(max_frames, 0);
        ip.free_slots = nslots;
        try {
            check_cuda(cudaSetDevice(p.device), "cudaSetDevice");
            check_cuda(cudaStreamWaitEvent(g->stream, g->pushed, 0), "cudaStreamWaitEvent(ingest)");
            if (nslots > 0)
                check_cuda(cudaMemcpyAsync(g->d_slots.p, g->h_slots, sizeof(int) * nslots, cudaMemcpyHostToDevice, g->stream),
                           "copy ingest slots");
            IngestState* d_state = reinterpret_cast<IngestState*>(g->d_out.p);
            IngestRecord* d_rec = reinterpret_cast<IngestRecord*>(g->d_out.p + sizeof(IngestState));
            check_cuda(cudaMemcpyAsync(d_state, g->h_state, sizeof(IngestState), cudaMemcpyHostToDevice, g->stream),
                       "copy ingest state");
            launch_ingest_extract(g->ring.p + window, static_cast<int>(n), p.preamble.p, p.sync_params(0), ip,
                                  g->d_slots.p, g->pool.p, d_rec, d_state, g->stream);
            check_cuda(cudaMemcpyAsync(g->h_out, g->d_out.p, sizeof(IngestState) + sizeof(IngestRecord) * nslots,
                                       cudaMemcpyDeviceToHost, g->stream),
                       "copy ingest state and records back");
            check_cuda(cudaStreamSynchronize(g->stream), "synchronize ingest step");
        } catch (...) {
            std::lock_guard<std::mutex> lock(g->mu);
            g->busy = false;
            throw;
        }
        const IngestState& r = *g->h_state;
        std::lock_guard<std::mutex> lock(g->mu);
        g->busy = false;
        for (int i = 0; i < r.frames; ++i) {
            const IngestRecord& rec = g->h_rec[i];
            g->leased[static_cast<size_t>(rec.slot)] = 1;
            g->free_slots.pop_front();  // the slots were taken in list order
            sicc_ingest_frame_t& o = out_frames[i];
            o.slot = rec.slot;
            o.peak = rec.peak;
            o.cfo_hz = rec.cfo_hz;
            o.pad = 0;
            o.position = w_index + rec.start;
        }
        *out_count = r.frames;
        g->acc.found += r.found;
        g->acc.miss += r.miss;
        g->acc.tracking_miss += r.tracking_miss;
        g->acc.incomplete += r.incomplete;
        g->acc.skipped_samples += r.skipped_samples;
        g->acc.max_start = std::max(g->acc.max_start, r.max_start);
        g->acc.pool_exhausted += r.pool_exhausted;
        g->tracking = r.tracking != 0;
        if (latest) {
            g->consume(n);  // the latest window was taken out of the ring
        } else if (r.base > 0) {
            g->consume(r.base);
        } else if (n > F) {  // nothing found: keep one frame's worth, search again from acquisition
            g->consume(n - F);
            g->tracking = false;
        }
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_ingest_frame_ptr(unsigned long long handle, int slot, const float** out_device_frame)
{
    return guarded([&] {
        auto g = get_ingest(handle);
        if (!out_device_frame) throw InvalidArgument("null argument");
        if (slot < 0 || slot >= g->cfg.pool_frames) throw InvalidArgument("invalid pool slot");
        *out_device_frame = reinterpret_cast<const float*>(g->pool.p + static_cast<size_t>(slot) * g->frame_samples);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_ingest_pool(unsigned long long handle, const float** out_device_pool, int* out_frame_samples)
{
    return guarded([&] {
        auto g = get_ingest(handle);
        if (!out_device_pool || !out_frame_samples) throw InvalidArgument("null argument");
        *out_device_pool = reinterpret_cast<const float*>(g->pool.p);
        *out_frame_samples = g->frame_samples;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_ingest_release(unsigned long long handle, int slot)
{
    return guarded([&] {
        auto g = get_ingest(handle);
        std::lock_guard<std::mutex> lock(g->mu);
        if (slot < 0 || slot >= g->cfg.pool_frames || !g->leased[static_cast<size_t>(slot)])
            throw InvalidArgument("pool slot is not leased");
        g->leased[static_cast<size_t>(slot)] = 0;
        g->free_slots.push_back(slot);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_ingest_stats(unsigned long long handle, sicc_ingest_stats_t* out)
{
    return guarded([&] {
        auto g = get_ingest(handle);
        if (!out) throw InvalidArgument("null argument");
        std::lock_guard<std::mutex> lock(g->mu);
        out->found = g->acc.found;
        out->miss = g->acc.miss;
        out->tracking_miss = g->acc.tracking_miss;
        out->incomplete = g->acc.incomplete;
        out->skipped_samples = g->acc.skipped_samples;
        out->max_start = g->acc.max_start;
        out->dropped_samples = g->dropped;
        out->pool_exhausted = g->acc.pool_exhausted;
        out->buffered = g->size;
        out->tracking = g->tracking ? 1 : 0;
        out->free_slots = static_cast<int>(g->free_slots.size());
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_ingest_close(unsigned long long handle)
{
    return guarded([&] {
        auto g = get_ingest(handle);
        {
            std::lock_guard<std::mutex> lock(g->mu);
            g->closed = true;
        }
        g->cv.notify_all();
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_set_demod_shape(unsigned long long handle, int symbols_per_cta)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        require_tables(*p);
        const int nd = static_cast<int>(p->h_p0.size());
        if (symbols_per_cta < 1 || symbols_per_cta > nd)
            throw InvalidArgument("symbols_per_cta must be in 1..data symbols per frame");
        if (pilot_span(*p, symbols_per_cta) > kDemodMaxPilots)
            throw InvalidArgument("the data symbols of one CTA would need more than " + std::to_string(kDemodMaxPilots) +
                                  " pilot symbols");
        p->symbols_per_cta = symbols_per_cta;
        p->view.max_pilots_per_cta = pilot_span(*p, symbols_per_cta);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_wait_timeouts(unsigned int* out_count)
{
    return guarded([&] {
        if (!out_count) throw InvalidArgument("null argument");
        *out_count = demod_wait_timeouts();
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_pipe_last_batch_ms(unsigned long long handle, float* out_sync_ms, float* out_demod_ms)
{
    return guarded([&] {
        auto p = get(handle);
        std::lock_guard<std::mutex> lock(p->mu);
        if (!p->batch_timed) throw InvalidArgument("no batch has run");
        check_cuda(cudaEventSynchronize(p->ev[2]), "cudaEventSynchronize");
        float a = 0.0f, b = 0.0f;
        check_cuda(cudaEventElapsedTime(&a, p->ev[0], p->ev[1]), "cudaEventElapsedTime");
        check_cuda(cudaEventElapsedTime(&b, p->ev[1], p->ev[2]), "cudaEventElapsedTime");
        if (out_sync_ms) *out_sync_ms = a;
        if (out_demod_ms) *out_demod_ms = b;
        return CUDA_OSD_STATUS_OK;
    });
}

}  // extern "C"
