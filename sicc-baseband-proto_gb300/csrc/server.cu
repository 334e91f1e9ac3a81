// Device-resident continuous-batching decode service (include/sicc_server.h).
//
// Request life cycle: submit (pending queue) -> admitted (arena block
// allocated first-in first-out, input copied host->device on the copy
// stream) -> ready (copy finished) -> running (part of a batch launched on
// one of the batch slots' streams) -> done (results copied back, arena block
// freed, completion queued).  One scheduler thread drives every transition
// except submit; up to max_inflight_batches batches overlap on the device,
// each slot with its own engine (the engine's scratch is per launch) and
// staging buffers.
#include "../../include/sicc_server.h"
#include "engine_internal.h"
#include "sicc_common.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace sicc {
namespace {

using Clock = std::chrono::steady_clock;

double us_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::micro>(b - a).count();
}

// First-fit allocator over [0, size) with coalescing; 256-byte granules.
class Arena {
public:
    explicit Arena(long long size) : size_(size) { free_[0] = size; }
    long long alloc(long long bytes)
    {
        bytes = (bytes + 255) & ~255LL;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                const long long off = it->first;
                const long long rest = it->second - bytes;
                free_.erase(it);
                if (rest > 0) free_[off + bytes] = rest;
                used_ += bytes;
                peak_ = std::max(peak_, used_);
                return off;
            }
        }
        return -1;
    }
    void release(long long off, long long bytes)
    {
        bytes = (bytes + 255) & ~255LL;
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    long long used() const { return used_; }
    long long peak() const { return peak_; }

private:
    long long size_;
    long long used_ = 0, peak_ = 0;
    std::map<long long, long long> free_;
};

struct CodeInfo {
    int n, k;
};

struct Phy {
    unsigned long long pipe = 0;
    int frame_stride = 0;  // complex samples per frame buffer
    int code_id = 0;
    int blocks = 0;        // codewords per frame
};

struct Req {
    unsigned long long id = 0;
    sicc_request_t spec{};
    int codewords = 0;
    int n = 0, k = 0;
    long long off = -1, bytes = 0;   // arena block
    long long in_off = 0, llr_off = 0, info_off = 0;  // offsets inside the arena
    Clock::time_point t_submit, t_admit, t_launch;
    int first_cw = 0;        // its first codeword in the batch
    bool completed = false;  // BP-only requests complete after BP, before the batch's OSD
    cudaEvent_t h2d = nullptr;
};

struct Slot {
    unsigned long long engine = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t early = nullptr;  // copies back the BP-only requests once BP is done
    cudaEvent_t start = nullptr, done = nullptr, bp_done = nullptr, early_done = nullptr;
    bool busy = false;
    bool early_pending = false;
    std::vector<std::shared_ptr<Req>> reqs;
    // per-codeword metadata: host staging (pinned) and device copies
    uint8_t* h_code = nullptr;
    uint8_t* h_prot = nullptr;
    long long* h_llr_off = nullptr;
    long long* h_info_off = nullptr;
    uint8_t* h_ok = nullptr;
    uint8_t* h_used = nullptr;
    long long* h_frame_off = nullptr;  // IQ frames of the batch: input offset (complex samples)
    long long* h_fllr_off = nullptr;   // and LLR offset (floats), both from the arena base
    uint8_t* d_meta = nullptr;         // one allocation holding the device arrays below
    uint8_t *d_code = nullptr, *d_prot = nullptr, *d_ok = nullptr, *d_used = nullptr;
    long long *d_llr_off = nullptr, *d_info_off = nullptr, *d_frame_off = nullptr, *d_fllr_off = nullptr;
    sicc_pipe_sync_record_t* d_sync = nullptr;
    int count = 0;
};

struct Server {
    sicc_server_config_t cfg{};
    int device = 0;
    unsigned char* arena_base = nullptr;
    std::unique_ptr<Arena> arena;
    std::vector<CodeInfo> codes;
    std::vector<sicc_engine_code_t> code_specs;
    std::vector<std::vector<int>> code_csr;  // keeps host CSR alive for the engines
    std::vector<Phy> phys;
    std::vector<Slot> slots;
    cudaStream_t copy_stream = nullptr;
    std::deque<std::shared_ptr<Req>> pending, admitted;
    std::deque<sicc_completion_t> completions;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    std::atomic<bool> running{false};
    bool started = false;
    std::string fatal;  // why the scheduler stopped (error text is per thread)
    unsigned long long next_id = 1;
    sicc_server_stats_t stats{};

    ~Server() { shutdown(); }

    void shutdown()
    {
        if (running.exchange(false)) {
            cv_work.notify_all();
            if (worker.joinable()) worker.join();
        }
        cudaSetDevice(device);
        for (auto& s : slots) {
            if (s.stream) cudaStreamSynchronize(s.stream);
            if (s.engine) sicc_engine_destroy(s.engine);
            if (s.stream) cudaStreamDestroy(s.stream);
            if (s.early) cudaStreamSynchronize(s.early);
            if (s.done) cudaEventDestroy(s.done);
            if (s.start) cudaEventDestroy(s.start);
            if (s.bp_done) cudaEventDestroy(s.bp_done);
            if (s.early_done) cudaEventDestroy(s.early_done);
            if (s.early) cudaStreamDestroy(s.early);
            for (void* p : {static_cast<void*>(s.h_code), static_cast<void*>(s.h_prot),
                            static_cast<void*>(s.h_llr_off), static_cast<void*>(s.h_info_off),
                            static_cast<void*>(s.h_ok), static_cast<void*>(s.h_used),
                            static_cast<void*>(s.h_frame_off), static_cast<void*>(s.h_fllr_off)})
                if (p) cudaFreeHost(p);
            if (s.d_meta) cudaFree(s.d_meta);
            s = Slot{};
        }
        for (auto& p : phys)
            if (p.pipe) sicc_pipe_destroy(p.pipe);
        phys.clear();
        if (copy_stream) {
            cudaStreamSynchronize(copy_stream);
            cudaStreamDestroy(copy_stream);
            copy_stream = nullptr;
        }
        for (auto& q : {&pending, &admitted})
            for (auto& r : *q)
                if (r->h2d) cudaEventDestroy(r->h2d);
        pending.clear();
        admitted.clear();
        if (arena_base) cudaFree(arena_base);
        arena_base = nullptr;
    }

    // -- scheduler steps (called with mu held) --
    void admit()
    {
        while (!pending.empty()) {
            auto r = pending.front();
            const long long off = arena->alloc(r->bytes);
            if (off < 0) break;  // first-in first-out: later requests wait behind this one
            r->off = off;
            r->in_off += off;
            r->llr_off += off;
            r->info_off += off;
            r->t_admit = Clock::now();
            const size_t in_bytes = r->spec.kind == 0 ? static_cast<size_t>(r->codewords) * r->n * sizeof(float)
                                                      : static_cast<size_t>(r->spec.count) *
                                                            phys[r->spec.phy_id].frame_stride * 2 * sizeof(float);
            check_cuda(cudaMemcpyAsync(arena_base + r->in_off, r->spec.host_input, in_bytes, cudaMemcpyHostToDevice,
                                       copy_stream),
                       "copy request input");
            check_cuda(cudaEventCreateWithFlags(&r->h2d, cudaEventDisableTiming), "cudaEventCreate(request)");
            check_cuda(cudaEventRecord(r->h2d, copy_stream), "cudaEventRecord(request)");
            pending.pop_front();
            admitted.push_back(r);
        }
        stats.arena_bytes_in_use = arena->used();
        stats.arena_bytes_peak = arena->peak();
    }

    bool launch()
    {
        int si = -1;
        for (size_t i = 0; i < slots.size(); ++i)
            if (!slots[i].busy) { si = static_cast<int>(i); break; }
        if (si < 0 || admitted.empty()) return false;
        Slot& s = slots[si];
        s.reqs.clear();
        s.count = 0;
        while (!admitted.empty()) {
            auto r = admitted.front();
            if (cudaEventQuery(r->h2d) != cudaSuccess) break;  // in submission order
            if (s.count > 0 && s.count + r->codewords > cfg.max_batch_codewords) break;
            s.reqs.push_back(r);
            s.count += r->codewords;
            admitted.pop_front();
        }
        if (s.reqs.empty()) return false;
        const auto t_launch = Clock::now();
        for (auto& r : s.reqs) r->t_launch = t_launch;
        check_cuda(cudaEventRecord(s.start, s.stream), "cudaEventRecord(batch)");
        // demodulate the IQ requests into their LLR areas: one gathered sync + demod launch pair per profile
        std::vector<int> phy_first(phys.size() + 1, 0);
        int nf = 0;
        for (size_t pi = 0; pi < phys.size(); ++pi) {
            phy_first[pi] = nf;
            for (auto& r : s.reqs) {
                if (r->spec.kind != 1 || r->spec.phy_id != static_cast<int>(pi)) continue;
                const Phy& p = phys[pi];
                for (int i = 0; i < r->spec.count; ++i, ++nf) {
                    s.h_frame_off[nf] = r->in_off / 8 + static_cast<long long>(i) * p.frame_stride;
                    s.h_fllr_off[nf] = r->llr_off / 4 + static_cast<long long>(i) * p.blocks * r->n;
                }
            }
        }
        phy_first[phys.size()] = nf;
        if (nf > 0) {
            check_cuda(cudaMemcpyAsync(s.d_frame_off, s.h_frame_off, nf * sizeof(long long), cudaMemcpyHostToDevice,
                                       s.stream),
                       "copy frame table");
            check_cuda(cudaMemcpyAsync(s.d_fllr_off, s.h_fllr_off, nf * sizeof(long long), cudaMemcpyHostToDevice,
                                       s.stream),
                       "copy frame table");
            for (size_t pi = 0; pi < phys.size(); ++pi) {
                const int f0 = phy_first[pi], f1 = phy_first[pi + 1];
                if (f1 == f0) continue;
                const Phy& p = phys[pi];
                const int st = sicc_pipe_demod_gather(p.pipe, reinterpret_cast<const float*>(arena_base),
                                                      s.d_frame_off + f0, p.frame_stride, f1 - f0,
                                                      reinterpret_cast<float*>(arena_base), s.d_fllr_off + f0,
                                                      s.d_sync + f0, s.stream);
                if (st != CUDA_OSD_STATUS_OK) throw std::runtime_error(std::string("demod: ") + last_error());
            }
        }
        // per-codeword metadata of the batch
        int c = 0;
        for (auto& r : s.reqs) {
            r->first_cw = c;
            r->completed = false;
            const int cid = r->spec.kind == 0 ? r->spec.code_id : phys[r->spec.phy_id].code_id;
            for (int i = 0; i < r->codewords; ++i, ++c) {
                s.h_code[c] = static_cast<uint8_t>(cid);
                s.h_prot[c] = static_cast<uint8_t>(r->spec.protection ? 1 : 0);
                s.h_llr_off[c] = (r->llr_off / static_cast<long long>(sizeof(float))) + static_cast<long long>(i) * r->n;
                s.h_info_off[c] = r->info_off + static_cast<long long>(i) * r->k;
            }
        }
        uint8_t* d_code = s.d_code;
        uint8_t* d_prot = s.d_prot;
        long long* d_llr_off = s.d_llr_off;
        long long* d_info_off = s.d_info_off;
        uint8_t* d_ok = s.d_ok;
        uint8_t* d_used = s.d_used;
        check_cuda(cudaMemcpyAsync(d_code, s.h_code, s.count, cudaMemcpyHostToDevice, s.stream), "copy meta");
        check_cuda(cudaMemcpyAsync(d_prot, s.h_prot, s.count, cudaMemcpyHostToDevice, s.stream), "copy meta");
        check_cuda(cudaMemcpyAsync(d_llr_off, s.h_llr_off, s.count * sizeof(long long), cudaMemcpyHostToDevice,
                                   s.stream),
                   "copy meta");
        check_cuda(cudaMemcpyAsync(d_info_off, s.h_info_off, s.count * sizeof(long long), cudaMemcpyHostToDevice,
                                   s.stream),
                   "copy meta");
        const int st = engine_decode(s.engine, s.count, d_code, d_prot, reinterpret_cast<const float*>(arena_base),
                                     d_llr_off, arena_base, d_info_off, d_ok, d_used, nullptr, s.stream, s.bp_done);
        if (st != CUDA_OSD_STATUS_OK) throw std::runtime_error(std::string("decode: ") + last_error());
        // BP-only requests are final once BP is done: copy them back on the early stream while
        // the batch's OSD runs (success flags are final after BP for every codeword)
        bool any_early = false;
        for (auto& r : s.reqs) any_early |= (r->spec.protection == 0);
        if (any_early) {
            check_cuda(cudaStreamWaitEvent(s.early, s.bp_done, 0), "cudaStreamWaitEvent(bp done)");
            check_cuda(cudaMemcpyAsync(s.h_ok, d_ok, s.count, cudaMemcpyDeviceToHost, s.early), "copy flags");
            for (auto& r : s.reqs)
                if (r->spec.protection == 0)
                    check_cuda(cudaMemcpyAsync(r->spec.host_info, arena_base + r->info_off,
                                               static_cast<size_t>(r->codewords) * r->k, cudaMemcpyDeviceToHost,
                                               s.early),
                               "copy results");
            check_cuda(cudaEventRecord(s.early_done, s.early), "cudaEventRecord(early)");
            s.early_pending = true;
        } else {
            check_cuda(cudaMemcpyAsync(s.h_ok, d_ok, s.count, cudaMemcpyDeviceToHost, s.stream), "copy flags");
        }
        check_cuda(cudaMemcpyAsync(s.h_used, d_used, s.count, cudaMemcpyDeviceToHost, s.stream), "copy flags");
        for (auto& r : s.reqs)
            if (r->spec.protection != 0)
                check_cuda(cudaMemcpyAsync(r->spec.host_info, arena_base + r->info_off,
                                           static_cast<size_t>(r->codewords) * r->k, cudaMemcpyDeviceToHost, s.stream),
                           "copy results");
        if (any_early) check_cuda(cudaStreamWaitEvent(s.stream, s.early_done, 0), "cudaStreamWaitEvent(early)");
        check_cuda(cudaEventRecord(s.done, s.stream), "cudaEventRecord(batch)");
        s.busy = true;
        stats.batches += 1;
        stats.codewords += static_cast<unsigned long long>(s.count);
        stats.mean_batch_codewords = static_cast<double>(stats.codewords) / static_cast<double>(stats.batches);
        return true;
    }

    // Completes request r of slot s (its results are on the host); with_used: the OSD flags are too.
    void complete(Slot& s, Req& r, Clock::time_point now, cudaEvent_t until, bool with_used)
    {
        float gpu_ms = 0.0f;
        cudaEventElapsedTime(&gpu_ms, s.start, until);
        sicc_completion_t done{};
        done.request_id = r.id;
        done.tag = r.spec.tag;
        done.codewords = r.codewords;
        for (int i = 0; i < r.codewords; ++i) {
            const int c = r.first_cw + i;
            const bool used = with_used && s.h_used[c];
            done.osd_codewords += used ? 1 : 0;
            done.failed_codewords += (!s.h_ok[c] && !used) ? 1 : 0;
        }
        done.latency_us = us_between(r.t_submit, now);
        done.queue_us = us_between(r.t_submit, r.t_admit);
        done.launch_us = us_between(r.t_submit, r.t_launch);
        done.batch_gpu_us = 1000.0 * gpu_ms;
        arena->release(r.off, r.bytes);  // no later work of the batch touches this block
        if (r.h2d) cudaEventDestroy(r.h2d);
        r.h2d = nullptr;
        r.completed = true;
        completions.push_back(done);
        stats.completed += 1;
    }

    bool retire()
    {
        bool any = false;
        for (auto& s : slots) {
            if (!s.busy) continue;
            if (s.early_pending && cudaEventQuery(s.early_done) == cudaSuccess) {  // BP-only requests
                const auto now = Clock::now();
                for (auto& r : s.reqs)
                    if (r->spec.protection == 0) complete(s, *r, now, s.early_done, false);
                s.early_pending = false;
                any = true;
            }
            if (cudaEventQuery(s.done) != cudaSuccess) continue;
            const auto now = Clock::now();
            for (auto& r : s.reqs)
                if (!r->completed) complete(s, *r, now, s.done, true);
            s.reqs.clear();
            s.busy = false;
            any = true;
        }
        if (any) cv_done.notify_all();
        return any;
    }

    void loop()
    {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lock(mu);
        while (running.load()) {
            bool progress = false;
            try {
                progress |= retire();
                admit();
                while (launch()) progress = true;
            } catch (const std::exception& e) {
                fatal = e.what();
                running.store(false);
                cv_done.notify_all();
                break;
            }
            if (!progress) cv_work.wait_for(lock, std::chrono::microseconds(20));
        }
    }
};

std::mutex g_mu;
std::map<unsigned long long, std::shared_ptr<Server>> g_servers;
unsigned long long g_next = 0xA100;

std::shared_ptr<Server> get(unsigned long long h)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_servers.find(h);
    if (it == g_servers.end()) throw InvalidArgument("invalid server handle");
    return it->second;
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

}  // namespace
}  // namespace sicc

using namespace sicc;

extern "C" {

int sicc_server_create(const sicc_server_config_t* config, unsigned long long* out_handle)
{
    return guarded([&]() -> int {
        if (!config || !out_handle) throw InvalidArgument("null argument");
        *out_handle = 0;
        const auto& c = *config;
        if (c.hbm_budget_bytes < (1 << 20)) throw InvalidArgument("hbm_budget_bytes must be at least 1 MiB");
        if (c.max_batch_codewords <= 0 || c.max_inflight_batches < 1 || c.max_inflight_batches > 4)
            throw InvalidArgument("max_batch_codewords > 0 and 1 <= max_inflight_batches <= 4 required");
        if (c.max_pending_requests <= 0 || c.max_codes <= 0 || c.max_codes > 64 || c.max_n <= 0)
            throw InvalidArgument("max_pending_requests, max_codes (<= 64) and max_n must be positive");
        auto s = std::make_shared<Server>();
        s->cfg = c;
        check_cuda(cudaGetDevice(&s->device), "cudaGetDevice");
        check_cuda(cudaMalloc(&s->arena_base, static_cast<size_t>(c.hbm_budget_bytes)), "cudaMalloc(arena)");
        s->arena = std::make_unique<Arena>(c.hbm_budget_bytes);
        check_cuda(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        std::lock_guard<std::mutex> lock(g_mu);
        *out_handle = ++g_next;
        g_servers[*out_handle] = s;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_server_destroy(unsigned long long handle)
{
    return guarded([&]() -> int {
        std::shared_ptr<Server> s;
        {
            std::lock_guard<std::mutex> lock(g_mu);
            auto it = g_servers.find(handle);
            if (it == g_servers.end()) throw InvalidArgument("invalid server handle");
            s = it->second;
            g_servers.erase(it);
        }
        s->shutdown();
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_server_add_code(unsigned long long handle, const sicc_engine_code_t* code, int* out_code_id)
{
    return guarded([&]() -> int {
        auto s = get(handle);
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->started) throw InvalidArgument("codes must be registered before start");
        if (!code || !out_code_id || !code->row_ptr || !code->col_ind) throw InvalidArgument("null argument");
        if (static_cast<int>(s->codes.size()) >= s->cfg.max_codes) throw InvalidArgument("server holds max_codes codes");
        if (code->n > s->cfg.max_n) throw InvalidArgument("code longer than max_n");
        if (code->m <= 0 || code->m >= code->n) throw InvalidArgument("need 0 < m < n");
        sicc_engine_code_t spec = *code;
        std::vector<int> rp(code->row_ptr, code->row_ptr + code->m + 1);
        std::vector<int> ci(code->col_ind, code->col_ind + rp.back());
        s->code_csr.push_back(rp);
        s->code_csr.push_back(ci);
        spec.row_ptr = s->code_csr[s->code_csr.size() - 2].data();
        spec.col_ind = s->code_csr.back().data();
        s->code_specs.push_back(spec);
        s->codes.push_back(CodeInfo{code->n, code->n - code->m});
        *out_code_id = static_cast<int>(s->codes.size()) - 1;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_server_add_phy(unsigned long long handle, const sicc_pipe_config_t* config, const sicc_pipe_tables_t* tables,
                        int frame_stride, int code_id, int* out_phy_id)
{
    return guarded([&]() -> int {
        auto s = get(handle);
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->started) throw InvalidArgument("PHY profiles must be registered before start");
        if (!config || !tables || !out_phy_id) throw InvalidArgument("null argument");
        if (code_id < 0 || code_id >= static_cast<int>(s->codes.size())) throw InvalidArgument("unknown code_id");
        if (config->code_n != s->codes[code_id].n) throw InvalidArgument("PHY code_n differs from the code's n");
        const int frame = config->preamble_len + config->num_symbols * (config->nfft + config->cp);
        if (frame_stride < frame) throw InvalidArgument("frame_stride shorter than a frame");
        check_cuda(cudaSetDevice(s->device), "cudaSetDevice");
        sicc_pipe_config_t pc = *config;
        pc.max_rx_search_samples = frame_stride;
        pc.max_batch_frames = std::max(pc.max_batch_frames, s->cfg.max_batch_codewords);  // frames <= codewords
        Phy p;
        if (sicc_pipe_create(&pc, 1, &p.pipe) != CUDA_OSD_STATUS_OK) throw InvalidArgument(last_error());
        if (sicc_pipe_upload_static_tables(p.pipe, tables) != CUDA_OSD_STATUS_OK) {
            sicc_pipe_destroy(p.pipe);
            throw InvalidArgument(last_error());
        }
        p.frame_stride = frame_stride;
        p.code_id = code_id;
        p.blocks = config->blocks_per_frame;
        s->phys.push_back(p);
        *out_phy_id = static_cast<int>(s->phys.size()) - 1;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_server_start(unsigned long long handle)
{
    return guarded([&]() -> int {
        auto s = get(handle);
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->started) throw InvalidArgument("server already started");
        if (s->codes.empty()) throw InvalidArgument("no code registered");
        check_cuda(cudaSetDevice(s->device), "cudaSetDevice");
        int nmax = 0;
        for (auto& c : s->codes) nmax = std::max(nmax, c.n);
        const int N = s->cfg.max_batch_codewords;
        s->slots.resize(s->cfg.max_inflight_batches);
        for (auto& sl : s->slots) {
            sicc_engine_config_t ec{N, static_cast<long long>(N) * nmax, static_cast<int>(s->codes.size())};
            if (sicc_engine_create(&ec, &sl.engine) != CUDA_OSD_STATUS_OK) throw InvalidArgument(last_error());
            for (auto& spec : s->code_specs) {
                int id = 0;
                if (sicc_engine_add_code(sl.engine, &spec, &id) != CUDA_OSD_STATUS_OK) throw InvalidArgument(last_error());
            }
            check_cuda(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking), "cudaStreamCreate(slot)");
            check_cuda(cudaEventCreate(&sl.done), "cudaEventCreate(slot)");
            check_cuda(cudaEventCreate(&sl.start), "cudaEventCreate(slot)");
            check_cuda(cudaEventCreate(&sl.early_done), "cudaEventCreate(slot)");
            check_cuda(cudaEventCreateWithFlags(&sl.bp_done, cudaEventDisableTiming), "cudaEventCreate(slot)");
            check_cuda(cudaStreamCreateWithFlags(&sl.early, cudaStreamNonBlocking), "cudaStreamCreate(slot)");
            check_cuda(cudaMallocHost(&sl.h_code, N), "cudaMallocHost");
            check_cuda(cudaMallocHost(&sl.h_prot, N), "cudaMallocHost");
            check_cuda(cudaMallocHost(&sl.h_llr_off, N * sizeof(long long)), "cudaMallocHost");
            check_cuda(cudaMallocHost(&sl.h_info_off, N * sizeof(long long)), "cudaMallocHost");
            check_cuda(cudaMallocHost(&sl.h_ok, N), "cudaMallocHost");
            check_cuda(cudaMallocHost(&sl.h_used, N), "cudaMallocHost");
            check_cuda(cudaMallocHost(&sl.h_frame_off, N * sizeof(long long)), "cudaMallocHost");
            check_cuda(cudaMallocHost(&sl.h_fllr_off, N * sizeof(long long)), "cudaMallocHost");
            // device arrays, each 256-byte aligned: 4 x N long long, N sync records, 4 x N bytes
            const size_t a8 = (static_cast<size_t>(N) * sizeof(long long) + 255) & ~size_t(255);
            const size_t as = (static_cast<size_t>(N) * sizeof(sicc_pipe_sync_record_t) + 255) & ~size_t(255);
            const size_t a1 = (static_cast<size_t>(N) + 255) & ~size_t(255);
            check_cuda(cudaMalloc(&sl.d_meta, 4 * a8 + as + 4 * a1), "cudaMalloc(batch meta)");
            uint8_t* q = sl.d_meta;
            sl.d_llr_off = reinterpret_cast<long long*>(q);
            sl.d_info_off = reinterpret_cast<long long*>(q + a8);
            sl.d_frame_off = reinterpret_cast<long long*>(q + 2 * a8);
            sl.d_fllr_off = reinterpret_cast<long long*>(q + 3 * a8);
            sl.d_sync = reinterpret_cast<sicc_pipe_sync_record_t*>(q + 4 * a8);
            sl.d_code = q + 4 * a8 + as;
            sl.d_prot = sl.d_code + a1;
            sl.d_ok = sl.d_prot + a1;
            sl.d_used = sl.d_ok + a1;
        }
        s->running.store(true);
        s->started = true;
        s->worker = std::thread([p = s.get()] { p->loop(); });
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_server_submit(unsigned long long handle, const sicc_request_t* request, unsigned long long* out_request_id)
{
    return guarded([&]() -> int {
        auto s = get(handle);
        if (!request || !out_request_id) throw InvalidArgument("null argument");
        const auto& q = *request;
        if (q.count <= 0 || !q.host_input || !q.host_info) throw InvalidArgument("empty request or null buffers");
        auto r = std::make_shared<Req>();
        r->spec = q;
        std::unique_lock<std::mutex> lock(s->mu);
        if (!s->started || !s->running.load())
            throw std::runtime_error(s->started ? "server stopped: " + s->fatal : std::string("server is not started"));
        if (q.kind == 0) {
            if (q.code_id < 0 || q.code_id >= static_cast<int>(s->codes.size())) throw InvalidArgument("unknown code_id");
            r->n = s->codes[q.code_id].n;
            r->k = s->codes[q.code_id].k;
            r->codewords = q.count;
            const long long in = static_cast<long long>(q.count) * r->n * 4;
            r->in_off = 0;
            r->llr_off = 0;  // decoded in place
            r->info_off = (in + 255) & ~255LL;
            r->bytes = r->info_off + static_cast<long long>(q.count) * r->k;
        } else if (q.kind == 1) {
            if (q.phy_id < 0 || q.phy_id >= static_cast<int>(s->phys.size())) throw InvalidArgument("unknown phy_id");
            const Phy& p = s->phys[q.phy_id];
            r->n = s->codes[p.code_id].n;
            r->k = s->codes[p.code_id].k;
            r->codewords = q.count * p.blocks;
            const long long in = static_cast<long long>(q.count) * p.frame_stride * 8;
            r->in_off = 0;
            r->llr_off = (in + 255) & ~255LL;
            r->info_off = (r->llr_off + static_cast<long long>(r->codewords) * r->n * 4 + 255) & ~255LL;
            r->bytes = r->info_off + static_cast<long long>(r->codewords) * r->k;
        } else {
            throw InvalidArgument("kind must be 0 (LLRs) or 1 (OFDM IQ)");
        }
        if (r->codewords > s->cfg.max_batch_codewords) throw InvalidArgument("request larger than max_batch_codewords");
        if (r->bytes > s->cfg.hbm_budget_bytes) throw InvalidArgument("request larger than the HBM budget");
        if (static_cast<int>(s->pending.size()) >= s->cfg.max_pending_requests) {
            s->stats.busy_rejections += 1;
            set_last_error("pending queue full");
            return static_cast<int>(SICC_SERVER_BUSY);
        }
        r->id = s->next_id++;
        r->t_submit = Clock::now();
        s->pending.push_back(r);
        s->stats.submitted += 1;
        *out_request_id = r->id;
        lock.unlock();
        s->cv_work.notify_one();
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_server_poll(unsigned long long handle, int max, sicc_completion_t* out, int* out_count, int wait_us)
{
    return guarded([&]() -> int {
        auto s = get(handle);
        if (!out || !out_count || max <= 0) throw InvalidArgument("bad arguments");
        *out_count = 0;
        std::unique_lock<std::mutex> lock(s->mu);
        if (s->completions.empty() && wait_us > 0)
            s->cv_done.wait_for(lock, std::chrono::microseconds(wait_us), [&] { return !s->completions.empty() || !s->running.load(); });
        while (*out_count < max && !s->completions.empty()) {
            out[(*out_count)++] = s->completions.front();
            s->completions.pop_front();
        }
        if (*out_count == 0 && !s->running.load() && s->started)
            throw std::runtime_error("server stopped: " + s->fatal);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_server_get_stats(unsigned long long handle, sicc_server_stats_t* out)
{
    return guarded([&]() -> int {
        auto s = get(handle);
        if (!out) throw InvalidArgument("null argument");
        std::lock_guard<std::mutex> lock(s->mu);
        *out = s->stats;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_server_replay(unsigned long long handle, const sicc_request_t* requests, const double* arrival_us, int count,
                       sicc_completion_t* out_completions, double* out_wall_us)
{
    return guarded([&]() -> int {
        auto s = get(handle);
        if (!requests || !arrival_us || !out_completions || count <= 0) throw InvalidArgument("bad arguments");
        // Both threads below touch index, orphans, out_completions and t_last under idx_mu.
        std::map<unsigned long long, int> index;  // request id -> position
        // A request can complete before sicc_server_submit has returned its id to the submitting
        // thread; such completions wait here until the submitter records the id, then finish.
        std::map<unsigned long long, sicc_completion_t> orphans;
        std::vector<double> late(count, 0.0);      // submit time minus scheduled arrival
        std::mutex idx_mu;
        std::atomic<int> done_count{0};
        std::atomic<bool> failed{false};
        std::string error;
        const auto t0 = Clock::now();
        Clock::time_point t_last = t0;
        auto finish = [&](int pos, const sicc_completion_t& c) {  // caller holds idx_mu
            out_completions[pos] = c;
            out_completions[pos].latency_us += late[pos];
            out_completions[pos].queue_us += late[pos];
            out_completions[pos].launch_us += late[pos];
            t_last = Clock::now();
            done_count.fetch_add(1);
        };
        std::thread collector([&] {
            std::vector<sicc_completion_t> buf(256);
            while (done_count.load() < count && !failed.load()) {
                int got = 0;
                if (sicc_server_poll(handle, 256, buf.data(), &got, 1000) != CUDA_OSD_STATUS_OK) {
                    error = last_error();
                    failed.store(true);
                    break;
                }
                std::lock_guard<std::mutex> lock(idx_mu);
                for (int i = 0; i < got; ++i) {
                    auto it = index.find(buf[i].request_id);
                    if (it != index.end()) finish(it->second, buf[i]);
                    else orphans.emplace(buf[i].request_id, buf[i]);
                }
            }
        });
        for (int i = 0; i < count && !failed.load(); ++i) {
            const auto due = t0 + std::chrono::nanoseconds(static_cast<long long>(arrival_us[i] * 1000.0));
            while (Clock::now() < due) {
                const auto left = due - Clock::now();
                if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
            }
            unsigned long long id = 0;
            int st;
            while ((st = sicc_server_submit(handle, &requests[i], &id)) == SICC_SERVER_BUSY && !failed.load())
                std::this_thread::sleep_for(std::chrono::microseconds(20));
            if (st != CUDA_OSD_STATUS_OK) {
                error = last_error();
                failed.store(true);
                break;
            }
            late[i] = us_between(due, Clock::now());
            std::lock_guard<std::mutex> lock(idx_mu);
            index[id] = i;
            auto early = orphans.find(id);
            if (early != orphans.end()) {
                finish(i, early->second);
                orphans.erase(early);
            }
        }
        collector.join();
        if (failed.load()) throw std::runtime_error("replay failed: " + error);
        if (out_wall_us) *out_wall_us = us_between(t0, t_last);
        return CUDA_OSD_STATUS_OK;
    });
}

}  // extern "C"
