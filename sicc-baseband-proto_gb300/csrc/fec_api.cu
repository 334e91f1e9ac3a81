// C ABI of the LDPC decoders: cuda_osd_* (the reference's decoder-library
// interface) plus the sicc_* device-resident extensions.  See include/sicc_fec.h.
#include "../../include/sicc_fec.h"
#include "bp_kernels.h"
#include "code_plan.h"
#include "tune_internal.h"
#include "../../include/sicc_tune.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

namespace sicc {

namespace {

// CCSDS (128,64) parity-check matrix, the reference library's built-in code:
// 4 x 8 blocks of 16 x 16 circulants, each a sum of the listed cyclic shifts
// (row t of shift s has its one in column (t + s) mod 16; empty = zero block).
const int kCcsdsShifts[4][8][2] = {
    {{0, 7}, {2, -1}, {14, -1}, {6, -1}, {-1, -1}, {0, -1}, {13, -1}, {0, -1}},
    {{6, -1}, {0, 15}, {0, -1}, {1, -1}, {0, -1}, {-1, -1}, {0, -1}, {7, -1}},
    {{4, -1}, {1, -1}, {0, 15}, {14, -1}, {11, -1}, {0, -1}, {-1, -1}, {3, -1}},
    {{0, -1}, {1, -1}, {9, -1}, {0, 13}, {14, -1}, {1, -1}, {0, -1}, {-1, -1}},
};

void ccsds_128_64(std::vector<int>& row_ptr, std::vector<int>& col_ind)
{
    row_ptr.assign(1, 0);
    col_ind.clear();
    for (int L = 0; L < 4; ++L)
        for (int t = 0; t < 16; ++t) {
            std::vector<int> cols;
            for (int b = 0; b < 8; ++b)
                for (int x = 0; x < 2; ++x)
                    if (kCcsdsShifts[L][b][x] >= 0) cols.push_back(b * 16 + (t + kCcsdsShifts[L][b][x]) % 16);
            std::sort(cols.begin(), cols.end());
            col_ind.insert(col_ind.end(), cols.begin(), cols.end());
            row_ptr.push_back(static_cast<int>(col_ind.size()));
        }
}

void csr_from_dense(const unsigned char* h, int m, int n, std::vector<int>& row_ptr, std::vector<int>& col_ind)
{
    row_ptr.assign(1, 0);
    col_ind.clear();
    for (int r = 0; r < m; ++r) {
        for (int c = 0; c < n; ++c)
            if (h[static_cast<size_t>(r) * n + c]) col_ind.push_back(c);
        row_ptr.push_back(static_cast<int>(col_ind.size()));
    }
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t count = 0;
    void alloc(size_t c)
    {
        release();
        count = c;
        if (c) check_cuda(cudaMalloc(&p, c * sizeof(T)), "cudaMalloc");
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        count = 0;
    }
    ~DevBuf() { release(); }
};

template <class T>
struct HostBuf {
    T* p = nullptr;
    size_t count = 0;
    void alloc(size_t c)
    {
        release();
        count = c;
        if (c) check_cuda(cudaMallocHost(&p, c * sizeof(T)), "cudaMallocHost");
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        count = 0;
    }
    ~HostBuf() { release(); }
};

uint64_t now_us()
{
    return static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::microseconds>(
                                     std::chrono::steady_clock::now().time_since_epoch())
                                     .count());
}

// Device scratch shared by every decode path of one handle.
struct Scratch {
    DevBuf<float> osd_llr;
    DevBuf<int> osd_index;
    DevBuf<int> counters;  // [0] osd count, [1] BP work counter, [2] OSD work counter
    DevBuf<uint8_t> success, used_osd, iterations, bits;
    void alloc(int cap, int n, int bits_per_cw)
    {
        osd_llr.alloc(static_cast<size_t>(cap) * n);
        osd_index.alloc(static_cast<size_t>(cap));
        counters.alloc(3);
        success.alloc(cap);
        used_osd.alloc(cap);
        iterations.alloc(cap);
        bits.alloc(static_cast<size_t>(cap) * bits_per_cw);
    }
};

// Optional per-kernel timing: CUDA events recorded on the launching stream
// around the BP and OSD kernels of every decode call since the last query, so
// a timed loop needs no synchronisation between calls.
struct KernelTiming {
    struct Rec {
        cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
        int* h_osd = nullptr;  // pinned copy of the OSD work-list length
    };
    bool enabled = false;
    std::vector<Rec> pool;
    size_t used = 0;
    ~KernelTiming()
    {
        for (auto& r : pool) {
            for (auto& e : r.ev)
                if (e) cudaEventDestroy(e);
            if (r.h_osd) cudaFreeHost(r.h_osd);
        }
    }
    Rec& next()
    {
        if (used == pool.size()) {
            Rec r;
            for (auto& e : r.ev) check_cuda(cudaEventCreate(&e), "cudaEventCreate(timing)");
            check_cuda(cudaMallocHost(&r.h_osd, sizeof(int)), "cudaMallocHost(timing)");
            pool.push_back(r);
        }
        return pool[used++];
    }
};

// Runs BP (and optionally OSD on the routed codewords) for `count` device LLRs.
void run_bp_osd(const DeviceCode& code, const BpParams& bp, const BpLaunch& shape, bool with_osd,
                const float* d_llr, int count, uint8_t* d_bits, int out_len, int out_stride, uint8_t* d_success,
                uint8_t* d_used_osd, uint8_t* d_iter, float* d_app, Scratch& s, cudaStream_t st,
                KernelTiming* tm = nullptr)
{
    KernelTiming::Rec* rec = (tm && tm->enabled) ? &tm->next() : nullptr;
    BpIO io{};
    io.llr = d_llr;
    io.count = count;
    io.out_bits = d_bits;
    io.out_len = out_len;
    io.out_stride = out_stride;
    io.success = d_success;
    io.iterations = d_iter;
    io.app_out = d_app;
    io.used_osd = d_used_osd;
    io.work_counter = s.counters.p + 1;
    BpParams p = bp;
    p.route_failures_to_osd = with_osd ? 1 : 0;
    if (with_osd) {
        io.osd_llr = s.osd_llr.p;
        io.osd_index = s.osd_index.p;
        io.osd_count = s.counters.p;
        check_cuda(cudaMemsetAsync(s.counters.p, 0, sizeof(int), st), "reset osd count");
    }
    if (rec) check_cuda(cudaEventRecord(rec->ev[0], st), "cudaEventRecord");
    if (code.layered()) launch_bp_layered(code.layered_view(), p, io, shape, st);
    else launch_bp_flooding(code.flood_view(), p, io, st);
    if (rec) check_cuda(cudaEventRecord(rec->ev[1], st), "cudaEventRecord");
    if (with_osd) {
        OsdIO oio{};
        oio.llr = s.osd_llr.p;
        oio.index = s.osd_index.p;
        oio.count_ptr = s.counters.p;
        oio.count = 0;
        oio.out_info = d_bits;
        oio.info_stride = out_stride;
        oio.used_osd = d_used_osd;
        oio.share_rounds = shape.osd_share_rounds;
        oio.work = s.counters.p + 2;
        launch_osd(code.osd_view(), oio, count, st, 0, shape.osd_ctas);
    }
    if (rec) {
        check_cuda(cudaEventRecord(rec->ev[2], st), "cudaEventRecord");
        if (with_osd)
            check_cuda(cudaMemcpyAsync(rec->h_osd, s.counters.p, sizeof(int), cudaMemcpyDeviceToHost, st),
                       "copy osd count");
        else
            *rec->h_osd = 0;
        check_cuda(cudaEventRecord(rec->ev[3], st), "cudaEventRecord");
    }
}

// ---------------------------------------------------------------------------
// decoder objects
// ---------------------------------------------------------------------------

struct Decoder {
    enum Kind { kStream, kOsd, kCsr } kind;
    int device = 0;
    int n = 0, k = 0, m = 0;
    int max_batch = 1;
    std::unique_ptr<DeviceCode> code;
    OsdSettings osd;
    bool osd_enabled = true;
    BpParams bp{};
    BpLaunch shape{};
    std::vector<int> h_row_ptr, h_col_ind;  // host copy of H for rebuilding the tables
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    Scratch scratch;
    KernelTiming timing;
    std::mutex mu;
    virtual ~Decoder()
    {
        if (stream) cudaStreamDestroy(stream);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
    }
    void init_common()
    {
        check_cuda(cudaGetDevice(&device), "cudaGetDevice");
        check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        check_cuda(cudaEventCreate(&ev0), "cudaEventCreate");
        check_cuda(cudaEventCreate(&ev1), "cudaEventCreate");
    }
};

// Stream decoder: codewords queue in a filling batch on the device; batches
// launch by size or age and complete asynchronously into a host ready queue.
struct StreamDecoder : Decoder {
    cuda_osd_stream_config_t cfg{};
    struct Batch {
        DevBuf<float> llr;
        DevBuf<uint8_t> info, used_osd, success;
        HostBuf<uint8_t> h_info, h_used_osd, h_success;
        std::vector<unsigned long long> ts, ids;
        std::vector<unsigned> blocks;
        int count = 0;
        uint64_t first_arrival_us = 0;  // decoder clock when the batch took its first codeword
        bool in_flight = false;
        bool held = false;  // retired: its results wait in the ready queue, read in place
        cudaEvent_t done = nullptr;
        cudaEvent_t start = nullptr;
        ~Batch()
        {
            if (done) cudaEventDestroy(done);
            if (start) cudaEventDestroy(start);
        }
    };
    // Ring of batches: two can decode while the caller fills the next one and still holds
    // the results of the one before.
    static constexpr int kRing = 4;
    std::vector<std::unique_ptr<Batch>> batches;
    int filling = 0;
    bool claimed = true;  // batches[filling] is free for new codewords
    std::deque<int> flight;  // batch ids in launch order
    // Results of retired batches, handed out by poll in ranges: read in place from the
    // batch's pinned host buffers (batch >= 0), or from copies when the ring needed the
    // batch again before the caller polled it (batch < 0).
    struct ReadySeg {
        int batch = -1;
        size_t count = 0;
        std::vector<uint8_t> info, used;
        std::vector<unsigned long long> ts, ids;
        std::vector<unsigned> blocks;
        size_t pos = 0;
    };
    std::deque<ReadySeg> ready;
    // Submitted LLRs are copied on their own stream, so a submit returns once its copy is
    // done (the caller's buffer is free) while earlier batches keep decoding.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copied = nullptr;

    ~StreamDecoder() override
    {
        if (copy_stream) {
            cudaStreamSynchronize(copy_stream);
            cudaStreamDestroy(copy_stream);
        }
        if (copied) cudaEventDestroy(copied);
    }
    bool draining = false;
    cuda_osd_stream_stats_t stats{};
    uint64_t last_arrival_us = 0;

    void setup(const cuda_osd_stream_config_t& c, const std::vector<int>& rp, const std::vector<int>& ci,
               const uint64_t* parity, int parity_words)
    {
        cfg = c;
        n = c.n;
        k = c.k;
        m = c.m;
        max_batch = std::max(1, c.max_batch_size);
        init_common();
        osd.order = 2;
        osd.max_flip_positions = std::min(k, 64);
        osd.max_tests = 4096;
        h_row_ptr = rp;
        h_col_ind = ci;
        code = std::make_unique<DeviceCode>(n, m, rp.data(), ci.data(), kFlatLayered, parity, parity_words, true, osd);
        if (code->k() != k) throw InvalidArgument("k does not match n - m of the parity-check matrix");
        bp.alpha = c.bp_normalization;
        bp.beta = c.bp_offset;
        bp.damping = c.bp_damping;
        bp.min_abs_accept = c.bp_min_abs_llr_accept;
        bp.max_iter = c.bp_max_iterations;
        scratch.alloc(max_batch, n, k);
        check_cuda(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "cudaStreamCreate(copy)");
        check_cuda(cudaEventCreateWithFlags(&copied, cudaEventDisableTiming), "cudaEventCreate(copy)");
        for (int i = 0; i < kRing; ++i) {
            auto b = std::make_unique<Batch>();
            b->llr.alloc(static_cast<size_t>(max_batch) * n);
            b->info.alloc(static_cast<size_t>(max_batch) * k);
            b->used_osd.alloc(max_batch);
            b->success.alloc(max_batch);
            b->h_info.alloc(static_cast<size_t>(max_batch) * k);
            b->h_used_osd.alloc(max_batch);
            b->h_success.alloc(max_batch);
            check_cuda(cudaEventCreate(&b->done), "cudaEventCreate");
            check_cuda(cudaEventCreate(&b->start), "cudaEventCreate");
            b->ts.reserve(max_batch);
            b->ids.reserve(max_batch);
            b->blocks.reserve(max_batch);
            batches.push_back(std::move(b));
        }
        stats.ewma_interarrival_us = static_cast<double>(c.default_interarrival_us);
    }

    void launch_filling()
    {
        if (!claimed) return;
        Batch& b = *batches[filling];
        if (b.count == 0) return;
        check_cuda(cudaEventRecord(copied, copy_stream), "cudaEventRecord(copy)");
        check_cuda(cudaStreamWaitEvent(stream, copied, 0), "cudaStreamWaitEvent(copy)");
        check_cuda(cudaEventRecord(b.start, stream), "cudaEventRecord");
        run_bp_osd(*code, bp, shape, osd_enabled, b.llr.p, b.count, b.info.p, k, k, b.success.p, b.used_osd.p,
                   nullptr, nullptr, scratch, stream, &timing);
        check_cuda(cudaMemcpyAsync(b.h_info.p, b.info.p, static_cast<size_t>(b.count) * k, cudaMemcpyDeviceToHost,
                                   stream),
                   "copy info bits");
        check_cuda(cudaMemcpyAsync(b.h_used_osd.p, b.used_osd.p, b.count, cudaMemcpyDeviceToHost, stream),
                   "copy used_osd");
        check_cuda(cudaMemcpyAsync(b.h_success.p, b.success.p, b.count, cudaMemcpyDeviceToHost, stream),
                   "copy success");
        check_cuda(cudaEventRecord(b.done, stream), "cudaEventRecord");
        b.in_flight = true;
        flight.push_back(filling);
        stats.decoded_batches += 1;
        // the next batch to fill; claimed by the next submit (by then the caller has usually
        // polled its previous results)
        filling = (filling + 1) % static_cast<int>(batches.size());
        claimed = !(batches[filling]->in_flight || batches[filling]->held);
    }

    // Frees batches[filling] for new codewords: waits for it if it is still decoding, copies
    // its results out if the caller has not polled them yet.
    void claim()
    {
        if (claimed) return;
        if (batches[filling]->in_flight) collect_until(filling);
        if (batches[filling]->held) spill(filling);
        claimed = true;
    }

    void release(Batch& b)
    {
        b.count = 0;
        b.held = false;
        b.ts.clear();  // capacity kept
        b.ids.clear();
        b.blocks.clear();
    }

    // Copies the unpolled results of held batch `id` into its ready segment and frees the batch.
    void spill(int id)
    {
        Batch& b = *batches[id];
        for (auto& sg : ready) {
            if (sg.batch != id) continue;
            sg.info.assign(b.h_info.p, b.h_info.p + static_cast<size_t>(b.count) * k);
            sg.used.assign(b.h_used_osd.p, b.h_used_osd.p + b.count);
            sg.ts = b.ts;
            sg.ids = b.ids;
            sg.blocks = b.blocks;
            sg.batch = -1;
        }
        release(b);
    }

    // Moves the front in-flight batch to the ready queue.
    void retire_front()
    {
        const int id = flight.front();
        Batch& b = *batches[id];
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, b.start, b.done);
        stats.total_decode_ms += ms;
        ReadySeg sg;
        sg.batch = id;
        sg.count = static_cast<size_t>(b.count);
        for (int i = 0; i < b.count; ++i) {
            stats.osd_fallback_codewords += b.h_used_osd.p[i] ? 1 : 0;
            stats.bp_success_codewords += b.h_success.p[i] ? 1 : 0;
        }
        ready.push_back(std::move(sg));
        stats.decoded_codewords += static_cast<unsigned long long>(b.count);
        stats.average_batch_size = static_cast<double>(stats.decoded_codewords) /
                                   static_cast<double>(std::max<unsigned long long>(stats.decoded_batches, 1));
        b.in_flight = false;
        b.held = true;
        flight.pop_front();
    }

    // Retires every completed batch; with wait_one, first waits for the oldest.
    void collect(bool wait_one)
    {
        while (!flight.empty()) {
            Batch& b = *batches[flight.front()];
            if (wait_one) {
                check_cuda(cudaEventSynchronize(b.done), "cudaEventSynchronize");
                wait_one = false;
            } else {
                const cudaError_t q = cudaEventQuery(b.done);
                if (q == cudaErrorNotReady) break;
                check_cuda(q, "cudaEventQuery");
            }
            retire_front();
        }
    }

    // Waits until batch `id` is no longer in flight (batches complete in order).
    void collect_until(int id)
    {
        while (batches[id]->in_flight) {
            check_cuda(cudaEventSynchronize(batches[flight.front()]->done), "cudaEventSynchronize");
            retire_front();
        }
    }

    unsigned long long pending() const
    {
        return claimed ? static_cast<unsigned long long>(batches[filling]->count) : 0ull;
    }

    void maybe_launch()
    {
        if (!claimed) return;
        Batch& b = *batches[filling];
        if (b.count <= 0) return;
        // the latency budget runs from the batch's first arrival at this decoder (not from the
        // caller's timestamps, which may count on another clock)
        const uint64_t now = now_us();
        const uint64_t age = now > b.first_arrival_us ? now - b.first_arrival_us : 0;
        if (b.count >= std::max(1, cfg.min_batch_size) || b.count >= max_batch ||
            age >= std::max<unsigned long long>(cfg.max_latency_us, 1))
            launch_filling();
    }

    void submit(const float* llrs, bool device_ptr, int count, const unsigned long long* ts,
                const unsigned long long* ids, const unsigned* blocks)
    {
        int done = 0;
        const uint64_t now = now_us();
        if (last_arrival_us != 0) {
            const double a = cfg.arrival_ewma_alpha > 0 ? cfg.arrival_ewma_alpha : 0.15;
            stats.ewma_interarrival_us = (1.0 - a) * stats.ewma_interarrival_us +
                                         a * static_cast<double>(now - last_arrival_us) / std::max(count, 1);
        }
        last_arrival_us = now;
        while (done < count) {
            claim();
            Batch& b = *batches[filling];
            const int take = std::min(count - done, max_batch - b.count);
            if (b.count == 0) b.first_arrival_us = now;
            const size_t bytes = static_cast<size_t>(take) * n * sizeof(float);
            check_cuda(cudaMemcpyAsync(b.llr.p + static_cast<size_t>(b.count) * n,
                                       llrs + static_cast<size_t>(done) * n, bytes,
                                       device_ptr ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, copy_stream),
                       "copy submitted LLRs");
            if (ts) b.ts.insert(b.ts.end(), ts + done, ts + done + take);
            else b.ts.insert(b.ts.end(), static_cast<size_t>(take), now);
            if (ids) b.ids.insert(b.ids.end(), ids + done, ids + done + take);
            else b.ids.insert(b.ids.end(), static_cast<size_t>(take), 0ull);
            if (blocks) {
                b.blocks.insert(b.blocks.end(), blocks + done, blocks + done + take);
            } else {
                for (int i = 0; i < take; ++i) b.blocks.push_back(static_cast<unsigned>(done + i));
            }
            b.count += take;
            done += take;
            stats.submitted_codewords += static_cast<unsigned long long>(take);
            if (b.count >= max_batch) launch_filling();
        }
        // the caller may reuse its buffer as soon as this returns
        check_cuda(cudaEventRecord(copied, copy_stream), "cudaEventRecord(copy)");
        check_cuda(cudaEventSynchronize(copied), "synchronize submit copy");
        stats.last_submit_timestamp_us = ts && count > 0 ? ts[count - 1] : now;
        stats.current_pending_codewords = pending();
        stats.max_pending_codewords = std::max(stats.max_pending_codewords, stats.current_pending_codewords);
        maybe_launch();
    }

    int poll(int max_cw, unsigned char* out_info, unsigned long long* out_ts, unsigned long long* out_ids,
             unsigned* out_blocks, unsigned char* out_used)
    {
        collect(false);
        if (ready.empty()) {
            maybe_launch();
            collect(false);
        }
        if (ready.empty() && draining) {
            if (pending() > 0) launch_filling();
            if (!flight.empty()) collect(true);
        }
        int out = 0;
        while (out < max_cw && !ready.empty()) {
            ReadySeg& sg = ready.front();
            Batch* b = sg.batch >= 0 ? batches[sg.batch].get() : nullptr;
            const uint8_t* info = b ? b->h_info.p : sg.info.data();
            const uint8_t* used = b ? b->h_used_osd.p : sg.used.data();
            const unsigned long long* ts = b ? b->ts.data() : sg.ts.data();
            const unsigned long long* ids = b ? b->ids.data() : sg.ids.data();
            const unsigned* blocks = b ? b->blocks.data() : sg.blocks.data();
            const size_t take = std::min<size_t>(sg.count - sg.pos, static_cast<size_t>(max_cw - out));
            if (out_info) std::memcpy(out_info + static_cast<size_t>(out) * k, info + sg.pos * k, take * k);
            if (out_ts) std::memcpy(out_ts + out, ts + sg.pos, take * sizeof(*ts));
            if (out_ids) std::memcpy(out_ids + out, ids + sg.pos, take * sizeof(*ids));
            if (out_blocks) std::memcpy(out_blocks + out, blocks + sg.pos, take * sizeof(*blocks));
            if (out_used) std::memcpy(out_used + out, used + sg.pos, take);
            sg.pos += take;
            out += static_cast<int>(take);
            if (sg.pos == sg.count) {
                if (b) release(*b);
                ready.pop_front();
            }
        }
        if (ready.empty() && flight.empty() && pending() == 0) draining = false;
        stats.current_pending_codewords = pending();
        return out;
    }

    void flush()
    {
        draining = true;
        if (pending() > 0) launch_filling();
    }
};

struct OsdDecoder : Decoder {
    DevBuf<float> llr;
    DevBuf<uint8_t> info;
    DevBuf<float> dist;
    void setup(const cuda_osd_osd_config_t& c, const std::vector<int>& rp, const std::vector<int>& ci)
    {
        n = c.n;
        k = c.k;
        m = n - k;
        max_batch = std::max(1, c.max_batch_size);
        init_common();
        osd.order = 2;
        osd.max_flip_positions = std::min(k, 64);
        osd.max_tests = 4096;
        code = std::make_unique<DeviceCode>(n, m, rp.data(), ci.data(), kFlatLayered, nullptr, 0, true, osd);
        llr.alloc(static_cast<size_t>(max_batch) * n);
        info.alloc(static_cast<size_t>(max_batch) * k);
        dist.alloc(max_batch);
    }
};

struct CsrDecoder : Decoder {
    DevBuf<float> llr;
    DevBuf<uint8_t> bits, success;
    void setup(const cuda_osd_bp_csr_config_t& c, const int* rp, const int* ci)
    {
        n = c.n;
        m = c.m;
        k = n - m;
        max_batch = std::max(1, c.max_batch_size);
        init_common();
        h_row_ptr.assign(rp, rp + m + 1);
        h_col_ind.assign(ci, ci + rp[m]);
        code = std::make_unique<DeviceCode>(n, m, rp, ci, c.schedule, nullptr, 0, false, osd);
        bp.alpha = c.normalization;
        bp.beta = c.offset;
        bp.damping = c.damping;
        bp.min_abs_accept = c.min_abs_llr_accept;
        bp.max_iter = c.max_iterations;
        scratch.alloc(1, n, 1);
        llr.alloc(static_cast<size_t>(max_batch) * n);
        bits.alloc(static_cast<size_t>(max_batch) * n);
        success.alloc(max_batch);
    }
};

// ---- launch shapes (include/sicc_tune.h) ----

uint64_t decoder_fingerprint(const Decoder& d)
{
    Fingerprint f;
    f.add(static_cast<int>(d.kind));
    f.add(d.n);
    f.add(d.m);
    f.add(d.h_row_ptr.data(), d.h_row_ptr.size());
    f.add(d.h_col_ind.data(), d.h_col_ind.size());
    f.add(d.code->schedule());
    f.add(d.bp.max_iter);
    f.add_float(d.bp.alpha);
    f.add_float(d.bp.beta);
    if (d.kind == Decoder::kStream) {
        f.add(d.osd_enabled ? 1 : 0);
        f.add(d.osd.order);
        f.add(d.osd.max_flip_positions);
        f.add(d.osd.max_tests);
    }
    return f.h;
}

// Lanes per codeword the layered tables get by default: the smallest power of two
// covering the widest layer, at most 32.
int default_layered_group(const Decoder& d)
{
    std::vector<int> order, sizes;
    if (d.code->schedule() == kColoredLayered)
        greedy_coloring(d.n, d.m, d.h_row_ptr.data(), d.h_col_ind.data(), order, sizes);
    else
        consecutive_layers(d.n, d.m, d.h_row_ptr.data(), d.h_col_ind.data(), sizes);
    int maxw = 1;
    for (int x : sizes) maxw = std::max(maxw, x);
    int g = 1;
    while (g < maxw && g < 32) g <<= 1;
    return g;
}

sicc_fec_shape_t current_shape(const Decoder& d)
{
    sicc_fec_shape_t s{};
    s.lanes_per_codeword = d.code->layered_group_request();
    s.slots_per_cta = d.shape.slots_per_cta;
    s.ctas = d.shape.ctas;
    s.osd_share_rounds = d.shape.osd_share_rounds;
    s.osd_ctas = d.shape.osd_ctas;
    return s;
}

// Rebuilds the decoder's code tables with `group` lanes per codeword (same schedule,
// parity table and OSD settings).  The caller holds d.mu and has drained d.stream.
void rebuild_code(Decoder& d, int group)
{
    if (group == d.code->layered_group_request()) return;
    const auto parity = d.code->parity_table();
    const bool need_osd = d.kind == Decoder::kStream;
    auto fresh = std::make_unique<DeviceCode>(d.n, d.m, d.h_row_ptr.data(), d.h_col_ind.data(), d.code->schedule(),
                                              parity.empty() ? nullptr : parity.data(), d.code->parity_words(),
                                              need_osd, d.osd, group);
    d.code = std::move(fresh);
}

void check_shape(const Decoder& d, const sicc_fec_shape_t& s)
{
    const int g = s.lanes_per_codeword;
    if (g < 0 || g > 32 || (g & (g - 1)) != 0)
        throw InvalidArgument("lanes_per_codeword must be 0 or a power of two <= 32");
    if (s.slots_per_cta < 0 || s.ctas < 0 || s.osd_ctas < 0 || s.osd_share_rounds < 0 || s.osd_share_rounds > 64)
        throw InvalidArgument("launch shape fields must be >= 0 (osd_share_rounds <= 64)");
    if (s.slots_per_cta > 0 && d.code->layered()) {
        const int eff = g > 0 ? std::min(g, default_layered_group(d)) : default_layered_group(d);
        if (s.slots_per_cta % std::max(1, 32 / eff) != 0 || s.slots_per_cta * eff > kBpThreads)
            throw InvalidArgument("slots_per_cta must be a multiple of 32 / lanes and slots x lanes <= 256");
    }
}

// The caller holds d.mu and has drained d.stream.
void apply_shape(Decoder& d, const sicc_fec_shape_t& s)
{
    check_shape(d, s);
    if (d.code->layered()) rebuild_code(d, s.lanes_per_codeword);
    d.shape.slots_per_cta = s.slots_per_cta;
    d.shape.ctas = s.ctas;
    d.shape.osd_share_rounds = s.osd_share_rounds;
    d.shape.osd_ctas = s.osd_ctas;
}

// Decoders start from the shape tuned for their code on this device, if any.
void apply_cached_shape(Decoder& d)
{
    std::vector<int> v;
    if (!tune_cache_get(tune_key("fec", decoder_fingerprint(d)), v) || v.size() != 5) return;
    const sicc_fec_shape_t s{v[0], v[1], v[2], v[3], v[4]};
    try {
        apply_shape(d, s);
    } catch (const InvalidArgument&) {
        // a stale or hand-edited entry: keep the defaults
    }
}

std::mutex g_registry_mu;
std::map<unsigned long long, std::shared_ptr<Decoder>> g_registry;
unsigned long long g_next_handle = 0x5100;

unsigned long long register_decoder(std::shared_ptr<Decoder> d)
{
    std::lock_guard<std::mutex> lock(g_registry_mu);
    const unsigned long long h = ++g_next_handle;
    g_registry[h] = std::move(d);
    return h;
}

template <class T>
std::shared_ptr<T> lookup(unsigned long long h, Decoder::Kind kind)
{
    std::lock_guard<std::mutex> lock(g_registry_mu);
    auto it = g_registry.find(h);
    if (it == g_registry.end() || it->second->kind != kind) throw InvalidArgument("invalid decoder handle");
    return std::static_pointer_cast<T>(it->second);
}

std::shared_ptr<Decoder> lookup_any(unsigned long long h)
{
    std::lock_guard<std::mutex> lock(g_registry_mu);
    auto it = g_registry.find(h);
    if (it == g_registry.end()) throw InvalidArgument("invalid decoder handle");
    return it->second;
}

int destroy(unsigned long long h, Decoder::Kind kind)
{
    std::shared_ptr<Decoder> d;
    {
        std::lock_guard<std::mutex> lock(g_registry_mu);
        auto it = g_registry.find(h);
        if (it == g_registry.end() || it->second->kind != kind) throw InvalidArgument("invalid decoder handle");
        d = it->second;
        g_registry.erase(it);
    }
    cudaSetDevice(d->device);
    if (d->stream) cudaStreamSynchronize(d->stream);
    return CUDA_OSD_STATUS_OK;
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
    } catch (...) {
        set_last_error("unknown error");
        return CUDA_OSD_STATUS_INTERNAL_ERROR;
    }
}

void require(bool ok, const char* msg)
{
    if (!ok) throw InvalidArgument(msg);
}

void validate_stream_config(const cuda_osd_stream_config_t* c)
{
    require(c != nullptr, "config is null");
    require(c->n > 0 && c->k > 0 && c->m > 0 && c->k + c->m == c->n, "stream decoder needs n = k + m > 0");
    require(c->n <= 256 && c->k <= 128 && c->n - c->k <= 128,
            "stream BP-OSD supports n <= 256, k <= 128, n-k <= 128");
    require(c->max_batch_size > 0, "max_batch_size must be positive");
    require(c->min_batch_size >= 0 && c->min_batch_size <= c->max_batch_size, "min_batch_size out of range");
    require(c->bp_max_iterations >= 1 && c->bp_max_iterations <= 255, "bp_max_iterations must be 1..255");
    require(c->bp_damping >= 0.0f && c->bp_damping < 1.0f, "bp_damping must be in [0,1)");
}

}  // namespace

// Decodes with a stream decoder's code tables and settings, but with the
// BP -> OSD hand-off scratch supplied by the caller (used by the entry point
// whose scratch is a static device array).  Layout of `scratch`:
// [0, 256) the counters (OSD items, BP work, OSD work); [256, 256 + 4*cap) OSD index list;
// then cap rows of n floats (256-byte aligned).
int decode_with_caller_scratch(unsigned long long handle, const float* d_llr, int count, uint8_t* d_info,
                               uint8_t* d_success, uint8_t* d_used_osd, uint8_t* d_iter,
                               unsigned char* (*scratch_on_current_device)(), int cap, cudaStream_t st)
{
    auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
    std::lock_guard<std::mutex> lock(d->mu);
    require(count > 0 && count <= cap, "codewords must be in 1..the static scratch capacity");
    require(d->n <= 256, "the static scratch holds codes with n <= 256");
    check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
    unsigned char* scratch = scratch_on_current_device();
    int* counters = reinterpret_cast<int*>(scratch);
    int* index = reinterpret_cast<int*>(scratch + 256);
    float* rows = reinterpret_cast<float*>(scratch + 256 + ((static_cast<size_t>(cap) * 4 + 255) & ~size_t(255)));
    BpIO io{};
    io.llr = d_llr;
    io.count = count;
    io.out_bits = d_info;
    io.out_len = d->k;
    io.out_stride = d->k;
    io.success = d_success;
    io.iterations = d_iter;
    io.used_osd = d_used_osd;
    io.work_counter = counters + 1;
    BpParams p = d->bp;
    p.route_failures_to_osd = d->osd_enabled ? 1 : 0;
    // both counters start at zero on every call: the array keeps the previous call's contents
    check_cuda(cudaMemsetAsync(counters, 0, 2 * sizeof(int), st), "clear static scratch counters");
    if (d->osd_enabled) {
        io.osd_llr = rows;
        io.osd_index = index;
        io.osd_count = counters;
    }
    if (d->code->layered()) launch_bp_layered(d->code->layered_view(), p, io, d->shape, st);
    else launch_bp_flooding(d->code->flood_view(), p, io, st);
    if (d->osd_enabled) {
        OsdIO oio{};
        oio.llr = rows;
        oio.index = index;
        oio.count_ptr = counters;
        oio.out_info = d_info;
        oio.info_stride = d->k;
        oio.used_osd = d_used_osd;
        oio.share_rounds = d->shape.osd_share_rounds;
        oio.work = counters + 2;  // inside the counters' 256 bytes
        launch_osd(d->code->osd_view(), oio, count, st, 0, d->shape.osd_ctas);
    }
    return CUDA_OSD_STATUS_OK;
}

}  // namespace sicc

using namespace sicc;

extern "C" {

const char* cuda_osd_get_last_error(void) { return sicc::last_error(); }

int cuda_osd_create_stream_decoder(const cuda_osd_stream_config_t* config, unsigned long long* out_handle)
{
    return guarded([&] {
        require(out_handle != nullptr, "out_handle is null");
        *out_handle = 0;
        validate_stream_config(config);
        require(config->n == 128 && config->k == 64 && config->m == 64,
                "the built-in code is CCSDS (128,64); use cuda_osd_create_stream_decoder_with_matrices");
        std::vector<int> rp, ci;
        ccsds_128_64(rp, ci);
        auto d = std::make_shared<StreamDecoder>();
        d->kind = Decoder::kStream;
        d->setup(*config, rp, ci, nullptr, 0);
        apply_cached_shape(*d);
        *out_handle = register_decoder(d);
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_create_stream_decoder_with_matrices(const cuda_osd_stream_config_t* config, const unsigned char* dense_h,
                                                 const unsigned long long* systematic_parity, int parity_words_per_row,
                                                 unsigned long long* out_handle)
{
    return guarded([&] {
        require(out_handle != nullptr, "out_handle is null");
        *out_handle = 0;
        validate_stream_config(config);
        require(dense_h != nullptr && systematic_parity != nullptr, "matrices are null");
        std::vector<int> rp, ci;
        csr_from_dense(dense_h, config->m, config->n, rp, ci);
        auto d = std::make_shared<StreamDecoder>();
        d->kind = Decoder::kStream;
        d->setup(*config, rp, ci, reinterpret_cast<const uint64_t*>(systematic_parity), parity_words_per_row);
        apply_cached_shape(*d);
        *out_handle = register_decoder(d);
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_destroy_stream_decoder(unsigned long long handle)
{
    return guarded([&] { return destroy(handle, Decoder::kStream); });
}

int cuda_osd_create_osd_decoder(const cuda_osd_osd_config_t* config, unsigned long long* out_handle)
{
    return guarded([&] {
        require(out_handle != nullptr, "out_handle is null");
        *out_handle = 0;
        require(config != nullptr, "config is null");
        require(config->n == 128 && config->k == 64,
                "the OSD-only decoder uses the built-in CCSDS (128,64) code (n=128, k=64)");
        require(config->max_batch_size > 0, "max_batch_size must be positive");
        std::vector<int> rp, ci;
        ccsds_128_64(rp, ci);
        auto d = std::make_shared<OsdDecoder>();
        d->kind = Decoder::kOsd;
        d->setup(*config, rp, ci);
        *out_handle = register_decoder(d);
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_destroy_osd_decoder(unsigned long long handle)
{
    return guarded([&] { return destroy(handle, Decoder::kOsd); });
}

int cuda_osd_create_bp_csr_decoder(const cuda_osd_bp_csr_config_t* config, const int* row_ptr, const int* col_ind,
                                   unsigned long long* out_handle)
{
    return guarded([&] {
        require(out_handle != nullptr, "out_handle is null");
        *out_handle = 0;
        require(config != nullptr && row_ptr != nullptr && col_ind != nullptr, "null argument");
        require(config->n > 0 && config->m > 0 && config->m < config->n, "need 0 < m < n");
        require(config->max_batch_size > 0, "max_batch_size must be positive");
        require(config->max_iterations >= 1 && config->max_iterations <= 255, "max_iterations must be 1..255");
        require(row_ptr[0] == 0 && row_ptr[config->m] == config->nnz, "row_ptr must start at 0 and end at nnz");
        require(config->damping >= 0.0f && config->damping < 1.0f, "damping must be in [0,1)");
        auto d = std::make_shared<CsrDecoder>();
        d->kind = Decoder::kCsr;
        d->setup(*config, row_ptr, col_ind);
        apply_cached_shape(*d);
        *out_handle = register_decoder(d);
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_destroy_bp_csr_decoder(unsigned long long handle)
{
    return guarded([&] { return destroy(handle, Decoder::kCsr); });
}

static int csr_decode(unsigned long long handle, const float* llrs, bool device_in, int codewords,
                      unsigned char* out_code_bits, unsigned char* out_success, double* out_ms)
{
    return guarded([&] {
        auto d = lookup<CsrDecoder>(handle, Decoder::kCsr);
        std::lock_guard<std::mutex> lock(d->mu);
        require(llrs != nullptr && codewords > 0, "empty batch");
        require(out_code_bits != nullptr, "out_code_bits is null");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        check_cuda(cudaEventRecord(d->ev0, d->stream), "cudaEventRecord");
        for (int off = 0; off < codewords; off += d->max_batch) {
            const int cnt = std::min(d->max_batch, codewords - off);
            const float* src = llrs + static_cast<size_t>(off) * d->n;
            if (!device_in) {
                check_cuda(cudaMemcpyAsync(d->llr.p, src, static_cast<size_t>(cnt) * d->n * sizeof(float),
                                           cudaMemcpyHostToDevice, d->stream),
                           "copy LLRs");
                src = d->llr.p;
            }
            run_bp_osd(*d->code, d->bp, d->shape, false, src, cnt, d->bits.p, d->n, d->n, d->success.p, nullptr,
                       nullptr, nullptr, d->scratch, d->stream);
            check_cuda(cudaMemcpyAsync(out_code_bits + static_cast<size_t>(off) * d->n, d->bits.p,
                                       static_cast<size_t>(cnt) * d->n, cudaMemcpyDeviceToHost, d->stream),
                       "copy code bits");
            if (out_success)
                check_cuda(cudaMemcpyAsync(out_success + off, d->success.p, cnt, cudaMemcpyDeviceToHost, d->stream),
                           "copy success");
            check_cuda(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
        }
        check_cuda(cudaEventRecord(d->ev1, d->stream), "cudaEventRecord");
        check_cuda(cudaEventSynchronize(d->ev1), "cudaEventSynchronize");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, d->ev0, d->ev1);
        if (out_ms) *out_ms = ms;
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_decode_bp_csr_batch(unsigned long long handle, const float* llrs, int codewords,
                                 unsigned char* out_code_bits, unsigned char* out_success, double* out_total_decode_ms)
{
    return csr_decode(handle, llrs, false, codewords, out_code_bits, out_success, out_total_decode_ms);
}

int cuda_osd_decode_bp_csr_device_batch(unsigned long long handle, const float* device_llrs, int codewords,
                                        unsigned char* out_code_bits, unsigned char* out_success,
                                        double* out_total_decode_ms)
{
    return csr_decode(handle, device_llrs, true, codewords, out_code_bits, out_success, out_total_decode_ms);
}

int cuda_osd_decode_osd_batch(unsigned long long handle, const float* llrs, int codewords,
                              unsigned char* out_info_bits, float* out_distances, double* out_total_decode_ms,
                              double* out_throughput_mbps)
{
    return guarded([&] {
        auto d = lookup<OsdDecoder>(handle, Decoder::kOsd);
        std::lock_guard<std::mutex> lock(d->mu);
        require(llrs != nullptr && codewords > 0, "empty batch");
        require(out_info_bits != nullptr, "out_info_bits is null");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        check_cuda(cudaEventRecord(d->ev0, d->stream), "cudaEventRecord");
        for (int off = 0; off < codewords; off += d->max_batch) {
            const int cnt = std::min(d->max_batch, codewords - off);
            check_cuda(cudaMemcpyAsync(d->llr.p, llrs + static_cast<size_t>(off) * d->n,
                                       static_cast<size_t>(cnt) * d->n * sizeof(float), cudaMemcpyHostToDevice,
                                       d->stream),
                       "copy LLRs");
            OsdIO io{};
            io.llr = d->llr.p;
            io.count = cnt;
            io.out_info = d->info.p;
            io.info_stride = d->k;
            io.out_metric = d->dist.p;
            io.share_rounds = d->shape.osd_share_rounds;
            launch_osd(d->code->osd_view(), io, cnt, d->stream, 0, d->shape.osd_ctas);
            check_cuda(cudaMemcpyAsync(out_info_bits + static_cast<size_t>(off) * d->k, d->info.p,
                                       static_cast<size_t>(cnt) * d->k, cudaMemcpyDeviceToHost, d->stream),
                       "copy info bits");
            if (out_distances)
                check_cuda(cudaMemcpyAsync(out_distances + off, d->dist.p, cnt * sizeof(float), cudaMemcpyDeviceToHost,
                                           d->stream),
                           "copy distances");
            check_cuda(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
        }
        check_cuda(cudaEventRecord(d->ev1, d->stream), "cudaEventRecord");
        check_cuda(cudaEventSynchronize(d->ev1), "cudaEventSynchronize");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, d->ev0, d->ev1);
        if (out_total_decode_ms) *out_total_decode_ms = ms;
        if (out_throughput_mbps)
            *out_throughput_mbps = ms > 0.0f ? static_cast<double>(codewords) * d->k / (ms * 1e3) : 0.0;
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_submit_codewords(unsigned long long handle, const float* llrs, int codewords,
                              const unsigned long long* timestamps_us, const unsigned long long* frame_ids,
                              const unsigned int* block_indices)
{
    return guarded([&] {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        require(llrs != nullptr && codewords > 0, "empty submit");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        d->submit(llrs, false, codewords, timestamps_us, frame_ids, block_indices);
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_submit_device_codewords(unsigned long long handle, const float* device_llrs, int codewords,
                                     const unsigned long long* timestamps_us, const unsigned long long* frame_ids,
                                     const unsigned int* block_indices)
{
    return guarded([&] {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        require(device_llrs != nullptr && codewords > 0, "empty submit");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        d->submit(device_llrs, true, codewords, timestamps_us, frame_ids, block_indices);
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_poll_ready(unsigned long long handle, int max_codewords, unsigned char* out_info_bits,
                        unsigned long long* out_timestamps_us, unsigned long long* out_frame_ids,
                        unsigned int* out_block_indices, unsigned char* out_used_osd, int* out_codewords)
{
    return guarded([&] {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        require(out_codewords != nullptr, "out_codewords is null");
        *out_codewords = 0;
        require(max_codewords >= 0, "max_codewords must be >= 0");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        *out_codewords = d->poll(max_codewords, out_info_bits, out_timestamps_us, out_frame_ids, out_block_indices,
                                 out_used_osd);
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_flush(unsigned long long handle)
{
    return guarded([&] {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        d->flush();
        return CUDA_OSD_STATUS_OK;
    });
}

int cuda_osd_get_stats(unsigned long long handle, cuda_osd_stream_stats_t* out_stats)
{
    return guarded([&] {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        require(out_stats != nullptr, "out_stats is null");
        *out_stats = d->stats;
        return CUDA_OSD_STATUS_OK;
    });
}

unsigned long long cuda_osd_get_decoded_codewords(unsigned long long handle)
{
    try {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        return d->stats.decoded_codewords;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return 0;
    }
}

double cuda_osd_get_total_decode_ms(unsigned long long handle)
{
    try {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        return d->stats.total_decode_ms;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return 0.0;
    }
}

int sicc_fec_set_schedule(unsigned long long handle, int schedule)
{
    return guarded([&] {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        require(schedule >= 0 && schedule <= 3, "schedule must be 0..3");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        check_cuda(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
        const auto& parity = d->code->parity_table();
        auto fresh = std::make_unique<DeviceCode>(d->n, d->m, d->h_row_ptr.data(), d->h_col_ind.data(), schedule,
                                                  parity.data(), d->code->parity_words(), true, d->osd);
        d->code = std::move(fresh);
        apply_cached_shape(*d);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_fec_set_osd_params(unsigned long long handle, int order, int max_flip_positions, int max_tests)
{
    return guarded([&] {
        auto d = lookup_any(handle);
        std::lock_guard<std::mutex> lock(d->mu);
        require(d->kind != Decoder::kCsr, "CSR BP decoders have no OSD stage");
        require(order >= 0 && order <= 3 && max_flip_positions >= 0 && max_tests >= 1, "invalid OSD parameters");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        check_cuda(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
        d->osd.order = order;
        d->osd.max_flip_positions = max_flip_positions;
        d->osd.max_tests = max_tests;
        d->code->set_osd(d->osd);
        if (d->kind == Decoder::kStream) apply_cached_shape(*d);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_fec_set_osd_enabled(unsigned long long handle, int enabled)
{
    return guarded([&] {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        d->osd_enabled = enabled != 0;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_fec_set_launch_shape(unsigned long long handle, int slots_per_cta, int ctas)
{
    return guarded([&] {
        auto d = lookup_any(handle);
        std::lock_guard<std::mutex> lock(d->mu);
        require(slots_per_cta >= 0 && ctas >= 0, "launch shape must be >= 0");
        d->shape.slots_per_cta = slots_per_cta;
        d->shape.ctas = ctas;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_fec_get_shape(unsigned long long handle, sicc_fec_shape_t* out_shape)
{
    return guarded([&] {
        auto d = lookup_any(handle);
        std::lock_guard<std::mutex> lock(d->mu);
        require(out_shape != nullptr, "null argument");
        *out_shape = current_shape(*d);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_fec_set_shape(unsigned long long handle, const sicc_fec_shape_t* shape)
{
    return guarded([&] {
        auto d = lookup_any(handle);
        std::lock_guard<std::mutex> lock(d->mu);
        require(shape != nullptr, "null argument");
        require(d->kind != Decoder::kOsd, "OSD-only decoders have no BP shape");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        check_cuda(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
        apply_shape(*d, *shape);
        return CUDA_OSD_STATUS_OK;
    });
}

// Coordinate search: for each lanes-per-codeword candidate (the default group, half and a
// quarter of it), the slots per CTA with the default grid, then the grid with the best slots;
// then the OSD exchange interval and grid with the best BP shape.  Each trial is one warm-up
// decode and `reps` timed decodes of the caller's batch (median).
int sicc_fec_autotune(unsigned long long handle, const float* device_llrs, int codewords, int reps,
                      sicc_fec_shape_t* out_best, sicc_tune_trial_t* out_trials, int max_trials, int* out_trial_count)
{
    return guarded([&] {
        auto d = lookup_any(handle);
        std::lock_guard<std::mutex> lock(d->mu);
        require(d->kind != Decoder::kOsd, "OSD-only decoders have no BP shape to tune");
        require(device_llrs != nullptr && codewords > 0 && codewords <= d->max_batch,
                "codewords must be in 1..max_batch_size");
        require(reps >= 1 && reps <= 50, "reps must be in 1..50");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        check_cuda(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
        const bool stream_kind = d->kind == Decoder::kStream;
        const bool with_osd = stream_kind && d->osd_enabled;
        const int out_len = stream_kind ? d->k : d->n;
        DevBuf<uint8_t> bits, ok, used, iters;
        bits.alloc(static_cast<size_t>(codewords) * out_len);
        ok.alloc(codewords);
        used.alloc(codewords);
        iters.alloc(codewords);
        std::vector<sicc_tune_trial_t> trials;

        auto time_shape = [&](const sicc_fec_shape_t& sh) -> float {
            apply_shape(*d, sh);
            std::vector<float> ms;
            for (int r = 0; r <= reps; ++r) {
                check_cuda(cudaEventRecord(d->ev0, d->stream), "cudaEventRecord");
                run_bp_osd(*d->code, d->bp, d->shape, with_osd, device_llrs, codewords, bits.p, out_len, out_len,
                           ok.p, with_osd ? used.p : nullptr, iters.p, nullptr, d->scratch, d->stream, nullptr);
                check_cuda(cudaEventRecord(d->ev1, d->stream), "cudaEventRecord");
                check_cuda(cudaEventSynchronize(d->ev1), "cudaEventSynchronize");
                float t = 0.0f;
                check_cuda(cudaEventElapsedTime(&t, d->ev0, d->ev1), "cudaEventElapsedTime");
                if (r > 0) ms.push_back(t);  // the first decode is the warm-up
            }
            const float med = median_of(ms);
            trials.push_back(sicc_tune_trial_t{sh, med});
            return med;
        };

        sicc_fec_shape_t best{};
        float best_ms = time_shape(best);  // the library defaults
        auto consider = [&](const sicc_fec_shape_t& sh) {
            const float t = time_shape(sh);
            if (t < best_ms) {
                best_ms = t;
                best = sh;
            }
        };
        const int sms = device_sm_count();
        if (d->code->layered()) {
            const LayeredView& lv = d->code->layered_view();
            const bool wide = layered_needs_wide(lv, with_osd);
            if (!wide) {
                const int g0 = default_layered_group(*d);
                for (int g = g0; g >= std::max(1, g0 / 4); g >>= 1) {
                    sicc_fec_shape_t base{};
                    base.lanes_per_codeword = g == g0 ? 0 : g;
                    const int step = std::max(1, 32 / g);
                    sicc_fec_shape_t g_best = base;
                    float g_ms = g == g0 ? best_ms : time_shape(base);
                    if (g != g0 && g_ms < best_ms) {
                        best_ms = g_ms;
                        best = base;
                    }
                    for (int slots = step; slots * g <= kBpThreads; slots *= 2) {
                        sicc_fec_shape_t sh = base;
                        sh.slots_per_cta = slots;
                        const float t = time_shape(sh);
                        if (t < g_ms) {
                            g_ms = t;
                            g_best = sh;
                        }
                        if (t < best_ms) {
                            best_ms = t;
                            best = sh;
                        }
                    }
                    for (int per_sm : {1, 2, 4}) {
                        sicc_fec_shape_t sh = g_best;
                        sh.ctas = per_sm * sms;
                        consider(sh);
                    }
                }
            }
        }
        if (with_osd && d->code->has_osd()) {
            const sicc_fec_shape_t bp_best = best;
            for (int share : {1, 4, 8}) {
                sicc_fec_shape_t sh = bp_best;
                sh.osd_share_rounds = share;
                consider(sh);
            }
            const sicc_fec_shape_t osd_best = best;
            for (int per_sm : {1, 2}) {
                sicc_fec_shape_t sh = osd_best;
                sh.osd_ctas = per_sm * sms;
                consider(sh);
            }
        }
        apply_shape(*d, best);
        tune_cache_put(tune_key("fec", decoder_fingerprint(*d)),
                       {best.lanes_per_codeword, best.slots_per_cta, best.ctas, best.osd_share_rounds, best.osd_ctas});
        if (out_best) *out_best = best;
        if (out_trials)
            for (int i = 0; i < std::min(max_trials, static_cast<int>(trials.size())); ++i) out_trials[i] = trials[i];
        if (out_trial_count) *out_trial_count = static_cast<int>(trials.size());
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_fec_set_timing(unsigned long long handle, int enabled)
{
    return guarded([&] {
        auto d = lookup_any(handle);
        std::lock_guard<std::mutex> lock(d->mu);
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        d->timing.enabled = enabled != 0;
        d->timing.used = 0;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_fec_get_kernel_ms(unsigned long long handle, int* out_calls, float* out_bp_ms, float* out_osd_ms,
                           long long* out_osd_codewords)
{
    return guarded([&] {
        auto d = lookup_any(handle);
        std::lock_guard<std::mutex> lock(d->mu);
        require(d->timing.enabled, "timing is not enabled");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        double bp = 0.0, osd = 0.0;
        long long cw = 0;
        for (size_t i = 0; i < d->timing.used; ++i) {
            auto& r = d->timing.pool[i];
            check_cuda(cudaEventSynchronize(r.ev[3]), "cudaEventSynchronize");
            float a = 0.0f, b = 0.0f;
            check_cuda(cudaEventElapsedTime(&a, r.ev[0], r.ev[1]), "cudaEventElapsedTime");
            check_cuda(cudaEventElapsedTime(&b, r.ev[1], r.ev[2]), "cudaEventElapsedTime");
            bp += a;
            osd += b;
            cw += *r.h_osd;
        }
        if (out_calls) *out_calls = static_cast<int>(d->timing.used);
        if (out_bp_ms) *out_bp_ms = static_cast<float>(bp);
        if (out_osd_ms) *out_osd_ms = static_cast<float>(osd);
        if (out_osd_codewords) *out_osd_codewords = cw;
        d->timing.used = 0;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_fec_decode_device(unsigned long long handle, const float* device_llrs, int codewords,
                           unsigned char* device_info_bits, unsigned char* device_success,
                           unsigned char* device_used_osd, unsigned char* device_iterations, void* cuda_stream)
{
    return guarded([&] {
        auto d = lookup<StreamDecoder>(handle, Decoder::kStream);
        std::lock_guard<std::mutex> lock(d->mu);
        require(device_llrs != nullptr && device_info_bits != nullptr, "null device pointer");
        require(codewords > 0 && codewords <= d->max_batch, "codewords must be in 1..max_batch_size");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        run_bp_osd(*d->code, d->bp, d->shape, d->osd_enabled, device_llrs, codewords, device_info_bits, d->k, d->k,
                   device_success, device_used_osd, device_iterations, nullptr, d->scratch,
                   static_cast<cudaStream_t>(cuda_stream), &d->timing);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_bp_csr_decode_device(unsigned long long handle, const float* device_llrs, int codewords,
                              unsigned char* device_code_bits, unsigned char* device_success, float* device_posteriors,
                              unsigned char* device_iterations, void* cuda_stream)
{
    return guarded([&] {
        auto d = lookup<CsrDecoder>(handle, Decoder::kCsr);
        std::lock_guard<std::mutex> lock(d->mu);
        require(device_llrs != nullptr && codewords > 0, "empty batch");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        run_bp_osd(*d->code, d->bp, d->shape, false, device_llrs, codewords, device_code_bits, d->n, d->n,
                   device_success, nullptr, device_iterations, device_posteriors, d->scratch,
                   static_cast<cudaStream_t>(cuda_stream), &d->timing);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_osd_decode_device(unsigned long long handle, const float* device_llrs, int codewords,
                           unsigned char* device_info_bits, unsigned char* device_code_bits, float* device_distances,
                           void* cuda_stream)
{
    return guarded([&] {
        auto d = lookup_any(handle);
        std::lock_guard<std::mutex> lock(d->mu);
        require(d->kind != Decoder::kCsr && d->code && d->code->has_osd(), "handle has no OSD stage");
        require(device_llrs != nullptr && codewords > 0, "empty batch");
        check_cuda(cudaSetDevice(d->device), "cudaSetDevice");
        OsdIO io{};
        io.llr = device_llrs;
        io.count = codewords;
        io.out_info = device_info_bits;
        io.info_stride = d->k;
        io.out_code = device_code_bits;
        io.out_metric = device_distances;
        io.share_rounds = d->shape.osd_share_rounds;
        launch_osd(d->code->osd_view(), io, codewords, static_cast<cudaStream_t>(cuda_stream), 0,
                   d->shape.osd_ctas);
        return CUDA_OSD_STATUS_OK;
    });
}

}  // extern "C"
