// Device-resident request loop (include/sicc_devloop.h).
//
// The loop is one or more lanes, each a CUDA graph on its own stream: a
// conditional while-node whose body is recorded once (stream capture into the
// node's body graph) and then repeated on the device until its condition
// kernel clears the condition.  The lanes share the request and completion
// rings, so while one lane decodes a batch another admits the next (the
// overlap a host scheduler gets from several batches in flight).  Body of one
// lane iteration, in stream order:
//   admit_kernel     one warp: takes the rings' admission lock (a try-lock in
//                    device memory: a lane that finds it held never waits for
//                    it, it only tries again within its bounded ~100 us of
//                    polling and otherwise admits nothing), fetches up to 32
//                    ring entries at a time from pinned host memory, takes
//                    requests in order while they fit the lane's codeword, LLR,
//                    frame and IQ budgets and the completion ring has room,
//                    reserves their completion slots, publishes the ring head
//                    and releases the lock; sets the condition of the
//                    conditional (if) node that holds the next four steps, so
//                    an iteration that admitted nothing goes straight to
//                    publish_kernel;
//   layout_kernel    copies the admitted inputs (LLRs, or IQ frames) from
//                    pinned host memory into the lane's batch in 64 KB chunks
//                    shared by every CTA, writes the per-codeword tables (code,
//                    protection, offsets) and each profile's frame tables;
//                    zeroes the frame search's tickets;
//   sync + demod     per registered OFDM profile, the batched frame search and
//                    demodulator over its admitted frames (device frame count),
//                    writing their LLRs into the batch;
//   engine decode    the lane's mixed-code engine: prepare, BP and OSD launches,
//                    sized for the largest batch, reading the batch size on the
//                    device;
//   classify_kernel  on a side stream as soon as BP is done: marks the requests
//     + complete_kernel that wait for OSD (a protected codeword failed BP and its
//     (phase 0)      code goes on to OSD) and completes every other request
//                    while the OSD launches run;
//   complete_kernel  (phase 1, after OSD and the side stream) the remaining
//                    requests.  Both phases copy the information bits to the
//                    requests' pinned host buffers in chunks shared by every CTA;
//                    the CTA that ends a request's last chunk writes its
//                    completion record into its reserved slot, sequence number
//                    last;
//   publish_kernel   one thread: makes the iteration's host writes visible,
//                    updates the lane's counters and sets the loop condition
//                    (host stop flag, idle timeout, iteration cap).
// The host side only fills the request ring and drains the completion ring,
// taking each record whose sequence number is set (lanes finish out of order).
// An idle lane announces its end (`ended`) and then reads the ring's tail once
// more; a submit appends, then reads every lane's `ended`, and launches again
// each lane that has gone (each side fences between its write and its read, so
// at least one of them sees the other).  A poll that finds lanes finished with
// requests still in the ring launches them again as well.
#include "../../include/sicc_devloop.h"
#include "engine_internal.h"
#include "pipe_internal.h"
#include "sicc_common.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace sicc {
namespace {

using Clock = std::chrono::steady_clock;

constexpr int kMaxPhys = 8;
constexpr int kMaxLanes = 16;

struct alignas(16) ReqEntry {  // host -> device, one per request
    unsigned long long id, tag;
    const float* in;            // kind 0: [count][n] LLRs; kind 1: [count][stride] complex IQ
                                // (device-addressable pinned host memory)
    unsigned char* out;         // [codewords][k] information bits, the same kind of memory
    int kind, code_id, phy_id, count, protection, n, k, codewords, stride, pad;
};

static_assert(sizeof(ReqEntry) % 16 == 0, "ring entries are read as 16-byte words");

struct PhyDev {  // a registered OFDM profile's device tables in one lane
    long long* frame_off;      // [max_frames] complex-sample offset of each admitted frame in the IQ buffer
    long long* llr_frame_off;  // [max_frames] float offset of its LLRs in the batch
    int* ticket;               // the frame search's tickets, zero before each search
    int ticket_ints;
    int blocks;                // codewords per frame
};

struct alignas(16) CmpEntry {  // device -> host, one per request
    unsigned long long id, tag;
    unsigned long long t_start_ns, t_done_ns;  // device clock: its iteration's decode start, publication
    int codewords, failed, osd, status;
    unsigned long long seq;                    // slot + 1 once the record is complete (written last)
};

struct alignas(128) HostSide {  // written by the host, read by the device (pinned)
    unsigned long long req_tail;   // requests published
    unsigned long long cmp_head;   // completion slots below this are consumed
    int stop;
};

struct alignas(128) DevSide {  // written by the admitting lane, read by the host (pinned)
    unsigned long long req_head;      // requests admitted
    unsigned long long cmp_reserved;  // completion slots reserved
};

struct alignas(128) LaneSide {  // written by one lane, read by the host (pinned)
    unsigned long long iterations, codewords, busy_iterations;
    int ended;                     // 0: running, 1: stop flag, 2: idle timeout, 3: iteration cap
};

struct Shared {  // device memory, shared by the lanes (changed under the admission lock)
    unsigned long long head;         // next request to admit
    unsigned long long cmp_reserve;  // next completion slot
    int lock;
};

struct LoopState {  // device memory, one per lane
    unsigned long long cmp_base;  // the iteration's first completion slot
    unsigned long long iterations, codewords, busy_iterations;
    unsigned long long last_active_ns, t_start_ns;
    int nreq, count;
    int in_chunks, out_chunks;  // copy chunks of the admitted requests
    int phy_frames[kMaxPhys];   // admitted frames of each profile
};

struct Admitted {
    ReqEntry e;
    long long llr_off, info_off, iq_off;
    int first_cw, frame_base;
    int in_chunk, out_chunk;  // its first input / output chunk in the iteration's chunk lists
};

// Host-memory copies are cut into chunks that every CTA of the layout and
// completion grids shares, so one large request is not copied by one CTA.
constexpr long long kInChunkFloats = 16384;  // 64 KB of LLRs or IQ samples
constexpr long long kOutChunkBytes = 32768;  // information bits

constexpr int kAdmitPolls = 50;            // ~2 us naps: an empty ring is watched ~100 us per iteration
constexpr unsigned long long kIterationCap = 1ull << 31;

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long load_acquire_sys(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int load_acquire_sys(const int* p)
{
    int v;
    asm volatile("ld.acquire.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void store_release_sys(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void store_release_sys_int(int* p, int v)
{
    asm volatile("st.release.sys.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long shared_head(const Shared* sh)
{
    return *reinterpret_cast<const volatile unsigned long long*>(&sh->head);
}

__global__ void __launch_bounds__(32) admit_kernel(const ReqEntry* ring, unsigned mask, const HostSide* hs,
                                                   DevSide* ds, Shared* sh, LoopState* st, Admitted* adm, int max_req,
                                                   int max_cw, long long max_floats, unsigned cmp_capacity,
                                                   int max_frames, long long max_iq, cudaGraphConditionalHandle work)
{
    // one warp: lane 0 takes the admission lock; the lanes fetch up to 32 ring entries at once (host
    // memory is far), lane 0 takes them in order while they fit
    __shared__ ReqEntry win[32];
    const int lane = threadIdx.x;
    int locked = 0;
    if (lane == 0) {
        for (int i = 0;; ++i) {
            const unsigned long long tail = load_acquire_sys(&hs->req_tail);
            if (tail != shared_head(sh) && atomicCAS(&sh->lock, 0, 1) == 0) {
                locked = 1;
                break;
            }
            if (i >= kAdmitPolls) break;  // bounded: a held lock or an empty ring ends in an empty iteration
            __nanosleep(2000);
        }
        __threadfence();  // the lock holder's view of the shared state follows the previous holder's writes
    }
    locked = __shfl_sync(0xffffffffu, locked, 0);
    int nreq = 0, cw = 0, frames = 0, in_chunks = 0, out_chunks = 0;
    long long floats = 0, info = 0, iq = 0;
    int pf[kMaxPhys];
#pragma unroll
    for (int p = 0; p < kMaxPhys; ++p) pf[p] = 0;
    if (locked) {
        unsigned long long head = 0, tail = 0, reserve = 0, consumed = 0;
        if (lane == 0) {
            head = shared_head(sh);
            reserve = *reinterpret_cast<const volatile unsigned long long*>(&sh->cmp_reserve);
            tail = load_acquire_sys(&hs->req_tail);
            consumed = load_acquire_sys(&hs->cmp_head);
        }
        __syncwarp();  // lane 0's acquire of the tail orders the other lanes' reads of the entries below it
        head = __shfl_sync(0xffffffffu, head, 0);
        tail = __shfl_sync(0xffffffffu, tail, 0);
        reserve = __shfl_sync(0xffffffffu, reserve, 0);
        consumed = __shfl_sync(0xffffffffu, consumed, 0);
        const unsigned long long room = cmp_capacity - (reserve - consumed);
        const unsigned long long limit = min(static_cast<unsigned long long>(max_req), room);
        bool full = false;
        while (!full && head < tail && static_cast<unsigned long long>(nreq) < limit) {
            const int avail = static_cast<int>(min(32ull, tail - head));
            if (lane < avail) {  // published before the tail (acquire above); read past every cache
                const uint4* src = reinterpret_cast<const uint4*>(ring + ((head + lane) & mask));
                uint4* dst = reinterpret_cast<uint4*>(&win[lane]);
#pragma unroll
                for (int q = 0; q < static_cast<int>(sizeof(ReqEntry) / 16); ++q) dst[q] = __ldcv(src + q);
            }
            __syncwarp();
            if (lane == 0) {
                for (int j = 0; j < avail && static_cast<unsigned long long>(nreq) < limit; ++j) {
                    const ReqEntry& e = win[j];
                    const long long f = static_cast<long long>(e.codewords) * e.n;
                    const bool iq_req = e.kind == 1;
                    const long long samples = iq_req ? static_cast<long long>(e.count) * e.stride : 0;
                    // in submission order: a request that does not fit waits for the next iteration, and so
                    // do those after it
                    if (cw + e.codewords > max_cw || floats + f > max_floats ||
                        (iq_req && (frames + e.count > max_frames || iq + samples > max_iq))) {
                        full = true;
                        break;
                    }
                    Admitted& a = adm[nreq];
                    a.e = e;
                    a.first_cw = cw;
                    a.llr_off = floats;
                    a.info_off = info;
                    a.iq_off = iq;
                    a.frame_base = iq_req ? pf[e.phy_id] : 0;
                    a.in_chunk = in_chunks;
                    a.out_chunk = out_chunks;
                    const long long in_floats = iq_req ? 2 * samples : f;
                    in_chunks += static_cast<int>((in_floats + kInChunkFloats - 1) / kInChunkFloats);
                    out_chunks += static_cast<int>((static_cast<long long>(e.codewords) * e.k + kOutChunkBytes - 1) /
                                                   kOutChunkBytes);
                    cw += e.codewords;
                    floats += f;
                    // each request's information bits and IQ samples start 16-byte aligned (whole 16-byte copies)
                    info += (static_cast<long long>(e.codewords) * e.k + 15) & ~15ll;
                    if (iq_req) {
                        frames += e.count;
                        iq += (samples + 1) & ~1ll;
                        pf[e.phy_id] += e.count;
                    }
                    ++nreq;
                    ++head;
                }
            }
            head = __shfl_sync(0xffffffffu, head, 0);
            nreq = __shfl_sync(0xffffffffu, nreq, 0);
            full = __shfl_sync(0xffffffffu, full ? 1 : 0, 0) != 0;
            __syncwarp();  // the window is rewritten by the next fetch
        }
        if (lane == 0) {
            sh->head = head;
            sh->cmp_reserve = reserve + static_cast<unsigned long long>(nreq);
            st->cmp_base = reserve;
            __threadfence_system();  // the admission table holds the entries before their slots are freed
            store_release_sys(&ds->cmp_reserved, reserve + static_cast<unsigned long long>(nreq));
            store_release_sys(&ds->req_head, head);
            __threadfence();
            atomicExch(&sh->lock, 0);
        }
    }
    if (lane != 0) return;
    st->nreq = nreq;
    st->count = cw;
    st->in_chunks = in_chunks;
    st->out_chunks = out_chunks;
#pragma unroll
    for (int p = 0; p < kMaxPhys; ++p) st->phy_frames[p] = pf[p];
    const unsigned long long now = globaltimer_ns();
    if (nreq > 0 || st->last_active_ns == 0) st->last_active_ns = now;
    st->t_start_ns = now;
    cudaGraphSetConditional(work, nreq > 0 ? 1u : 0u);  // an empty iteration skips to publication
}

// The admitted request whose chunk list holds chunk g: the last r with first(r) <= g.
template <class F>
__device__ __forceinline__ int owner_of(int g, int nreq, F first)
{
    int lo = 0, hi = nreq - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first(mid) <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// dst[0, count) = src[0, count) by one CTA, four 16-byte accesses in flight per thread when both
// ends are 16-byte aligned (host memory is far: the loads must overlap)
__device__ __forceinline__ void copy_bytes(const unsigned char* __restrict__ src, unsigned char* __restrict__ dst,
                                           long long count)
{
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) {
        const long long n16 = count >> 4;
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(dst);
        const long long step = blockDim.x;
        long long i = threadIdx.x;
        for (; i + 3 * step < n16; i += 4 * step) {
            const uint4 a = s4[i], b = s4[i + step], c = s4[i + 2 * step], d = s4[i + 3 * step];
            d4[i] = a;
            d4[i + step] = b;
            d4[i + 2 * step] = c;
            d4[i + 3 * step] = d;
        }
        for (; i < n16; i += step) d4[i] = s4[i];
        for (long long j = (n16 << 4) + threadIdx.x; j < count; j += step) dst[j] = src[j];
    } else {
        for (long long j = threadIdx.x; j < count; j += blockDim.x) dst[j] = src[j];
    }
}

// One iteration's layout: the admitted requests' inputs are copied chunk by chunk
// (all CTAs share every request), then each request's codeword and frame tables
// are written; CTA 0 also zeroes every profile's frame-search tickets and the
// completion counters.
__global__ void layout_kernel(const LoopState* st, const Admitted* __restrict__ adm, float* __restrict__ llr,
                              float* __restrict__ iq, const PhyDev* __restrict__ phys, int nphys,
                              uint8_t* __restrict__ code_of, uint8_t* __restrict__ protect,
                              long long* __restrict__ llr_off, long long* __restrict__ info_off,
                              int* __restrict__ chunks_done)
{
    __shared__ int s_r;
    const int nreq = st->nreq;
    if (blockIdx.x == 0) {
        for (int p = 0; p < nphys; ++p)
            for (int i = threadIdx.x; i < phys[p].ticket_ints; i += blockDim.x) phys[p].ticket[i] = 0;
        for (int r = threadIdx.x; r < nreq; r += blockDim.x) chunks_done[r] = 0;
    }
    const int total = st->in_chunks;
    for (int g = blockIdx.x; g < total; g += gridDim.x) {
        if (threadIdx.x == 0) s_r = owner_of(g, nreq, [&](int r) { return adm[r].in_chunk; });
        __syncthreads();
        const Admitted& a = adm[s_r];
        const long long c = g - a.in_chunk;
        const long long floats =
            a.e.kind == 0 ? static_cast<long long>(a.e.codewords) * a.e.n : 2 * static_cast<long long>(a.e.count) * a.e.stride;
        const long long lo = c * kInChunkFloats, hi = min(floats, lo + kInChunkFloats);
        float* dst = a.e.kind == 0 ? llr + a.llr_off : iq + 2 * a.iq_off;
        copy_bytes(reinterpret_cast<const unsigned char*>(a.e.in + lo), reinterpret_cast<unsigned char*>(dst + lo),
                   (hi - lo) * static_cast<long long>(sizeof(float)));
        __syncthreads();  // s_r is rewritten by the next chunk
    }
    for (int r = blockIdx.x; r < nreq; r += gridDim.x) {
        const Admitted& a = adm[r];
        if (a.e.kind == 1) {
            const PhyDev ph = phys[a.e.phy_id];
            for (int f = threadIdx.x; f < a.e.count; f += blockDim.x) {
                ph.frame_off[a.frame_base + f] = a.iq_off + static_cast<long long>(f) * a.e.stride;
                ph.llr_frame_off[a.frame_base + f] = a.llr_off + static_cast<long long>(f) * ph.blocks * a.e.n;
            }
        }
        for (int c = threadIdx.x; c < a.e.codewords; c += blockDim.x) {
            const int w = a.first_cw + c;
            code_of[w] = static_cast<uint8_t>(a.e.code_id);
            protect[w] = static_cast<uint8_t>(a.e.protection);
            llr_off[w] = a.llr_off + static_cast<long long>(c) * a.e.n;
            info_off[w] = a.info_off + static_cast<long long>(c) * a.e.k;
        }
    }
}

// After BP: a request is late (phase 1) when one of its codewords failed BP,
// is protected and its code goes on to OSD; every other request's bits are
// final (phase 0).  One CTA per request (grid-strided).
__global__ void classify_kernel(const LoopState* st, const Admitted* __restrict__ adm,
                                const uint8_t* __restrict__ code_of, const uint8_t* __restrict__ protect,
                                const uint8_t* __restrict__ success, const uint8_t* __restrict__ routes,
                                uint8_t* __restrict__ late)
{
    const int nreq = st->nreq;
    for (int r = blockIdx.x; r < nreq; r += gridDim.x) {
        const Admitted& a = adm[r];
        int osd = 0;
        for (int c = threadIdx.x; c < a.e.codewords; c += blockDim.x) {
            const int w = a.first_cw + c;
            osd |= (!success[w] && protect[w] && routes[code_of[w]]) ? 1 : 0;
        }
        osd = __syncthreads_or(osd);
        if (threadIdx.x == 0) late[r] = static_cast<uint8_t>(osd);
    }
}

// One iteration's completion of the requests of one phase (0: final after BP,
// 1: after OSD): the information bits go to the requests' host buffers chunk
// by chunk (all CTAs share every request); the CTA that finishes a request's
// last chunk counts its BP failures and OSD codewords and writes its
// completion record into the slot its admission reserved, the sequence number
// last.
__global__ void complete_kernel(const LoopState* st, const Admitted* __restrict__ adm,
                                const uint8_t* __restrict__ info, const uint8_t* __restrict__ success,
                                const uint8_t* __restrict__ used_osd, CmpEntry* ring, unsigned mask,
                                int* __restrict__ chunks_done, const uint8_t* __restrict__ late, int phase)
{
    __shared__ int s_r, s_last, s_failed, s_osd;
    const int nreq = st->nreq;
    const int total = st->out_chunks;
    for (int g = blockIdx.x; g < total; g += gridDim.x) {
        if (threadIdx.x == 0) {
            s_r = owner_of(g, nreq, [&](int r) { return adm[r].out_chunk; });
            s_failed = 0;
            s_osd = 0;
        }
        __syncthreads();
        const int r = s_r;
        if (late[r] != phase) {  // the other phase's request (uniform over the CTA)
            __syncthreads();  // s_r is rewritten by the next chunk
            continue;
        }
        const Admitted& a = adm[r];
        const long long bytes = static_cast<long long>(a.e.codewords) * a.e.k;
        const int nchunks = static_cast<int>((bytes + kOutChunkBytes - 1) / kOutChunkBytes);
        const long long lo = static_cast<long long>(g - a.out_chunk) * kOutChunkBytes;
        const long long hi = min(bytes, lo + kOutChunkBytes);
        copy_bytes(info + a.info_off + lo, a.e.out + lo, hi - lo);
        __threadfence_system();  // this CTA's bits reach host memory before the request's record
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(&chunks_done[r], 1) == nchunks - 1;
        __syncthreads();
        if (s_last) {
            __threadfence();  // the other CTAs' chunks of this request are complete (their fences came first)
            int failed = 0, osd = 0;
            for (int c = threadIdx.x; c < a.e.codewords; c += blockDim.x) {
                const int w = a.first_cw + c;
                const int u = used_osd[w], ok = success[w];
                osd += u;
                failed += (!u && !ok) ? 1 : 0;
            }
            if (failed) atomicAdd(&s_failed, failed);
            if (osd) atomicAdd(&s_osd, osd);
            __syncthreads();
            if (threadIdx.x == 0) {
                const unsigned long long slot = st->cmp_base + static_cast<unsigned long long>(r);
                CmpEntry* c = ring + (slot & mask);
                c->id = a.e.id;
                c->tag = a.e.tag;
                c->t_start_ns = st->t_start_ns;
                c->t_done_ns = globaltimer_ns();
                c->codewords = a.e.codewords;
                c->failed = s_failed;
                c->osd = s_osd;
                c->status = 0;
                __threadfence_system();
                store_release_sys(&c->seq, slot + 1);
            }
        }
        __syncthreads();  // the shared scalars are rewritten by the next chunk
    }
}

__global__ void publish_kernel(LoopState* st, const HostSide* hs, const Shared* sh, LaneSide* ls,
                               cudaGraphConditionalHandle cond, unsigned long long idle_ns)
{
    __threadfence_system();  // every host write of this iteration is out before the counters move
    st->iterations += 1;
    st->codewords += static_cast<unsigned long long>(st->count);
    st->busy_iterations += st->nreq > 0 ? 1ull : 0ull;
    ls->iterations = st->iterations;
    ls->codewords = st->codewords;
    ls->busy_iterations = st->busy_iterations;
    int reason = 0;
    if (load_acquire_sys(&hs->stop)) reason = 1;
    else if (st->nreq == 0 && globaltimer_ns() - st->last_active_ns > idle_ns) reason = 2;
    else if (st->iterations >= kIterationCap) reason = 3;
    if (reason) {
        // Announce the end, then read the ring's tail once more.  The host appends a request, then
        // reads `ended` (each side with a full fence between its write and its read), so either the
        // host sees the announcement and launches the lane again, or this read sees the request and
        // an idle lane carries on.
        store_release_sys_int(&ls->ended, reason);
        asm volatile("fence.sc.sys;" ::: "memory");
        if (reason == 2 && load_acquire_sys(&hs->req_tail) != shared_head(sh)) {
            store_release_sys_int(&ls->ended, 0);
            st->last_active_ns = globaltimer_ns();
            reason = 0;
        }
    }
    cudaGraphSetConditional(cond, reason ? 0u : 1u);
}

__global__ void clock_kernel(unsigned long long* out) { *out = globaltimer_ns(); }

template <class T>
struct Pinned {
    T* h = nullptr;  // host address
    T* d = nullptr;  // device address of the same memory
    void alloc(size_t count)
    {
        check_cuda(cudaHostAlloc(reinterpret_cast<void**>(&h), count * sizeof(T), cudaHostAllocMapped),
                   "cudaHostAlloc(loop)");
        std::memset(static_cast<void*>(h), 0, count * sizeof(T));
        check_cuda(cudaHostGetDevicePointer(reinterpret_cast<void**>(&d), h, 0), "cudaHostGetDevicePointer");
    }
    ~Pinned()
    {
        if (h) cudaFreeHost(h);
    }
};

template <class T>
struct Dev {
    T* p = nullptr;
    void alloc(size_t count)
    {
        check_cuda(cudaMalloc(reinterpret_cast<void**>(&p), std::max<size_t>(count, 1) * sizeof(T)),
                   "cudaMalloc(loop)");
        check_cuda(cudaMemset(p, 0, std::max<size_t>(count, 1) * sizeof(T)), "cudaMemset(loop)");
    }
    ~Dev()
    {
        if (p) cudaFree(p);
    }
};

struct CodeDims {
    int n, k;
};

struct Pending {
    Clock::time_point t_submit;
};

struct PhyHost {  // a registered OFDM profile (its tables serve every lane)
    unsigned long long pipe = 0;
    int stride = 0, code_id = 0, blocks = 0;
    size_t scratch_bytes = 0, ticket_offset = 0, ticket_bytes = 0;
    ~PhyHost()
    {
        if (pipe) sicc_pipe_destroy(pipe);
    }
};

struct LanePhy {  // a profile's per-lane buffers
    Dev<long long> frame_off, llr_frame_off;
    Dev<unsigned char> sync, scratch;
};

struct Lane {  // one loop graph, its stream, engine and batch state
    unsigned long long engine = 0;
    Dev<LoopState> st;
    Dev<Admitted> adm;
    Dev<float> llr;
    Dev<uint8_t> info, code_of, protect, success, used, iters;
    Dev<long long> llr_off, info_off;
    Dev<int> chunks_done;  // [max_req] finished output chunks of each admitted request
    Dev<uint8_t> late;     // [max_req] 1: the request waits for OSD
    Dev<uint8_t> routes;   // [max_codes] 1: the code's protected BP failures go to OSD
    cudaStream_t side = nullptr;  // completion of the requests that are final after BP
    cudaEvent_t bp_done = nullptr, early_done = nullptr;
    Dev<float> iqbuf;      // [max_batch_iq_samples] complex samples
    std::vector<std::unique_ptr<LanePhy>> phys;
    Dev<PhyDev> d_phys;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::atomic<bool> launched{false};  // written under the loop's mu; poll reads it

    ~Lane()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (bp_done) cudaEventDestroy(bp_done);
        if (early_done) cudaEventDestroy(early_done);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
        if (engine) sicc_engine_destroy(engine);
    }

    bool graph_done() const
    {
        if (!launched) return true;
        const cudaError_t q = cudaStreamQuery(stream);
        if (q == cudaErrorNotReady) return false;
        check_cuda(q, "loop stream");
        return true;
    }
};

struct Loop {
    sicc_devloop_config_t cfg{};
    int device = 0;
    std::vector<CodeDims> codes;
    int max_req = 0;
    unsigned mask = 0;
    // rings and control blocks (pinned, mapped)
    Pinned<ReqEntry> ring;
    Pinned<CmpEntry> cring;
    Pinned<HostSide> hs;
    Pinned<DevSide> ds;
    Pinned<LaneSide> lane_side;  // [lanes]
    Pinned<unsigned long long> clock;
    Dev<Shared> sh;
    std::vector<std::unique_ptr<PhyHost>> phys;
    std::vector<std::unique_ptr<Lane>> lanes;
    long long info_cap = 0;
    bool recorded = false;
    // host bookkeeping
    unsigned long long next_id = 1, req_tail = 0, cmp_head = 0;
    std::vector<uint8_t> taken;  // [ring] completion slots consumed ahead of cmp_head
    std::map<unsigned long long, Pending> pending;
    long long clock_offset_ns = 0;  // device globaltimer - host steady clock (ns)
    Clock::time_point clock_base;
    sicc_devloop_stats_t stats{};
    std::mutex mu;          // submit side
    std::mutex poll_mu;     // poll side (one poller at a time)
    std::mutex pending_mu;  // pending and completed: held briefly by submit and poll
    unsigned long long completed = 0;

    int ended(int l) const
    {
        return reinterpret_cast<const std::atomic<int>*>(&lane_side.h[l].ended)->load(std::memory_order_acquire);
    }

    bool all_done() const
    {
        for (const auto& ln : lanes)
            if (!ln->graph_done()) return false;
        return true;
    }

    void record_lane(Lane& ln, int l)
    {
        if (engine_prepare_capture(ln.engine, cfg.max_batch_codewords) != CUDA_OSD_STATUS_OK)
            throw std::runtime_error(last_error());
        ln.info.alloc(static_cast<size_t>(info_cap));
        {
            unsigned char r[64] = {0};
            int nc = 0;
            if (engine_code_routes(ln.engine, r, 64, &nc) != CUDA_OSD_STATUS_OK) throw std::runtime_error(last_error());
            ln.routes.alloc(64);
            check_cuda(cudaMemcpy(ln.routes.p, r, sizeof(r), cudaMemcpyHostToDevice), "upload code routes");
        }
        std::vector<PhyDev> pd;
        for (size_t q = 0; q < phys.size(); ++q) {
            PhyDev d{};
            d.frame_off = ln.phys[q]->frame_off.p;
            d.llr_frame_off = ln.phys[q]->llr_frame_off.p;
            d.ticket = reinterpret_cast<int*>(ln.phys[q]->scratch.p + phys[q]->ticket_offset);
            d.ticket_ints = static_cast<int>(phys[q]->ticket_bytes / sizeof(int));
            d.blocks = phys[q]->blocks;
            pd.push_back(d);
        }
        ln.d_phys.alloc(std::max<size_t>(pd.size(), 1));
        if (!pd.empty())
            check_cuda(cudaMemcpy(ln.d_phys.p, pd.data(), pd.size() * sizeof(PhyDev), cudaMemcpyHostToDevice),
                       "upload profiles");
        cudaStream_t stream = ln.stream;
        check_cuda(cudaGraphCreate(&ln.graph, 0), "cudaGraphCreate");
        // graph: while (loop) { admit; if (admitted) { layout; demod; decode; complete } publish }
        cudaGraphConditionalHandle loop_cond, work_cond;
        check_cuda(cudaGraphConditionalHandleCreate(&loop_cond, ln.graph, 1, cudaGraphCondAssignDefault),
                   "cudaGraphConditionalHandleCreate(loop)");
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = loop_cond;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t node;
        check_cuda(cudaGraphAddNode(&node, ln.graph, nullptr, nullptr, 0, &p), "cudaGraphAddNode(while)");
        cudaGraph_t body = p.conditional.phGraph_out[0];
        check_cuda(cudaGraphConditionalHandleCreate(&work_cond, body, 0, cudaGraphCondAssignDefault),
                   "cudaGraphConditionalHandleCreate(work)");
        auto end_capture = [&](const char* what) {
            cudaGraph_t out = nullptr;
            check_cuda(cudaStreamEndCapture(stream, &out), what);
        };
        auto abandon = [&](const std::string& why) {
            cudaGraph_t dummy = nullptr;
            cudaStreamEndCapture(stream, &dummy);
            throw std::runtime_error(why);
        };
        // 1. admission, the body's first node
        check_cuda(cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
                   "cudaStreamBeginCaptureToGraph(admit)");
        admit_kernel<<<1, 32, 0, stream>>>(ring.d, mask, hs.d, ds.d, sh.p, ln.st.p, ln.adm.p, max_req,
                                            cfg.max_batch_codewords, cfg.max_batch_llr_floats, mask + 1,
                                            cfg.max_batch_frames, cfg.max_batch_iq_samples, work_cond);
        end_capture("cudaStreamEndCapture(admit)");
        cudaGraphNode_t admit_node = nullptr;
        size_t nodes = 1;
        check_cuda(cudaGraphGetNodes(body, &admit_node, &nodes), "cudaGraphGetNodes(admit)");
        if (nodes != 1 || !admit_node) throw std::runtime_error("recording the loop: admission is not one node");
        // 2. the iteration's work, run when admit_kernel admitted a request
        cudaGraphNodeParams ip{};
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = work_cond;
        ip.conditional.type = cudaGraphCondTypeIf;
        ip.conditional.size = 1;
        cudaGraphNode_t if_node;
        check_cuda(cudaGraphAddNode(&if_node, body, &admit_node, nullptr, 1, &ip), "cudaGraphAddNode(if)");
        cudaGraph_t work = ip.conditional.phGraph_out[0];
        check_cuda(cudaStreamBeginCaptureToGraph(stream, work, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
                   "cudaStreamBeginCaptureToGraph(work)");
        const int sms = device_sm_count();
        layout_kernel<<<2 * sms, 256, 0, stream>>>(ln.st.p, ln.adm.p, ln.llr.p, ln.iqbuf.p, ln.d_phys.p,
                                                    static_cast<int>(phys.size()), ln.code_of.p, ln.protect.p,
                                                    ln.llr_off.p, ln.info_off.p, ln.chunks_done.p);
        for (size_t q = 0; q < phys.size(); ++q) {  // each profile's admitted frames: search + demodulation
            const PhyHost& ph = *phys[q];
            LanePhy& lp = *ln.phys[q];
            if (pipe_gather_counted(ph.pipe, ln.iqbuf.p, lp.frame_off.p, ph.stride, cfg.max_batch_frames,
                                    &ln.st.p->phy_frames[q], ln.llr.p, lp.llr_frame_off.p, lp.sync.p, lp.scratch.p,
                                    ph.scratch_bytes, stream) != CUDA_OSD_STATUS_OK)
                abandon(std::string("recording the loop's demodulation: ") + last_error());
        }
        const int rc = engine_decode(ln.engine, cfg.max_batch_codewords, ln.code_of.p, ln.protect.p, ln.llr.p,
                                     ln.llr_off.p, ln.info.p, ln.info_off.p, ln.success.p, ln.used.p, ln.iters.p,
                                     stream, ln.bp_done, &ln.st.p->count);
        if (rc != CUDA_OSD_STATUS_OK) abandon(std::string("recording the loop's decode: ") + last_error());
        // requests final after BP complete on the side stream while OSD runs; the rest after OSD
        check_cuda(cudaStreamWaitEvent(ln.side, ln.bp_done, 0), "cudaStreamWaitEvent(bp done)");
        classify_kernel<<<2 * sms, 256, 0, ln.side>>>(ln.st.p, ln.adm.p, ln.code_of.p, ln.protect.p, ln.success.p,
                                                      ln.routes.p, ln.late.p);
        complete_kernel<<<2 * sms, 256, 0, ln.side>>>(ln.st.p, ln.adm.p, ln.info.p, ln.success.p, ln.used.p,
                                                      cring.d, mask, ln.chunks_done.p, ln.late.p, 0);
        check_cuda(cudaEventRecord(ln.early_done, ln.side), "cudaEventRecord(early completions)");
        check_cuda(cudaStreamWaitEvent(stream, ln.early_done, 0), "cudaStreamWaitEvent(early completions)");
        complete_kernel<<<2 * sms, 256, 0, stream>>>(ln.st.p, ln.adm.p, ln.info.p, ln.success.p, ln.used.p, cring.d,
                                                      mask, ln.chunks_done.p, ln.late.p, 1);
        end_capture("cudaStreamEndCapture(work)");
        // 3. publication, after the work node
        check_cuda(cudaStreamBeginCaptureToGraph(stream, body, &if_node, nullptr, 1, cudaStreamCaptureModeRelaxed),
                   "cudaStreamBeginCaptureToGraph(publish)");
        publish_kernel<<<1, 1, 0, stream>>>(ln.st.p, hs.d, sh.p, lane_side.d + l, loop_cond,
                                            static_cast<unsigned long long>(cfg.idle_timeout_ms) * 1000000ull);
        end_capture("cudaStreamEndCapture(publish)");
        check_cuda(cudaGraphInstantiate(&ln.exec, ln.graph, 0), "cudaGraphInstantiate(loop)");
    }

    void record()
    {
        int n_max = 0, k_max = 0;
        if (engine_bounds(lanes[0]->engine, &n_max, &k_max) != CUDA_OSD_STATUS_OK)
            throw std::runtime_error(last_error());
        info_cap = static_cast<long long>(cfg.max_batch_codewords) * k_max + 16ll * max_req;  // + per-request alignment
        for (size_t l = 0; l < lanes.size(); ++l) record_lane(*lanes[l], static_cast<int>(l));
        recorded = true;
    }

    void calibrate()
    {
        const auto t0 = Clock::now();
        clock_kernel<<<1, 1, 0, lanes[0]->stream>>>(clock.d);
        check_cuda(cudaStreamSynchronize(lanes[0]->stream), "clock");
        const auto t1 = Clock::now();
        const auto mid = t0 + (t1 - t0) / 2;
        clock_base = mid;
        clock_offset_ns = static_cast<long long>(*clock.h);
    }

    // device ns -> host time point
    Clock::time_point host_time(unsigned long long dev_ns) const
    {
        return clock_base + std::chrono::nanoseconds(static_cast<long long>(dev_ns) - clock_offset_ns);
    }

    // Launches every lane that is not running (the caller holds mu).  Called after a request was
    // appended: a lane that has announced its end (publish_kernel) either took the request back and
    // carries on, or finishes and is launched again here.
    void ensure_running()
    {
        std::atomic_thread_fence(std::memory_order_seq_cst);  // the tail is out before `ended` is read
        if (!recorded) {
            record();
            calibrate();
        }
        for (size_t l = 0; l < lanes.size(); ++l) {
            Lane& ln = *lanes[l];
            if (ln.launched) {
                if (ended(static_cast<int>(l)) == 0) continue;  // running (no stream query on this path)
                const auto deadline = Clock::now() + std::chrono::seconds(10);
                bool carries_on = false;
                while (!ln.graph_done()) {
                    if (ended(static_cast<int>(l)) == 0) {
                        carries_on = true;  // it saw the request and goes on
                        break;
                    }
                    if (Clock::now() > deadline) throw std::runtime_error("a device-loop lane did not finish ending");
                    std::this_thread::sleep_for(std::chrono::microseconds(2));
                }
                if (carries_on) continue;
            }
            reinterpret_cast<std::atomic<int>*>(&lane_side.h[l].ended)->store(0, std::memory_order_relaxed);
            reinterpret_cast<std::atomic<int>*>(&hs.h->stop)->store(0, std::memory_order_release);
            check_cuda(cudaMemsetAsync(&ln.st.p->last_active_ns, 0, sizeof(unsigned long long), ln.stream),
                       "loop reset");
            check_cuda(cudaGraphLaunch(ln.exec, ln.stream), "cudaGraphLaunch(loop)");
            ln.launched = true;
            ++stats.launches;
        }
    }
};

std::mutex g_mu;
std::map<unsigned long long, std::shared_ptr<Loop>> g_loops;
unsigned long long g_next = 0xD100;

std::shared_ptr<Loop> get(unsigned long long h)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_loops.find(h);
    if (it == g_loops.end()) throw InvalidArgument("invalid device-loop handle");
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

template <class T>
T load_acquire(const T* p)
{
    return reinterpret_cast<const std::atomic<T>*>(p)->load(std::memory_order_acquire);
}

template <class T>
void store_release(T* p, T v)
{
    reinterpret_cast<std::atomic<T>*>(p)->store(v, std::memory_order_release);
}

// The device address of pinned host memory the GPU can use, or nullptr.
const void* device_address(const void* p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost && a.type != cudaMemoryTypeManaged) return nullptr;
    return a.devicePointer;
}

double us_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::micro>(b - a).count();
}

}  // namespace
}  // namespace sicc

using namespace sicc;

extern "C" {

int sicc_devloop_create(const sicc_devloop_config_t* config, unsigned long long* out_handle)
{
    return guarded([&]() -> int {
        if (!config || !out_handle) throw InvalidArgument("null argument");
        *out_handle = 0;
        const sicc_devloop_config_t& c = *config;
        if (c.max_batch_codewords <= 0 || c.max_batch_llr_floats <= 0)
            throw InvalidArgument("the iteration budgets must be positive");
        if (c.max_codes <= 0 || c.max_codes > 64) throw InvalidArgument("max_codes must be 1..64");
        if (c.ring_requests < 2 || (c.ring_requests & (c.ring_requests - 1)))
            throw InvalidArgument("ring_requests must be a power of two >= 2");
        if (c.idle_timeout_ms < 1) throw InvalidArgument("idle_timeout_ms must be >= 1");
        if (c.max_batch_frames < 0 || c.max_batch_iq_samples < 0 || (c.max_batch_frames > 0) != (c.max_batch_iq_samples > 0))
            throw InvalidArgument("max_batch_frames and max_batch_iq_samples: both positive (IQ requests) or both 0");
        if (c.lanes < 0 || c.lanes > kMaxLanes) throw InvalidArgument("lanes must be 0..16 (0: one lane)");
        auto L = std::make_shared<Loop>();
        L->cfg = c;
        L->cfg.lanes = std::max(1, c.lanes);
        check_cuda(cudaGetDevice(&L->device), "cudaGetDevice");
        L->mask = static_cast<unsigned>(c.ring_requests - 1);
        L->max_req = std::min(c.ring_requests, c.max_batch_codewords);
        L->ring.alloc(c.ring_requests);
        L->cring.alloc(c.ring_requests);
        L->taken.assign(static_cast<size_t>(c.ring_requests), 0);
        L->hs.alloc(1);
        L->ds.alloc(1);
        L->lane_side.alloc(static_cast<size_t>(L->cfg.lanes));
        L->clock.alloc(1);
        L->sh.alloc(1);
        for (int l = 0; l < L->cfg.lanes; ++l) {
            auto ln = std::make_unique<Lane>();
            sicc_engine_config_t ec{};
            ec.max_codewords = c.max_batch_codewords;
            ec.max_llr_floats = c.max_batch_llr_floats;
            ec.max_codes = c.max_codes;
            if (sicc_engine_create(&ec, &ln->engine) != CUDA_OSD_STATUS_OK) throw std::runtime_error(last_error());
            ln->st.alloc(1);
            ln->adm.alloc(static_cast<size_t>(L->max_req));
            ln->llr.alloc(static_cast<size_t>(c.max_batch_llr_floats));
            for (auto* b : {&ln->code_of, &ln->protect, &ln->success, &ln->used, &ln->iters})
                b->alloc(static_cast<size_t>(c.max_batch_codewords));
            ln->llr_off.alloc(static_cast<size_t>(c.max_batch_codewords));
            ln->info_off.alloc(static_cast<size_t>(c.max_batch_codewords));
            ln->chunks_done.alloc(static_cast<size_t>(L->max_req));
            ln->late.alloc(static_cast<size_t>(L->max_req));
            ln->iqbuf.alloc(2 * static_cast<size_t>(std::max<long long>(c.max_batch_iq_samples, 1)));
            check_cuda(cudaStreamCreateWithFlags(&ln->stream, cudaStreamNonBlocking), "cudaStreamCreate(loop)");
            check_cuda(cudaStreamCreateWithFlags(&ln->side, cudaStreamNonBlocking), "cudaStreamCreate(loop side)");
            check_cuda(cudaEventCreateWithFlags(&ln->bp_done, cudaEventDisableTiming), "cudaEventCreate(loop)");
            check_cuda(cudaEventCreateWithFlags(&ln->early_done, cudaEventDisableTiming), "cudaEventCreate(loop)");
            L->lanes.push_back(std::move(ln));
        }
        std::lock_guard<std::mutex> lock(g_mu);
        const unsigned long long h = ++g_next;
        g_loops[h] = L;
        *out_handle = h;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_devloop_stop(unsigned long long handle, int wait_ms)
{
    return guarded([&]() -> int {
        auto L = get(handle);
        std::lock_guard<std::mutex> lock(L->mu);
        check_cuda(cudaSetDevice(L->device), "cudaSetDevice");
        store_release(&L->hs.h->stop, 1);
        const auto deadline = Clock::now() + std::chrono::milliseconds(std::max(wait_ms, 1));
        while (!L->all_done()) {
            if (Clock::now() > deadline) throw std::runtime_error("the device loop did not stop in time");
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
        for (auto& ln : L->lanes) ln->launched = false;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_devloop_destroy(unsigned long long handle)
{
    return guarded([&]() -> int {
        std::shared_ptr<Loop> L;
        {
            std::lock_guard<std::mutex> lock(g_mu);
            auto it = g_loops.find(handle);
            if (it == g_loops.end()) throw InvalidArgument("invalid device-loop handle");
            L = it->second;
        }
        if (sicc_devloop_stop(handle, 10000) != CUDA_OSD_STATUS_OK) throw std::runtime_error(last_error());
        std::lock_guard<std::mutex> lock(g_mu);
        g_loops.erase(handle);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_devloop_add_code(unsigned long long handle, const sicc_engine_code_t* code, int* out_code_id)
{
    return guarded([&]() -> int {
        auto L = get(handle);
        std::lock_guard<std::mutex> lock(L->mu);
        if (L->recorded) throw InvalidArgument("codes must be added before the loop starts");
        if (!code || !out_code_id) throw InvalidArgument("null argument");
        check_cuda(cudaSetDevice(L->device), "cudaSetDevice");
        int id = -1;
        for (auto& ln : L->lanes) {  // every lane's engine holds the same codes under the same ids
            int lid = -1;
            if (sicc_engine_add_code(ln->engine, code, &lid) != CUDA_OSD_STATUS_OK) throw InvalidArgument(last_error());
            if (id >= 0 && lid != id) throw std::runtime_error("the lanes' engines gave different code ids");
            id = lid;
        }
        L->codes.push_back(CodeDims{code->n, code->n - code->m});
        *out_code_id = id;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_devloop_add_phy(unsigned long long handle, const sicc_pipe_config_t* config, const sicc_pipe_tables_t* tables,
                         int frame_stride, int code_id, int* out_phy_id)
{
    return guarded([&]() -> int {
        auto L = get(handle);
        std::lock_guard<std::mutex> lock(L->mu);
        if (L->recorded) throw InvalidArgument("profiles must be added before the loop starts");
        if (!config || !tables || !out_phy_id) throw InvalidArgument("null argument");
        if (L->cfg.max_batch_frames <= 0) throw InvalidArgument("the loop was created without frame budgets");
        if (static_cast<int>(L->phys.size()) >= kMaxPhys) throw InvalidArgument("at most 8 OFDM profiles");
        if (code_id < 0 || code_id >= static_cast<int>(L->codes.size())) throw InvalidArgument("invalid code id");
        check_cuda(cudaSetDevice(L->device), "cudaSetDevice");
        auto ph = std::make_unique<PhyHost>();
        sicc_pipe_config_t c = *config;
        c.max_batch_frames = L->cfg.max_batch_frames;
        if (sicc_pipe_create(&c, 1, &ph->pipe) != CUDA_OSD_STATUS_OK) throw InvalidArgument(last_error());
        if (sicc_pipe_upload_static_tables(ph->pipe, tables) != CUDA_OSD_STATUS_OK) throw InvalidArgument(last_error());
        PipeDims dims{};
        if (pipe_dims(ph->pipe, &dims) != CUDA_OSD_STATUS_OK) throw std::runtime_error(last_error());
        const CodeDims cd = L->codes[code_id];
        if (dims.code_n != cd.n || dims.code_k != cd.k)
            throw InvalidArgument("the profile's code_n / code_k differ from the registered code");
        if (frame_stride < dims.frame_samples) throw InvalidArgument("frame_stride must hold a whole frame");
        if (static_cast<long long>(frame_stride) > L->cfg.max_batch_iq_samples)
            throw InvalidArgument("one frame exceeds the iteration's IQ budget");
        ph->stride = frame_stride;
        ph->code_id = code_id;
        ph->blocks = dims.blocks;
        const int F = L->cfg.max_batch_frames;
        if (pipe_gather_scratch(ph->pipe, frame_stride, F, &ph->scratch_bytes, &ph->ticket_offset, &ph->ticket_bytes) !=
            CUDA_OSD_STATUS_OK)
            throw std::runtime_error(last_error());
        for (auto& ln : L->lanes) {  // the search and demodulator's buffers, one set per lane
            auto lp = std::make_unique<LanePhy>();
            lp->frame_off.alloc(static_cast<size_t>(F));
            lp->llr_frame_off.alloc(static_cast<size_t>(F));
            lp->sync.alloc(static_cast<size_t>(F) * sizeof(sicc_pipe_sync_record_t));
            lp->scratch.alloc(ph->scratch_bytes);
            ln->phys.push_back(std::move(lp));
        }
        L->phys.push_back(std::move(ph));
        *out_phy_id = static_cast<int>(L->phys.size()) - 1;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_devloop_start(unsigned long long handle)
{
    return guarded([&]() -> int {
        auto L = get(handle);
        std::lock_guard<std::mutex> lock(L->mu);
        if (L->codes.empty()) throw InvalidArgument("no code registered");
        check_cuda(cudaSetDevice(L->device), "cudaSetDevice");
        L->ensure_running();
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_devloop_submit(unsigned long long handle, const sicc_request_t* request, unsigned long long* out_request_id)
{
    return guarded([&]() -> int {
        auto L = get(handle);
        if (!request) throw InvalidArgument("null request");
        const sicc_request_t& r = *request;
        if (r.kind != 0 && r.kind != 1) throw InvalidArgument("request kind must be 0 (LLRs) or 1 (OFDM IQ)");
        std::lock_guard<std::mutex> lock(L->mu);
        if (r.protection != 0 && r.protection != 1) throw InvalidArgument("protection must be 0 or 1");
        if (r.count <= 0) throw InvalidArgument("count must be positive");
        int code_id = r.code_id, stride = 0, codewords = r.count;
        if (r.kind == 1) {
            if (r.phy_id < 0 || r.phy_id >= static_cast<int>(L->phys.size())) throw InvalidArgument("invalid profile id");
            const PhyHost& ph = *L->phys[r.phy_id];
            code_id = ph.code_id;
            stride = ph.stride;
            codewords = r.count * ph.blocks;
            if (r.count > L->cfg.max_batch_frames ||
                static_cast<long long>(r.count) * stride > L->cfg.max_batch_iq_samples)
                throw InvalidArgument("request larger than one iteration's frame budget");
        } else if (code_id < 0 || code_id >= static_cast<int>(L->codes.size())) {
            throw InvalidArgument("invalid code id");
        }
        const CodeDims cd = L->codes[code_id];
        if (codewords > L->cfg.max_batch_codewords ||
            static_cast<long long>(codewords) * cd.n > L->cfg.max_batch_llr_floats)
            throw InvalidArgument("request larger than one iteration's budget");
        check_cuda(cudaSetDevice(L->device), "cudaSetDevice");
        const void* in = device_address(r.host_input);
        void* out = const_cast<void*>(device_address(r.host_info));
        if (!in || !out)
            throw InvalidArgument("host_input and host_info must be page-locked host memory the GPU can address");
        if (L->req_tail - load_acquire(&L->ds.h->req_head) >= static_cast<unsigned long long>(L->mask) + 1) {
            ++L->stats.busy_rejections;
            set_last_error("request ring full");
            return static_cast<int>(SICC_SERVER_BUSY);  // an int like every other return of this lambda
        }
        const unsigned long long id = L->next_id++;
        ReqEntry e{};
        e.id = id;
        e.tag = r.tag;
        e.in = static_cast<const float*>(in);
        e.out = static_cast<unsigned char*>(out);
        e.kind = r.kind;
        e.code_id = code_id;
        e.phy_id = r.kind == 1 ? r.phy_id : 0;
        e.count = r.count;
        e.protection = r.protection;
        e.n = cd.n;
        e.k = cd.k;
        e.codewords = codewords;
        e.stride = stride;
        {
            std::lock_guard<std::mutex> plock(L->pending_mu);
            L->pending[id] = Pending{Clock::now()};
        }
        L->ring.h[L->req_tail & L->mask] = e;
        ++L->req_tail;
        store_release(&L->hs.h->req_tail, L->req_tail);  // the entry is complete before the tail moves
        ++L->stats.submitted;
        L->ensure_running();
        if (out_request_id) *out_request_id = id;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_devloop_poll(unsigned long long handle, int max, sicc_completion_t* out, int* out_count, int wait_us)
{
    return guarded([&]() -> int {
        auto L = get(handle);
        if (!out || !out_count || max <= 0) throw InvalidArgument("bad arguments");
        *out_count = 0;
        std::lock_guard<std::mutex> plock(L->poll_mu);
        const auto deadline = Clock::now() + std::chrono::microseconds(std::max(wait_us, 0));
        unsigned spins = 0;
        for (;;) {
            // lanes finish out of order: take every record whose sequence number is set, then move the
            // head over the consumed prefix (which frees those slots for the lanes)
            const unsigned long long reserved = load_acquire(&L->ds.h->cmp_reserved);
            std::unique_lock<std::mutex> pend(L->pending_mu, std::defer_lock);
            for (unsigned long long s = L->cmp_head; s < reserved && *out_count < max; ++s) {
                const size_t slot = static_cast<size_t>(s & L->mask);
                if (L->taken[slot]) continue;
                const CmpEntry& c = L->cring.h[slot];
                if (load_acquire(&c.seq) != s + 1) continue;
                L->taken[slot] = 1;
                if (!pend.owns_lock()) pend.lock();
                sicc_completion_t& o = out[(*out_count)++];
                o = sicc_completion_t{};
                o.request_id = c.id;
                o.tag = c.tag;
                o.status = c.status;
                o.codewords = c.codewords;
                o.failed_codewords = c.failed;
                o.osd_codewords = c.osd;
                const auto now = Clock::now();
                auto it = L->pending.find(c.id);
                if (it != L->pending.end()) {
                    o.latency_us = us_between(it->second.t_submit, now);
                    o.queue_us = std::max(0.0, us_between(it->second.t_submit, L->host_time(c.t_start_ns)));
                    o.launch_us = o.queue_us;
                    L->pending.erase(it);
                }
                o.batch_gpu_us = static_cast<double>(c.t_done_ns - c.t_start_ns) * 1e-3;
                ++L->completed;
            }
            if (pend.owns_lock()) pend.unlock();
            while (L->cmp_head < reserved && L->taken[L->cmp_head & L->mask]) {
                L->taken[L->cmp_head & L->mask] = 0;
                ++L->cmp_head;
            }
            store_release(&L->hs.h->cmp_head, L->cmp_head);
            if (*out_count > 0) break;
            // nothing to report: a lane that failed is reported, and lanes that ended with requests still
            // in the ring are launched again (when no submit holds the loop's lock)
            if ((++spins & 127) == 0 &&
                load_acquire(&L->hs.h->req_tail) != load_acquire(&L->ds.h->req_head)) {
                bool stopped = false;
                for (auto& ln : L->lanes)
                    if (ln->launched.load() && ln->graph_done()) stopped = true;
                if (stopped) {
                    std::unique_lock<std::mutex> lock(L->mu, std::try_to_lock);
                    if (lock.owns_lock()) L->ensure_running();
                }
            }
            if (Clock::now() >= deadline) break;
            std::this_thread::sleep_for(std::chrono::microseconds(5));
        }
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_devloop_get_stats(unsigned long long handle, sicc_devloop_stats_t* out)
{
    return guarded([&]() -> int {
        auto L = get(handle);
        if (!out) throw InvalidArgument("null argument");
        std::lock_guard<std::mutex> lock(L->mu);
        *out = L->stats;
        {
            std::lock_guard<std::mutex> plock(L->pending_mu);
            out->completed = L->completed;
        }
        out->iterations = out->codewords = out->busy_iterations = 0;
        out->running = 0;
        for (size_t l = 0; l < L->lanes.size(); ++l) {
            const LaneSide& s = L->lane_side.h[l];
            out->iterations += load_acquire(&s.iterations);
            out->codewords += load_acquire(&s.codewords);
            out->busy_iterations += load_acquire(&s.busy_iterations);
            if (L->lanes[l]->launched && !L->lanes[l]->graph_done()) ++out->running;
        }
        out->lanes = static_cast<int>(L->lanes.size());
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_devloop_replay(unsigned long long handle, const sicc_request_t* requests, const double* arrival_us, int count,
                        sicc_completion_t* out_completions, double* out_wall_us)
{
    return guarded([&]() -> int {
        auto L = get(handle);
        if (!requests || !arrival_us || !out_completions || count <= 0) throw InvalidArgument("bad arguments");
        // completions can come back before the submitting thread has recorded the id; they wait in
        // `early` until it has (both threads hold idx_mu around index, early, out_completions, t_last)
        std::map<unsigned long long, int> index;
        std::map<unsigned long long, sicc_completion_t> early;
        std::vector<double> late(count, 0.0);
        std::mutex idx_mu;
        std::atomic<int> done{0};
        std::atomic<bool> failed{false};
        std::string error;
        const auto t0 = Clock::now();
        Clock::time_point t_last = t0;
        auto finish = [&](int pos, const sicc_completion_t& c) {
            out_completions[pos] = c;
            out_completions[pos].latency_us += late[pos];
            out_completions[pos].queue_us += late[pos];
            out_completions[pos].launch_us += late[pos];
            t_last = Clock::now();
            done.fetch_add(1);
        };
        std::thread collector([&] {
            std::vector<sicc_completion_t> buf(256);
            const auto give_up = [&] { return Clock::now() - t_last > std::chrono::seconds(30); };
            while (done.load() < count && !failed.load()) {
                int got = 0;
                if (sicc_devloop_poll(handle, 256, buf.data(), &got, 1000) != CUDA_OSD_STATUS_OK) {
                    error = last_error();
                    failed.store(true);
                    break;
                }
                std::lock_guard<std::mutex> lock(idx_mu);
                for (int i = 0; i < got; ++i) {
                    auto it = index.find(buf[i].request_id);
                    if (it != index.end()) finish(it->second, buf[i]);
                    else early.emplace(buf[i].request_id, buf[i]);
                }
                if (got == 0 && give_up()) {
                    sicc_devloop_stats_t s{};
                    sicc_devloop_get_stats(handle, &s);
                    error = "no completion for 30 s (requests submitted " + std::to_string(s.submitted) +
                            ", admitted " + std::to_string(load_acquire(&L->ds.h->req_head)) + ", completed " +
                            std::to_string(s.completed) + "; loop iterations " + std::to_string(s.iterations) +
                            ", lanes running " + std::to_string(s.running) + ")";
                    failed.store(true);
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
            while ((st = sicc_devloop_submit(handle, &requests[i], &id)) == SICC_SERVER_BUSY && !failed.load())
                std::this_thread::sleep_for(std::chrono::microseconds(20));
            if (st != CUDA_OSD_STATUS_OK) {
                error = last_error();
                failed.store(true);
                break;
            }
            late[i] = us_between(due, Clock::now());
            std::lock_guard<std::mutex> lock(idx_mu);
            index[id] = i;
            auto e = early.find(id);
            if (e != early.end()) {
                finish(i, e->second);
                early.erase(e);
            }
        }
        collector.join();
        if (failed.load()) throw std::runtime_error("replay failed: " + error);
        if (out_wall_us) *out_wall_us = us_between(t0, t_last);
        return CUDA_OSD_STATUS_OK;
    });
}

}  // extern "C"
