// Mixed-code batched decoding (include/sicc_engine.h).
//
// One batch holds codewords of several codes.  prepare_kernel groups them by
// code (a counting sort in the queue order: widest layers, then largest cost
// first) and sizes the work units; bp_mixed_kernel then runs persistently in
// three phases, each unit decoded with its code's layered schedule (the same
// arithmetic as bp_layered_kernel, so results are bit-exact with the
// single-code decoders):
//   1. groups of 4 warps take codewords of codes whose layers are >= 128 rows
//      wide (one codeword per group, synchronised by a named barrier);
//   2. groups of 2 warps take codes with 64-row layers;
//   3. single warps take units of up to 32/G codewords of the narrower codes,
//      G lanes each.
// Wide codewords thus run on up to 128 lanes (a 2048-bit codeword is not
// serialised on one warp) and every warp's shared-memory slot only has to
// hold a quarter of the largest code's state.  Codewords whose syndrome fails
// go to one OSD launch that reads each item's code tables.
#include "../../include/sicc_engine.h"
#include "bp_device.cuh"
#include "bp_kernels.h"
#include "code_plan.h"
#include "engine_internal.h"
#include "tune_internal.h"
#include "../../include/sicc_tune.h"

#include <algorithm>
#include <cfloat>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

namespace sicc {

namespace {

constexpr int kMaxCodes = 64;

struct CodeDesc {
    int n, k, num_layers, width, maxdeg, group, rows_per_lane, max_iter;
    int warps;        // 4 or 2: decoded by a group of that many warps (group = 32 * warps); 1: narrow
    float alpha, beta;
    int route_osd;
    int slot_floats;  // shared-memory floats per codeword slot
    const int* vars;  // [num_layers][maxdeg][width]
};

struct MixedIO {
    const CodeDesc* codes;
    const uint8_t* code_of;      // [count]
    const float* llr;
    const long long* llr_off;    // [count]
    uint8_t* info;
    const long long* info_off;   // [count]
    uint8_t* success;
    uint8_t* used_osd;
    uint8_t* iterations;
    const uint8_t* protect;      // [count] 1 = OSD fallback allowed (null: every codeword of an OSD code)
    const int* order;            // [count] codeword indices grouped by code, queue order
    const int* q_code;           // [K] code id at queue position q
    const int* q_start;          // [K+1] first entry of queue position q in `order`
    const int* q_units;          // [K+1] first unit of queue position q
    int K;
    int* work4;                  // unit counters of the three phases
    int* work2;
    int* work1;
    const int* bounds;           // [2] end of the 4-warp units, end of the 2-warp units
    float* best;                 // [warps][best_slots][n_max] best-syndrome posteriors (global scratch)
    int best_slots;              // codewords a warp holds at once (32 / group of the narrowest code, >= 1)
    int n_max;
    float* osd_llr;              // compact rows of the codewords handed to OSD
    int* osd_index;              // [items] codeword of each row
    long long* osd_rowoff;       // [items] float offset of each row in osd_llr
    int* osd_count;
    unsigned long long* osd_floats;  // row allocation counter
};

// prepare: counts per code, queue-ordered starts, units, scatter into `order`.
__global__ void __launch_bounds__(1024)
prepare_kernel(const uint8_t* __restrict__ code_of, int count_max, const int* __restrict__ count_ptr,
               const int* __restrict__ q_code, int K, const int* __restrict__ per_warp,
               const int* __restrict__ q_warps, int* __restrict__ order, int* __restrict__ q_start,
               int* __restrict__ q_units, int* __restrict__ counters)
{
    // the batch's codewords: a launch argument, or (a launch recorded once and replayed over
    // batches of different sizes) a device count, at most count_max
    const int count = count_ptr ? min(max(*count_ptr, 0), count_max) : count_max;
    __shared__ int cnt[kMaxCodes], fill[kMaxCodes], pos_of_code[kMaxCodes];
    for (int i = threadIdx.x; i < kMaxCodes; i += blockDim.x) {
        cnt[i] = 0;
        fill[i] = 0;
    }
    __syncthreads();
    // codewords whose code id is not registered are left out (their outputs are not written)
    for (int i = threadIdx.x; i < count; i += blockDim.x)
        if (code_of[i] < K) atomicAdd(&cnt[code_of[i]], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0, u = 0, end4 = 0, end2 = 0;
        for (int q = 0; q < K; ++q) {
            const int c = q_code[q];
            pos_of_code[c] = s;
            q_start[q] = s;
            q_units[q] = u;
            s += cnt[c];
            u += (cnt[c] + per_warp[c] - 1) / per_warp[c];
            if (q_warps[q] >= 4) end4 = u;  // the queue holds the 4-warp codes first, then the 2-warp ones
            if (q_warps[q] >= 2) end2 = u;
        }
        q_start[K] = s;
        q_units[K] = u;
        if (end2 < end4) end2 = end4;
        counters[0] = 0;       // 4-warp unit counter
        counters[1] = 0;       // OSD items
        *reinterpret_cast<unsigned long long*>(counters + 2) = 0ull;  // OSD row floats
        counters[4] = end4;    // 2-warp unit counter
        counters[5] = end2;    // single-warp unit counter
        counters[6] = end4;
        counters[7] = end2;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < count; i += blockDim.x) {
        const int c = code_of[i];
        if (c < K) order[pos_of_code[c] + atomicAdd(&fill[c], 1)] = i;
    }
}

// Variable of slot j of row rs in layer L.
__device__ __forceinline__ int row_var(const CodeDesc& d, int L, int j, int rs)
{
    return __ldg(d.vars + (L * d.maxdeg + j) * d.width + rs);
}

// Empty edge slots (short rows, row slots past a layer's last row) point at a
// dummy posterior held at +inf right after a slot's posteriors: such an edge
// never sets a row's minima, argmin or sign and never flips a parity, and its
// update leaves it at +inf, so the row loops need no per-edge test.
__device__ __forceinline__ int dummy_var(const CodeDesc& d) { return (d.n + 3) & ~3; }

// Variable of slot j (j < D) of row rs in layer L, or the dummy.
__device__ __forceinline__ int slot_var(const CodeDesc& d, int L, int j, int rs)
{
    const int v = (j < d.maxdeg) ? row_var(d, L, j, rs) : -1;
    return v >= 0 ? v : dummy_var(d);
}

// Unsatisfied checks among the rows gl, gl + G, ... of every layer; a row's
// D slots are loaded together (no chain of dependent loads per slot).
template <int D>
__device__ __forceinline__ int lane_syndrome(const CodeDesc& d, const float* app, int gl, int G)
{
    int cnt = 0;
    for (int L = 0; L < d.num_layers; ++L) {
        for (int rr = 0; rr < d.rows_per_lane; ++rr) {
            const int rs = gl + rr * G;
            unsigned par = 0;
#pragma unroll
            for (int j0 = 0; j0 < D; j0 += 8) {  // groups of 8 slots bound the registers held
                int v[8];
#pragma unroll
                for (int x = 0; x < 8; ++x) v[x] = (j0 + x < D) ? slot_var(d, L, j0 + x, rs) : 0;
#pragma unroll
                for (int x = 0; x < 8; ++x)
                    if (j0 + x < D) par ^= (app[v[x]] < 0.0f) ? 1u : 0u;
            }
            cnt += static_cast<int>(par);
        }
    }
    return cnt;
}

template <int D>
__device__ __forceinline__ int mixed_syndrome(const CodeDesc& d, const float* app, int gl, int G, unsigned gmask)
{
    return static_cast<int>(__reduce_add_sync(gmask, static_cast<unsigned>(lane_syndrome<D>(d, app, gl, G))));
}

// Layered normalized min-sum update of row rs of layer L: extrinsic inputs
// from the posteriors and the row's compressed previous messages, new
// (alpha*min1, alpha*min2, argmin, signs), posteriors updated in place.
template <int D>
__device__ __forceinline__ void update_row(const CodeDesc& d, float* app, float* r1, float* r2, unsigned* meta, int L,
                                           int rs)
{
    const int ridx = L * d.width + rs;
    int v[D];
#pragma unroll
    for (int j = 0; j < D; ++j) v[j] = slot_var(d, L, j, rs);
    if (v[0] == dummy_var(d)) return;  // row slot past the layer's last row
    const float o1 = r1[ridx], o2 = r2[ridx];
    const unsigned om = meta[ridx];
    float qv[D];
    float m1 = FLT_MAX, m2 = FLT_MAX;
    int idx = 0;
    unsigned neg = 0;
#pragma unroll
    for (int j = 0; j < D; ++j) {
        const float qj = __fsub_rn(app[v[j]], rebuild(o1, o2, om, j));
        qv[j] = qj;
        neg |= (qj < 0.0f) ? (1u << j) : 0u;
        const float a = fabsf(qj);
        // first strict minimum and second minimum (magnitudes are >= +0)
        idx = (a < m1) ? j : idx;
        m2 = fminf(m2, fmaxf(m1, a));
        m1 = fminf(m1, a);
    }
    const unsigned tot = static_cast<unsigned>(__popc(neg)) & 1u;
    const float n1 = nms_mag(d.alpha, d.beta, m1);
    const float n2 = nms_mag(d.alpha, d.beta, m2);
    // new message signs (tot ^ sign of the input) for every slot in one step; bits of empty
    // slots are never read back
    const unsigned nm = ((neg ^ (0u - tot)) & 0x07FFFFFFu) | (static_cast<unsigned>(idx) << 27);
#pragma unroll
    for (int j = 0; j < D; ++j) {
        const unsigned sgn = (nm >> j) & 1u;
        const float mag = (j == idx) ? n2 : n1;
        app[v[j]] = __fadd_rn(qv[j], sgn ? -mag : mag);
    }
    r1[ridx] = n1;
    r2[ridx] = n2;
    meta[ridx] = nm;
}

__device__ __forceinline__ void group_sync(int id, int threads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

// One codeword on a group of W warps (named barrier `bar`).
template <int D, int W>
__device__ __forceinline__ void wide_unit(const MixedIO& io, const CodeDesc& d, int cw, float* app, float* best, int g,
                                          int gl, int bar, int* s_red, unsigned long long* s_off)
{
    constexpr int G = W * 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = d.n;
    const int mp = d.num_layers * d.width;
    float* r1 = app + dummy_var(d) + 4;
    float* r2 = r1 + mp;
    unsigned* meta = reinterpret_cast<unsigned*>(r2 + mp);
    const float* src = io.llr + io.llr_off[cw];
    if (gl == 0) app[dummy_var(d)] = __int_as_float(0x7f800000);  // +inf
    for (int i = gl; i < n; i += G) {
        const float x = __ldcs(src + i);
        app[i] = x;
        if (d.route_osd) best[i] = x;
    }
    for (int r = gl; r < mp; r += G) {
        r1[r] = 0.0f;
        r2[r] = 0.0f;
        meta[r] = 0u;
    }
    group_sync(bar, G);
    auto syndrome = [&]() -> int {
        const unsigned c = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(lane_syndrome<D>(d, app, gl, G)));
        if (lane == 0) s_red[g * W + (warp % W)] = static_cast<int>(c);
        group_sync(bar, G);
        int tot = 0;
#pragma unroll
        for (int i = 0; i < W; ++i) tot += s_red[g * W + i];
        return tot;
    };
    int best_w = syndrome();
    int iter = 0;
    for (;;) {
        for (int L = 0; L < d.num_layers; ++L) {
            for (int rr = 0; rr < d.rows_per_lane; ++rr) update_row<D>(d, app, r1, r2, meta, L, gl + rr * G);
            group_sync(bar, G);
        }
        const int w = syndrome();
        ++iter;
        if (d.route_osd && (w < best_w || w == 0)) {
            for (int i = gl; i < n; i += G) best[i] = app[i];
            group_sync(bar, G);  // copied before the next layer rewrites the posteriors
        }
        if (w < best_w) best_w = w;
        if (w == 0 || iter >= d.max_iter) {
            const bool ok = (w == 0);
            if (gl == 0) {
                if (io.success) io.success[cw] = ok ? 1 : 0;
                if (io.iterations) io.iterations[cw] = static_cast<uint8_t>(iter);
                if (io.used_osd) io.used_osd[cw] = 0;
            }
            uint8_t* dst = io.info + io.info_off[cw];
            for (int i = gl; i < d.k; i += G) dst[i] = app[i] < 0.0f ? 1 : 0;
            if (!ok && d.route_osd && (io.protect == nullptr || io.protect[cw])) {
                if (gl == 0) {
                    const int it = atomicAdd(io.osd_count, 1);
                    const unsigned long long off = atomicAdd(io.osd_floats, static_cast<unsigned long long>(n));
                    io.osd_index[it] = cw;
                    io.osd_rowoff[it] = static_cast<long long>(off);
                    s_off[g] = off;
                }
                group_sync(bar, G);
                float* o = io.osd_llr + s_off[g];
                for (int i = gl; i < n; i += G) o[i] = best[i];
            }
            return;
        }
    }
}

// Phase of groups of W warps (W = 4: named barriers 1-2, W = 2: 3-6), one
// codeword per group at a time from `counter`, up to unit `u_end`.  The
// group scalars (s_unit, s_red, s_off) are the phase's own: a group of the
// 2-warp phase can start while a 4-warp group of the same CTA is still
// running, so the two phases must not share them.
template <int D, int W>
__device__ void wide_phase(const MixedIO& io, float* smem_f, int warp_floats, int* counter, int u_end, int* s_unit,
                           int* s_red, unsigned long long* s_off)
{
    constexpr int G = W * 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = warp / W;
    const int gl = (warp % W) * 32 + lane;
    const int bar = (W == 4 ? 1 : 3) + g;
    float* app = smem_f + static_cast<size_t>(g * W) * warp_floats;
    const int gwarp0 = blockIdx.x * (blockDim.x >> 5) + g * W;
    float* best = io.best + static_cast<size_t>(gwarp0) * io.best_slots * io.n_max;
    for (;;) {
        if (gl == 0) s_unit[g] = atomicAdd(counter, 1);
        group_sync(bar, G);
        const int u = s_unit[g];
        if (u >= u_end) break;  // the same value for the whole group
        int q = 0;
        while (q + 1 < io.K && u >= io.q_units[q + 1]) ++q;
        const CodeDesc d = io.codes[io.q_code[q]];
        const int cw = io.order[io.q_start[q] + (u - io.q_units[q])];
        // row loops unrolled to the closest D above the code's row degree
        if (d.maxdeg <= 10) wide_unit<10, W>(io, d, cw, app, best, g, gl, bar, s_red, s_off);
        else if (d.maxdeg <= 12) wide_unit<12, W>(io, d, cw, app, best, g, gl, bar, s_red, s_off);
        else if (d.maxdeg <= 14) wide_unit<14, W>(io, d, cw, app, best, g, gl, bar, s_red, s_off);
        else wide_unit<D, W>(io, d, cw, app, best, g, gl, bar, s_red, s_off);
        group_sync(bar, G);  // the slot and s_unit are rewritten by the next unit
    }
}

// Up to 32/G codewords of one code on one warp, G lanes each.
template <int D>
__device__ __forceinline__ void narrow_unit(const MixedIO& io, const CodeDesc& d, int q, int u, float* wbase, int gwarp)
{
    const int lane = threadIdx.x & 31;
    const int G = d.group;
    const int per = 32 / G;
    const int sub = lane / G;
    const int gl = lane & (G - 1);
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (sub * G));
    const int local = (u - io.q_units[q]) * per + sub;
    bool active = local < io.q_start[q + 1] - io.q_start[q];
    const int cw = active ? io.order[io.q_start[q] + local] : 0;
    const int n = d.n;
    const int n_pad = (n + 3) & ~3;
    const int mp = d.num_layers * d.width;
    float* app = wbase + sub * d.slot_floats;
    float* r1 = app + n_pad + 4;  // app[n_pad]: the dummy posterior
    float* r2 = r1 + mp;
    unsigned* meta = reinterpret_cast<unsigned*>(r2 + mp);
    float* best = io.best + (static_cast<size_t>(gwarp) * io.best_slots + sub) * io.n_max;
    int iter = 0, best_w = 0;
    if (active) {
        const float* src = io.llr + io.llr_off[cw];
        if (gl == 0) app[n_pad] = __int_as_float(0x7f800000);  // +inf, before the __syncwarp below
        for (int i = gl; i < n; i += G) {
            const float v = __ldcs(src + i);
            app[i] = v;
            if (d.route_osd) best[i] = v;
        }
        for (int r = gl; r < mp; r += G) {
            r1[r] = 0.0f;
            r2[r] = 0.0f;
            meta[r] = 0u;
        }
        __syncwarp(gmask);
        best_w = mixed_syndrome<D>(d, app, gl, G, gmask);
    }
    while (__any_sync(0xffffffffu, active)) {
        if (!active) continue;
        for (int L = 0; L < d.num_layers; ++L) {
            for (int rr = 0; rr < d.rows_per_lane; ++rr) update_row<D>(d, app, r1, r2, meta, L, gl + rr * G);
            __syncwarp(gmask);
        }
        const int w = mixed_syndrome<D>(d, app, gl, G, gmask);
        ++iter;
        if (d.route_osd && (w < best_w || w == 0)) {
            for (int i = gl; i < n; i += G) best[i] = app[i];
            __syncwarp(gmask);
        }
        if (w < best_w) best_w = w;
        if (w == 0 || iter >= d.max_iter) {
            const bool ok = (w == 0);
            if (gl == 0) {
                if (io.success) io.success[cw] = ok ? 1 : 0;
                if (io.iterations) io.iterations[cw] = static_cast<uint8_t>(iter);
                if (io.used_osd) io.used_osd[cw] = 0;
            }
            uint8_t* dst = io.info + io.info_off[cw];
            for (int i = gl; i < d.k; i += G) dst[i] = app[i] < 0.0f ? 1 : 0;
            if (!ok && d.route_osd && (io.protect == nullptr || io.protect[cw])) {
                unsigned long long off = 0ull;
                if (gl == 0) {
                    const int it = atomicAdd(io.osd_count, 1);
                    off = atomicAdd(io.osd_floats, static_cast<unsigned long long>(n));
                    io.osd_index[it] = cw;
                    io.osd_rowoff[it] = static_cast<long long>(off);
                }
                const unsigned lo = __shfl_sync(gmask, static_cast<unsigned>(off), sub * G);
                const unsigned hi = __shfl_sync(gmask, static_cast<unsigned>(off >> 32), sub * G);
                float* o = io.osd_llr + ((static_cast<unsigned long long>(hi) << 32) | lo);
                for (int i = gl; i < n; i += G) o[i] = best[i];
            }
            active = false;
        }
    }
    __syncwarp();
}

template <int D>
__global__ void __launch_bounds__(256)
bp_mixed_kernel(MixedIO io, int warp_floats)
{
    extern __shared__ __align__(16) float smem_f[];
    __shared__ int s_unit4[2], s_unit2[4];
    __shared__ int s_red4[8], s_red2[8];
    __shared__ unsigned long long s_off4[2], s_off2[4];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;

    // phases 1 and 2: codewords of wide codes on groups of 4, then 2 warps
    wide_phase<D, 4>(io, smem_f, warp_floats, io.work4, io.bounds[0], s_unit4, s_red4, s_off4);
    wide_phase<D, 2>(io, smem_f, warp_floats, io.work2, io.bounds[1], s_unit2, s_red2, s_off2);

    // phase 3: one warp per unit
    float* wbase = smem_f + static_cast<size_t>(warp) * warp_floats;
    const int gwarp = blockIdx.x * (blockDim.x >> 5) + warp;
    const int total_units = io.q_units[io.K];
    for (;;) {
        int u = 0;
        if (lane == 0) u = atomicAdd(io.work1, 1);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= total_units) break;
        int q = 0;
        while (q + 1 < io.K && u >= io.q_units[q + 1]) ++q;
        const CodeDesc d = io.codes[io.q_code[q]];
        if (d.maxdeg <= 10) narrow_unit<10>(io, d, q, u, wbase, gwarp);
        else if (d.maxdeg <= 12) narrow_unit<12>(io, d, q, u, wbase, gwarp);
        else if (d.maxdeg <= 14) narrow_unit<14>(io, d, q, u, wbase, gwarp);
        else narrow_unit<D>(io, d, q, u, wbase, gwarp);
    }
}

struct EngineCode {
    std::unique_ptr<DeviceCode> code;
    CodeDesc desc{};
    bool osd = false;    // OSD by the warp kernel (n <= 256, k <= 128)
    bool osd_h = false;  // OSD by the large-code kernel
    long long cost = 0;
    uint64_t fingerprint = 0;  // key of the code's tuned warps per codeword
};

// Warps that decode one codeword of a code with layers of `width` rows: 4 (128 lanes)
// for layers of >= 128 rows, 2 (64 lanes) for 64-row layers, else one warp.
int default_code_warps(int width)
{
    if (width >= 128 && width % 128 == 0) return 4;
    if (width >= 64 && width % 64 == 0) return 2;
    return 1;
}

bool code_warps_allowed(int width, int warps)
{
    return warps == 1 || ((warps == 2 || warps == 4) && width >= 32 * warps && width % (32 * warps) == 0);
}

// Lanes and rows per lane of a code decoded by `warps` warps per codeword, and the
// shared-memory floats of one codeword slot.
void set_code_warps(EngineCode& ec, int warps)
{
    const LayeredView& lv = ec.code->layered_view();
    CodeDesc& d = ec.desc;
    if (!code_warps_allowed(lv.width, warps)) throw InvalidArgument("warps per codeword must be 1, 2 or 4 and divide the layer width in 32-lane units");
    d.warps = warps;
    d.group = lv.group;
    d.rows_per_lane = lv.rows_per_lane;
    if (warps > 1) {
        d.group = 32 * warps;
        d.rows_per_lane = lv.width / d.group;
    }
    const int n_pad = (d.n + 3) & ~3;
    // posteriors, the dummy edge's +inf (padded to 4 floats), then the row messages
    int sf = (n_pad + 4 + 3 * d.num_layers * d.width + 3) & ~3;
    sf = pad_slot_stride(sf, d.group);
    d.slot_floats = sf;
}

struct Engine {
    sicc_engine_config_t cfg{};
    int device = 0;
    std::vector<EngineCode> codes;
    int n_max = 0, k_max = 0, maxdeg = 0, osd_nmax = 0, osd_kmax = 0;
    OsdHBounds h_cls[kOsdHClasses];  // large-code OSD launch bounds, by class
    int warps_per_cta = 0, ctas = 0;
    // device state
    CodeDesc* d_codes = nullptr;
    OsdView* d_views = nullptr;
    OsdHView* d_hviews = nullptr;
    int* d_per_warp = nullptr;
    int* d_q_warps = nullptr;   // [K] warps per codeword of the code at each queue position
    int* d_q_code = nullptr;
    int* d_q_start = nullptr;
    int* d_q_units = nullptr;
    int* d_order = nullptr;
    // [0] 4-warp units, [1] OSD items, [2..3] OSD row floats (64-bit), [4] 2-warp units,
    // [5] single-warp units, [6..7] ends of the 4-warp and 2-warp units
    int* d_counters = nullptr;
    long long* d_osd_rowoff = nullptr;
    int* d_osd_index = nullptr;
    float* d_osd_llr = nullptr;
    float* d_best = nullptr;
    size_t best_floats = 0;
    bool dirty = true;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaStream_t side[kOsdHClasses - 1] = {};  // large-code OSD classes beside the first
    cudaEvent_t fork = nullptr, join[kOsdHClasses - 1] = {};
    cudaStream_t warp_side = nullptr;  // the short-code (warp) OSD beside the large-code classes
    cudaEvent_t warp_fork = nullptr, warp_join = nullptr;
    bool timed = false;
    std::mutex mu;
    ~Engine()
    {
        for (void* p : {static_cast<void*>(d_codes), static_cast<void*>(d_views), static_cast<void*>(d_hviews),
                        static_cast<void*>(d_per_warp), static_cast<void*>(d_q_warps),
                        static_cast<void*>(d_q_code), static_cast<void*>(d_q_start), static_cast<void*>(d_q_units),
                        static_cast<void*>(d_order), static_cast<void*>(d_counters), static_cast<void*>(d_osd_index),
                        static_cast<void*>(d_osd_llr), static_cast<void*>(d_best), static_cast<void*>(d_osd_rowoff)})
            if (p) cudaFree(p);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        for (auto& e : join)
            if (e) cudaEventDestroy(e);
        for (auto& q : side)
            if (q) cudaStreamDestroy(q);
        if (warp_fork) cudaEventDestroy(warp_fork);
        if (warp_join) cudaEventDestroy(warp_join);
        if (warp_side) cudaStreamDestroy(warp_side);
    }
    bool has_osd_h() const
    {
        for (const auto& c : h_cls)
            if (!c.empty()) return true;
        return false;
    }

    // shared-memory floats per warp: a narrow code's 32/G slots, or a W-warp
    // group's slot spread over its W warps
    int warp_floats() const
    {
        int w = 0;
        for (const auto& c : codes) {
            const int need = c.desc.warps > 1 ? (c.desc.slot_floats + c.desc.warps - 1) / c.desc.warps
                                              : (32 / c.desc.group) * c.desc.slot_floats;
            w = std::max(w, need);
        }
        return (w + 3) & ~3;
    }

    // Uploads the code descriptors and the queue order after codes change.
    void commit()
    {
        if (!dirty) return;
        const int K = static_cast<int>(codes.size());
        std::vector<CodeDesc> descs(K);
        std::vector<OsdView> views(K);
        std::vector<OsdHView> hviews(K);
        std::vector<int> per(K), qcode(K), qwarps(K);
        for (int c = 0; c < K; ++c) {
            descs[c] = codes[c].desc;
            per[c] = codes[c].desc.warps > 1 ? 1 : 32 / codes[c].desc.group;
            views[c] = codes[c].osd ? codes[c].code->osd_view() : OsdView{};
            hviews[c] = codes[c].osd_h ? codes[c].code->osd_h_view() : OsdHView{};
            qcode[c] = c;
        }
        // queue order: 4-warp codes, 2-warp codes, then the rest; within each, most expensive first
        std::stable_sort(qcode.begin(), qcode.end(), [&](int a, int b) {
            if (codes[a].desc.warps != codes[b].desc.warps) return codes[a].desc.warps > codes[b].desc.warps;
            return codes[a].cost > codes[b].cost;
        });
        for (int q = 0; q < K; ++q) qwarps[q] = codes[qcode[q]].desc.warps;
        auto up = [](auto*& dst, const auto& v) {
            using T = std::remove_reference_t<decltype(v[0])>;
            if (dst) cudaFree(dst);
            check_cuda(cudaMalloc(&dst, std::max<size_t>(v.size(), 1) * sizeof(T)), "cudaMalloc(engine)");
            check_cuda(cudaMemcpy(dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload(engine)");
        };
        up(d_codes, descs);
        up(d_views, views);
        up(d_hviews, hviews);
        up(d_per_warp, per);
        up(d_q_warps, qwarps);
        up(d_q_code, qcode);
        dirty = false;
    }
};

std::mutex g_mu;
std::map<unsigned long long, std::shared_ptr<Engine>> g_engines;
unsigned long long g_next = 0x9100;

std::shared_ptr<Engine> get(unsigned long long h)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_engines.find(h);
    if (it == g_engines.end()) throw InvalidArgument("invalid engine handle");
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

template <int D>
void launch_mixed(Engine& e, const MixedIO& io, cudaStream_t st)
{
    const int wf = e.warp_floats();
    // whole groups of 4 warps (the wide phases split a CTA into groups of 4 and 2 warps)
    int warps = e.warps_per_cta == 4 ? 4 : 8;
    if (static_cast<size_t>(warps) * wf * sizeof(float) > 200 * 1024) warps = 4;
    const size_t smem = static_cast<size_t>(warps) * wf * sizeof(float);
    if (smem > 227 * 1024) throw InvalidArgument("a registered code is too large for the mixed kernel");
    check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(bp_mixed_kernel<D>), smem),
               "cudaFuncSetAttribute(bp_mixed)");
    int ctas = e.ctas;
    if (ctas <= 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bp_mixed_kernel<D>, warps * 32, smem) !=
                cudaSuccess ||
            per_sm <= 0)
            per_sm = 1;
        ctas = per_sm * device_sm_count();
    }
    // a warp holds one codeword of a wide code, or 32 / group codewords of a narrow one
    int slots = 1;
    for (const auto& c : e.codes)
        if (c.desc.warps == 1) slots = std::max(slots, 32 / c.desc.group);
    const size_t need = static_cast<size_t>(ctas) * warps * slots * static_cast<size_t>(e.n_max);
    if (need > e.best_floats) {
        if (e.d_best) cudaFree(e.d_best);
        check_cuda(cudaMalloc(&e.d_best, need * sizeof(float)), "cudaMalloc(best)");
        e.best_floats = need;
    }
    MixedIO m = io;
    m.best = e.d_best;
    m.best_slots = slots;
    bp_mixed_kernel<D><<<ctas, warps * 32, smem, st>>>(m, wf);
    check_cuda(cudaGetLastError(), "bp_mixed_kernel launch");
}

}  // namespace
}  // namespace sicc

using namespace sicc;

extern "C" {

int sicc_engine_create(const sicc_engine_config_t* config, unsigned long long* out_handle)
{
    return guarded([&] {
        if (!config || !out_handle) throw InvalidArgument("null argument");
        *out_handle = 0;
        if (config->max_codewords <= 0 || config->max_llr_floats <= 0)
            throw InvalidArgument("max_codewords and max_llr_floats must be positive");
        if (config->max_codes <= 0 || config->max_codes > kMaxCodes) throw InvalidArgument("max_codes must be 1..64");
        auto e = std::make_shared<Engine>();
        e->cfg = *config;
        check_cuda(cudaGetDevice(&e->device), "cudaGetDevice");
        check_cuda(cudaMalloc(&e->d_order, sizeof(int) * config->max_codewords), "cudaMalloc(order)");
        check_cuda(cudaMalloc(&e->d_q_start, sizeof(int) * (kMaxCodes + 1)), "cudaMalloc(q_start)");
        check_cuda(cudaMalloc(&e->d_q_units, sizeof(int) * (kMaxCodes + 1)), "cudaMalloc(q_units)");
        check_cuda(cudaMalloc(&e->d_counters, sizeof(int) * 16), "cudaMalloc(counters)");  // [8..11]: OSD work
        check_cuda(cudaMalloc(&e->d_osd_rowoff, sizeof(long long) * config->max_codewords), "cudaMalloc(osd rows)");
        check_cuda(cudaMalloc(&e->d_osd_index, sizeof(int) * config->max_codewords), "cudaMalloc(osd index)");
        check_cuda(cudaMalloc(&e->d_osd_llr, sizeof(float) * config->max_llr_floats), "cudaMalloc(osd rows)");
        for (auto& ev : e->ev) check_cuda(cudaEventCreate(&ev), "cudaEventCreate(engine)");
        for (auto& q : e->side) check_cuda(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking), "cudaStreamCreate(engine side)");
        check_cuda(cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming), "cudaEventCreate(engine fork)");
        for (auto& ev : e->join) check_cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate(engine join)");
        check_cuda(cudaStreamCreateWithFlags(&e->warp_side, cudaStreamNonBlocking), "cudaStreamCreate(engine warp OSD)");
        check_cuda(cudaEventCreateWithFlags(&e->warp_fork, cudaEventDisableTiming), "cudaEventCreate(engine warp fork)");
        check_cuda(cudaEventCreateWithFlags(&e->warp_join, cudaEventDisableTiming), "cudaEventCreate(engine warp join)");
        std::lock_guard<std::mutex> lock(g_mu);
        *out_handle = ++g_next;
        g_engines[*out_handle] = e;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_engine_destroy(unsigned long long handle)
{
    return guarded([&] {
        std::shared_ptr<Engine> e;
        {
            std::lock_guard<std::mutex> lock(g_mu);
            auto it = g_engines.find(handle);
            if (it == g_engines.end()) throw InvalidArgument("invalid engine handle");
            e = it->second;
            g_engines.erase(it);
        }
        cudaSetDevice(e->device);
        cudaDeviceSynchronize();
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_engine_add_code(unsigned long long handle, const sicc_engine_code_t* code, int* out_code_id)
{
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (!code || !out_code_id || !code->row_ptr || !code->col_ind) throw InvalidArgument("null argument");
        if (static_cast<int>(e->codes.size()) >= e->cfg.max_codes) throw InvalidArgument("engine holds max_codes codes");
        if (code->max_iterations < 1 || code->max_iterations > 255) throw InvalidArgument("max_iterations must be 1..255");
        check_cuda(cudaSetDevice(e->device), "cudaSetDevice");
        const bool want_osd = code->osd_order >= 0;
        OsdSettings os;
        if (want_osd) {
            os.order = code->osd_order;
            os.max_flip_positions = code->osd_max_flip_positions;
            os.max_tests = code->osd_max_tests;
        }
        // short codes: the warp OSD kernel (generator tables); longer ones: the CTA kernel on H
        const bool warp_osd = want_osd && code->n <= 256 && code->n - code->m <= 128;
        EngineCode ec;
        ec.code = std::make_unique<DeviceCode>(code->n, code->m, code->row_ptr, code->col_ind, kFlatLayered, nullptr,
                                               0, warp_osd, os);
        if (want_osd && !warp_osd) {
            std::vector<uint64_t> parity;
            int words = 0, kk = 0;
            if (!systematic_parity(code->n, code->m, code->row_ptr, code->col_ind, parity, words, kk))
                throw InvalidArgument("OSD needs a full-rank code with the information bits first (systematic-front)");
            ec.code->set_osd_h(os);
        }
        const LayeredView& lv = ec.code->layered_view();
        if (lv.maxdeg > 16) throw InvalidArgument("the mixed kernel supports row degree <= 16");
        CodeDesc& d = ec.desc;
        d.n = code->n;
        d.k = ec.code->k();
        d.num_layers = lv.num_layers;
        d.width = lv.width;
        d.maxdeg = lv.maxdeg;
        d.group = lv.group;
        d.rows_per_lane = lv.rows_per_lane;
        d.max_iter = code->max_iterations;
        d.alpha = code->normalization;
        d.beta = code->offset;
        d.route_osd = want_osd ? 1 : 0;
        d.vars = lv.vars;
        Fingerprint fp;
        fp.add(code->n);
        fp.add(code->m);
        fp.add(code->row_ptr, static_cast<size_t>(code->m) + 1);
        fp.add(code->col_ind, static_cast<size_t>(code->row_ptr[code->m]));
        fp.add(code->max_iterations);
        fp.add_float(code->normalization);
        fp.add_float(code->offset);
        ec.fingerprint = fp.h;
        int warps = default_code_warps(lv.width);
        std::vector<int> cached;
        if (tune_cache_get(tune_key("engine-code", fp.h), cached) && cached.size() == 1 &&
            code_warps_allowed(lv.width, cached[0]))
            warps = cached[0];  // tuned earlier for this code on this device
        set_code_warps(ec, warps);
        ec.osd = warp_osd;
        ec.osd_h = want_osd && !warp_osd;
        ec.cost = static_cast<long long>(ec.code->edges()) * d.max_iter;
        e->n_max = std::max(e->n_max, d.n);
        e->k_max = std::max(e->k_max, d.k);
        if (ec.osd) {
            e->osd_nmax = std::max(e->osd_nmax, d.n);
            e->osd_kmax = std::max(e->osd_kmax, d.k);
        }
        if (ec.osd_h) e->h_cls[osd_h_class(code->m)].add(d.n, code->m, ec.code->osd_h_view().pool, ec.code->edges());
        e->codes.push_back(std::move(ec));
        e->dirty = true;
        *out_code_id = static_cast<int>(e->codes.size()) - 1;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_engine_set_code_warps(unsigned long long handle, int code_id, int warps)
{
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (code_id < 0 || code_id >= static_cast<int>(e->codes.size())) throw InvalidArgument("invalid code id");
        check_cuda(cudaSetDevice(e->device), "cudaSetDevice");
        set_code_warps(e->codes[code_id], warps);
        e->dirty = true;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_engine_get_code_warps(unsigned long long handle, int code_id, int* out_warps)
{
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (code_id < 0 || code_id >= static_cast<int>(e->codes.size()) || !out_warps)
            throw InvalidArgument("invalid code id or null argument");
        *out_warps = e->codes[code_id].desc.warps;
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_engine_set_launch_shape(unsigned long long handle, int warps_per_cta, int ctas)
{
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (warps_per_cta < 0 || warps_per_cta > 8 || ctas < 0) throw InvalidArgument("warps_per_cta must be 0..8");
        e->warps_per_cta = warps_per_cta;
        e->ctas = ctas;
        return CUDA_OSD_STATUS_OK;
    });
}

}  // extern "C"

namespace sicc {

int engine_bounds(unsigned long long handle, int* out_n_max, int* out_k_max)
{
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (out_n_max) *out_n_max = e->n_max;
        if (out_k_max) *out_k_max = e->k_max;
        return CUDA_OSD_STATUS_OK;
    });
}

int engine_code_routes(unsigned long long handle, unsigned char* out_routes, int max_codes, int* out_count)
{
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (!out_routes || !out_count) throw InvalidArgument("null argument");
        const int K = static_cast<int>(e->codes.size());
        if (K > max_codes) throw InvalidArgument("more codes than the output holds");
        for (int i = 0; i < K; ++i) out_routes[i] = e->codes[i].desc.route_osd ? 1 : 0;
        *out_count = K;
        return CUDA_OSD_STATUS_OK;
    });
}

int engine_prepare_capture(unsigned long long handle, int max_codewords)
{
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (e->codes.empty()) throw InvalidArgument("no code registered");
        if (max_codewords <= 0 || max_codewords > e->cfg.max_codewords)
            throw InvalidArgument("codewords must be in 1..max_codewords");
        check_cuda(cudaSetDevice(e->device), "cudaSetDevice");
        e->commit();
        // the mixed kernel's best-posterior scratch for the grid it will use (no allocation later)
        const int wf = e->warp_floats();
        int warps = e->warps_per_cta == 4 ? 4 : 8;
        if (static_cast<size_t>(warps) * wf * sizeof(float) > 200 * 1024) warps = 4;
        const size_t smem = static_cast<size_t>(warps) * wf * sizeof(float);
        check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(bp_mixed_kernel<16>), smem),
                   "cudaFuncSetAttribute(bp_mixed)");
        int ctas = e->ctas;
        if (ctas <= 0) {
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bp_mixed_kernel<16>, warps * 32, smem) !=
                    cudaSuccess ||
                per_sm <= 0)
                per_sm = 1;
            ctas = per_sm * device_sm_count();
        }
        int slots = 1;
        for (const auto& c : e->codes)
            if (c.desc.warps == 1) slots = std::max(slots, 32 / c.desc.group);
        const size_t need = static_cast<size_t>(ctas) * warps * slots * static_cast<size_t>(e->n_max);
        if (need > e->best_floats) {
            if (e->d_best) cudaFree(e->d_best);
            e->d_best = nullptr;
            check_cuda(cudaMalloc(&e->d_best, need * sizeof(float)), "cudaMalloc(best)");
            e->best_floats = need;
        }
        return CUDA_OSD_STATUS_OK;
    });
}

int engine_decode(unsigned long long handle, int codewords, const unsigned char* device_code_ids,
                  const unsigned char* device_protection, const float* device_llr, const long long* device_llr_offsets,
                  unsigned char* device_info, const long long* device_info_offsets, unsigned char* device_success,
                  unsigned char* device_used_osd, unsigned char* device_iterations, cudaStream_t stream,
                  cudaEvent_t bp_done, const int* device_count)
{
    void* cuda_stream = stream;
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (e->codes.empty()) throw InvalidArgument("no code registered");
        if (codewords <= 0 || codewords > e->cfg.max_codewords) throw InvalidArgument("codewords must be in 1..max_codewords");
        if (!device_code_ids || !device_llr || !device_llr_offsets || !device_info || !device_info_offsets)
            throw InvalidArgument("null device pointer");
        check_cuda(cudaSetDevice(e->device), "cudaSetDevice");
        e->commit();
        cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
        const int K = static_cast<int>(e->codes.size());
        check_cuda(cudaEventRecord(e->ev[0], st), "cudaEventRecord");
        prepare_kernel<<<1, 1024, 0, st>>>(device_code_ids, codewords, device_count, e->d_q_code, K, e->d_per_warp,
                                           e->d_q_warps, e->d_order, e->d_q_start, e->d_q_units, e->d_counters);
        check_cuda(cudaGetLastError(), "prepare_kernel launch");
        check_cuda(cudaEventRecord(e->ev[1], st), "cudaEventRecord");
        MixedIO io{};
        io.codes = e->d_codes;
        io.code_of = device_code_ids;
        io.llr = device_llr;
        io.llr_off = device_llr_offsets;
        io.info = device_info;
        io.info_off = device_info_offsets;
        io.success = device_success;
        io.used_osd = device_used_osd;
        io.iterations = device_iterations;
        io.protect = device_protection;
        io.order = e->d_order;
        io.q_code = e->d_q_code;
        io.q_start = e->d_q_start;
        io.q_units = e->d_q_units;
        io.K = K;
        io.work4 = e->d_counters;
        io.work2 = e->d_counters + 4;
        io.work1 = e->d_counters + 5;
        io.bounds = e->d_counters + 6;
        io.n_max = e->n_max;
        io.osd_llr = e->d_osd_llr;
        io.osd_index = e->d_osd_index;
        io.osd_rowoff = e->d_osd_rowoff;
        io.osd_count = e->d_counters + 1;
        io.osd_floats = reinterpret_cast<unsigned long long*>(e->d_counters + 2);
        launch_mixed<16>(*e, io, st);
        check_cuda(cudaEventRecord(e->ev[2], st), "cudaEventRecord");
        if (bp_done) check_cuda(cudaEventRecord(bp_done, st), "cudaEventRecord(bp done)");
        if (e->osd_nmax > 0 || e->has_osd_h()) {
            OsdIO oio{};
            oio.llr = e->d_osd_llr;
            oio.index = e->d_osd_index;
            oio.count_ptr = e->d_counters + 1;
            oio.out_info = device_info;
            oio.used_osd = device_used_osd;
            oio.views = e->d_views;
            oio.hviews = e->d_hviews;
            oio.code_of = device_code_ids;
            oio.row_off = e->d_osd_rowoff;
            oio.info_off = device_info_offsets;
            oio.work = e->d_counters + 8;
            oio.work_h = e->d_counters + 9;
            // short codes (one warp per codeword) beside the long-code classes (one CTA per
            // codeword): the kernels take disjoint codewords of the work list
            const bool both = e->osd_nmax > 0 && e->has_osd_h();
            if (e->osd_nmax > 0) {
                OsdView shape{};
                shape.n = e->osd_nmax;
                shape.k = e->osd_kmax;
                cudaStream_t ws = st;
                if (both) {
                    check_cuda(cudaEventRecord(e->warp_fork, st), "cudaEventRecord(warp OSD fork)");
                    check_cuda(cudaStreamWaitEvent(e->warp_side, e->warp_fork, 0), "cudaStreamWaitEvent(warp OSD)");
                    ws = e->warp_side;
                }
                launch_osd(shape, oio, codewords, ws);
                if (both) check_cuda(cudaEventRecord(e->warp_join, ws), "cudaEventRecord(warp OSD join)");
            }
            if (e->has_osd_h()) launch_osd_h(e->h_cls, oio, codewords, st, e->side, e->fork, e->join);
            if (both) check_cuda(cudaStreamWaitEvent(st, e->warp_join, 0), "cudaStreamWaitEvent(warp OSD join)");
        }
        check_cuda(cudaEventRecord(e->ev[3], st), "cudaEventRecord");
        e->timed = true;
        return CUDA_OSD_STATUS_OK;
    });
}

}  // namespace sicc

extern "C" {

int sicc_engine_decode_device_protected(unsigned long long handle, int codewords, const unsigned char* device_code_ids,
                                        const unsigned char* device_protection, const float* device_llr,
                                        const long long* device_llr_offsets, unsigned char* device_info,
                                        const long long* device_info_offsets, unsigned char* device_success,
                                        unsigned char* device_used_osd, unsigned char* device_iterations,
                                        void* cuda_stream)
{
    return engine_decode(handle, codewords, device_code_ids, device_protection, device_llr, device_llr_offsets,
                         device_info, device_info_offsets, device_success, device_used_osd, device_iterations,
                         static_cast<cudaStream_t>(cuda_stream), nullptr);
}

int sicc_engine_osd_device(unsigned long long handle, int codewords, const unsigned char* device_code_ids,
                           const float* device_llr, const long long* device_llr_offsets, unsigned char* device_info,
                           const long long* device_info_offsets, unsigned char* device_used_osd, float* device_metric,
                           void* cuda_stream)
{
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (e->codes.empty()) throw InvalidArgument("no code registered");
        if (codewords <= 0 || codewords > e->cfg.max_codewords) throw InvalidArgument("codewords must be in 1..max_codewords");
        if (!device_code_ids || !device_llr || !device_llr_offsets || !device_info || !device_info_offsets)
            throw InvalidArgument("null device pointer");
        check_cuda(cudaSetDevice(e->device), "cudaSetDevice");
        e->commit();
        cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
        OsdIO oio{};
        oio.llr = device_llr;
        oio.count = codewords;
        oio.out_info = device_info;
        oio.out_metric = device_metric;
        oio.used_osd = device_used_osd;
        oio.views = e->d_views;
        oio.hviews = e->d_hviews;
        oio.code_of = device_code_ids;
        oio.llr_off = device_llr_offsets;
        oio.info_off = device_info_offsets;
        if (e->osd_nmax > 0) {
            OsdView shape{};
            shape.n = e->osd_nmax;
            shape.k = e->osd_kmax;
            launch_osd(shape, oio, codewords, st);
        }
        if (e->has_osd_h()) launch_osd_h(e->h_cls, oio, codewords, st, e->side, e->fork, e->join);
        return CUDA_OSD_STATUS_OK;
    });
}

int sicc_engine_decode_device(unsigned long long handle, int codewords, const unsigned char* device_code_ids,
                              const float* device_llr, const long long* device_llr_offsets, unsigned char* device_info,
                              const long long* device_info_offsets, unsigned char* device_success,
                              unsigned char* device_used_osd, unsigned char* device_iterations, void* cuda_stream)
{
    return sicc_engine_decode_device_protected(handle, codewords, device_code_ids, nullptr, device_llr,
                                               device_llr_offsets, device_info, device_info_offsets, device_success,
                                               device_used_osd, device_iterations, cuda_stream);
}

int sicc_engine_last_ms(unsigned long long handle, float* out_prepare_ms, float* out_bp_ms, float* out_osd_ms)
{
    return guarded([&] {
        auto e = get(handle);
        std::lock_guard<std::mutex> lock(e->mu);
        if (!e->timed) throw InvalidArgument("no decode has run");
        check_cuda(cudaEventSynchronize(e->ev[3]), "cudaEventSynchronize");
        float a = 0, b = 0, c = 0;
        cudaEventElapsedTime(&a, e->ev[0], e->ev[1]);
        cudaEventElapsedTime(&b, e->ev[1], e->ev[2]);
        cudaEventElapsedTime(&c, e->ev[2], e->ev[3]);
        if (out_prepare_ms) *out_prepare_ms = a;
        if (out_bp_ms) *out_bp_ms = b;
        if (out_osd_ms) *out_osd_ms = c;
        return CUDA_OSD_STATUS_OK;
    });
}

// Coordinate search on the caller's batch: codes in decreasing BP cost, each tried at every
// allowed warps per codeword (kept when the mixed BP kernel gets at least 1% faster), then the
// engine's warps per CTA.  Trials decode with every codeword's protection at BP only, so OSD
// time stays out of the comparison; each trial is one warm-up and `reps` timed decodes.
int sicc_engine_autotune(unsigned long long handle, int codewords, const unsigned char* device_code_ids,
                         const float* device_llr, const long long* device_llr_offsets, unsigned char* device_info,
                         const long long* device_info_offsets, int reps, float* out_default_ms, float* out_tuned_ms)
{
    return guarded([&] {
        auto e = get(handle);
        if (!device_code_ids || !device_llr || !device_llr_offsets || !device_info || !device_info_offsets)
            throw InvalidArgument("null device pointer");
        if (codewords <= 0 || codewords > e->cfg.max_codewords) throw InvalidArgument("codewords out of range");
        if (reps < 1 || reps > 50) throw InvalidArgument("reps must be in 1..50");
        check_cuda(cudaSetDevice(e->device), "cudaSetDevice");
        struct Bytes {  // per-codeword scratch of the trials, freed on every exit
            uint8_t* p = nullptr;
            ~Bytes() { if (p) cudaFree(p); }
        } protect, ok, used, iters;
        for (Bytes* b : {&protect, &ok, &used, &iters})
            check_cuda(cudaMalloc(&b->p, static_cast<size_t>(codewords)), "cudaMalloc(autotune)");
        check_cuda(cudaMemset(protect.p, 0, codewords), "clear protection");
        cudaStream_t st = nullptr;
        check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate(tune)");
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamDestroy(s); }
        } guard{st};

        auto time_bp = [&]() -> float {
            std::vector<float> ms;
            for (int r = 0; r <= reps; ++r) {
                if (engine_decode(handle, codewords, device_code_ids, protect.p, device_llr, device_llr_offsets,
                                  device_info, device_info_offsets, ok.p, used.p, iters.p, st, nullptr) !=
                    CUDA_OSD_STATUS_OK)
                    throw std::runtime_error(std::string("autotune decode: ") + last_error());
                std::lock_guard<std::mutex> lock(e->mu);
                check_cuda(cudaEventSynchronize(e->ev[2]), "cudaEventSynchronize");
                float t = 0.0f;
                check_cuda(cudaEventElapsedTime(&t, e->ev[1], e->ev[2]), "cudaEventElapsedTime");
                if (r > 0) ms.push_back(t);
            }
            return median_of(ms);
        };
        auto set_warps = [&](int c, int w) {
            std::lock_guard<std::mutex> lock(e->mu);
            set_code_warps(e->codes[c], w);
            e->dirty = true;
        };

        const float default_ms = time_bp();
        float best = default_ms;
        std::vector<int> order;
        {
            std::lock_guard<std::mutex> lock(e->mu);
            for (int c = 0; c < static_cast<int>(e->codes.size()); ++c) order.push_back(c);
            std::sort(order.begin(), order.end(),
                      [&](int a, int b) { return e->codes[a].cost > e->codes[b].cost; });
        }
        for (int c : order) {
            int width = 0, keep = 0;
            {
                std::lock_guard<std::mutex> lock(e->mu);
                width = e->codes[c].code->layered_view().width;
                keep = e->codes[c].desc.warps;
            }
            for (int w : {1, 2, 4}) {
                if (w == keep || !code_warps_allowed(width, w)) continue;
                set_warps(c, w);
                const float t = time_bp();
                if (t < 0.99f * best) {
                    best = t;
                    keep = w;
                } else {
                    set_warps(c, keep);
                }
            }
        }
        int wpc_keep = 0;
        {
            std::lock_guard<std::mutex> lock(e->mu);
            wpc_keep = e->warps_per_cta;
        }
        for (int wpc : {4, 8}) {
            if (wpc == (wpc_keep == 0 ? 8 : wpc_keep)) continue;
            {
                std::lock_guard<std::mutex> lock(e->mu);
                e->warps_per_cta = wpc;
            }
            const float t = time_bp();
            if (t < 0.99f * best) {
                best = t;
                wpc_keep = wpc;
            }
        }
        {
            std::lock_guard<std::mutex> lock(e->mu);
            e->warps_per_cta = wpc_keep;
            for (const auto& c : e->codes) tune_cache_put(tune_key("engine-code", c.fingerprint), {c.desc.warps});
        }
        if (out_default_ms) *out_default_ms = default_ms;
        if (out_tuned_ms) *out_tuned_ms = best;
        return CUDA_OSD_STATUS_OK;
    });
}

}  // extern "C"
