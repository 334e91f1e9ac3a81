// Belief propagation for long codes (DVB-S2 N16200 / N64800 class) whose
// decoder state does not fit one CTA's shared memory.
//
// One CTA of 512 threads decodes one codeword at a time and takes the next
// from a global counter when it stops.  The posteriors live in shared memory
// when they fit (n <= ~50k); for longer codes the layered kernel keeps the
// first 56,320 in shared memory and the rest in the CTA's slice of a global
// scratch block (the flooding kernel keeps them all there); the compressed check messages (alpha*min1, alpha*min2, argmin,
// signs per row) and, for the flooding schedule, the variable-to-check
// messages of every edge live in that slice too.  A slice is touched by one
// CTA only, so it stays in L2 when the grid's slices fit there (the launcher
// sizes the grid for that).
//
//   layered (schedules 2, 3): the rows of a layer touch disjoint variables,
//     so the CTA's threads update them in parallel, one barrier per layer;
//     the per-row arithmetic is the shared-memory layered kernel's
//     (bp_kernels.cu), operation for operation.
//   flooding (schedules 0, 1): check phase over all rows, variable phase
//     over all columns (the reference CPU decoder, uhd_ldpc_ofdm_link.cpp:
//     3013-3094, with the MB damping of cpu_bp_osd_decode.m:180-183), the
//     shared-memory flooding kernel's arithmetic with CTA-wide loops.
//
// Results, stopping rule (zero syndrome or the iteration cap), best-syndrome
// tracking and the OSD hand-off are those of the shared-memory kernels, so
// both give the same bits for a code that fits either.
#include "bp_device.cuh"
#include "bp_kernels.h"

#include <algorithm>
#include <cfloat>

namespace sicc {

namespace {

constexpr int kWideThreads = 512;
constexpr int kWideWarps = kWideThreads / 32;

// CTA-wide sum; every thread gets the total.  `red` holds kWideWarps ints.
__device__ __forceinline__ int cta_sum(int v, int* red)
{
    v = static_cast<int>(__reduce_add_sync(0xffffffffu, static_cast<unsigned>(v)));
    __syncthreads();  // the previous reduction's reads are done
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
#pragma unroll
    for (int i = 0; i < kWideWarps; ++i) t += red[i];
    return t;
}

__device__ __forceinline__ unsigned cta_min(unsigned v, int* red)
{
    v = __reduce_min_sync(0xffffffffu, v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = static_cast<int>(v);
    __syncthreads();
    unsigned t = 0xffffffffu;
#pragma unroll
    for (int i = 0; i < kWideWarps; ++i) t = min(t, static_cast<unsigned>(red[i]));
    return t;
}

// Outputs of a finished codeword (the shared-memory kernels' finalize step).
template <class App>
__device__ void wide_finish(const BpParams& p, const BpIO& io, int c, int n, int w, int iter, const App& app,
                            const float* best, bool track_best, int* red, int* s_slot)
{
    const int tid = threadIdx.x;
    bool accept = (w == 0);
    if (accept && p.min_abs_accept > 0.0f) {
        unsigned mn = 0x7f800000u;
        for (int i = tid; i < n; i += kWideThreads) mn = min(mn, __float_as_uint(fabsf(app.ld(i))));
        accept = __uint_as_float(cta_min(mn, red)) >= p.min_abs_accept;
    }
    const bool route = !accept && p.route_failures_to_osd && io.osd_llr != nullptr;
    if (tid == 0) {
        if (io.success) io.success[c] = accept ? 1 : 0;
        if (io.iterations) io.iterations[c] = static_cast<uint8_t>(iter);
        if (io.used_osd) io.used_osd[c] = 0;
        if (route) *s_slot = atomicAdd(io.osd_count, 1);
    }
    if (io.out_bits) {
        uint8_t* dst = io.out_bits + static_cast<size_t>(c) * io.out_stride;
        for (int i = tid; i < io.out_len; i += kWideThreads) dst[i] = app.ld(i) < 0.0f ? 1 : 0;
    }
    if (io.app_out) {
        float* dst = io.app_out + static_cast<size_t>(c) * n;
        for (int i = tid; i < n; i += kWideThreads) dst[i] = app.ld(i);
    }
    __syncthreads();  // s_slot
    if (route) {
        const int s = *s_slot;
        float* dst = io.osd_llr + static_cast<size_t>(s) * n;
        for (int i = tid; i < n; i += kWideThreads) dst[i] = track_best ? best[i] : app.ld(i);
        if (tid == 0) io.osd_index[s] = c;
    }
}

// Next codeword of this CTA (all threads get it).
__device__ __forceinline__ int wide_next(const BpIO& io, int* s_next)
{
    __syncthreads();  // every thread is done with the current codeword's state
    if (threadIdx.x == 0) *s_next = static_cast<int>(gridDim.x) + atomicAdd(io.work_counter, 1);
    __syncthreads();
    return *s_next;
}

// Posteriors of the layered wide kernel: those of variables below `split` in shared
// memory, the rest in the CTA's global slice (L2), so a code a little too long for shared
// memory keeps most of its posterior gathers on chip.
struct SplitApp {
    float* s;   // shared memory, variables [0, split)
    float* g;   // global slice, indexed by the variable (entries below split unused)
    int split;
    __device__ __forceinline__ float ld(int v) const { return v < split ? s[v] : g[v]; }
    __device__ __forceinline__ void st(int v, float x) const
    {
        if (v < split) s[v] = x;
        else g[v] = x;
    }
};

// Rows a thread updates together in a layer: their loads are all issued before the
// first store (the rows of a layer touch disjoint variables), so the latencies overlap.
// Two for row degrees up to 16; one above, where the registers would spill.
template <int D>
constexpr int row_batch() { return D <= 16 ? 2 : 1; }

// Empty edge slots of short rows point at a dummy posterior (+inf: never a row's minimum,
// argmin or sign, never a parity flip, and left at +inf by its update), so the edge loops
// test only `j < cv.maxdeg`, the same for every thread.  Above D = 8 the slots keep -1 and
// a per-edge test: the dummy form's registers would spill there.
template <int D>
constexpr bool dummy_slots() { return D <= 8; }

// Layered update of rows rs0, rs0 + kWideThreads, ... (kRowBatch of them, those below
// `rows`) of layer L, whose messages start at row `first` of the layer-ordered message
// arrays: the shared-memory layered kernel's per-row arithmetic (bp_kernels.cu).
template <int D, int kRowBatch = row_batch<D>()>
__device__ __forceinline__ void wide_rows(const LayeredView& cv, const BpParams& p, int L, int rs0, int rows,
                                          int first, const SplitApp& app, int dummy, float* r1, float* r2,
                                          unsigned* meta)
{
    int v[kRowBatch][D];
    float o1[kRowBatch], o2[kRowBatch], x[kRowBatch][D];
    unsigned om[kRowBatch];
#pragma unroll
    for (int b = 0; b < kRowBatch; ++b) {
        const int rs = rs0 + b * kWideThreads;
        const bool live = rs < rows;
        const int* vp = cv.vars + (L * cv.maxdeg) * cv.width + rs;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            const int vj = (live && j < cv.maxdeg) ? __ldg(vp + j * cv.width) : -1;
            v[b][j] = (vj >= 0 || !dummy_slots<D>()) ? vj : dummy;
        }
        const int ridx = first + rs;
        o1[b] = live ? r1[ridx] : 0.0f;
        o2[b] = live ? r2[ridx] : 0.0f;
        om[b] = live ? meta[ridx] : 0u;
    }
    auto used = [&](int b, int j) { return dummy_slots<D>() ? j < cv.maxdeg : v[b][j] >= 0; };
    if constexpr (dummy_slots<D>()) {
#pragma unroll
        for (int b = 0; b < kRowBatch; ++b) {
            if (rs0 + b * kWideThreads < rows) {
#pragma unroll
                for (int j = 0; j < D; ++j) x[b][j] = (j < cv.maxdeg) ? app.ld(v[b][j]) : 0.0f;
            }
        }
    } else {
#pragma unroll
        for (int b = 0; b < kRowBatch; ++b)
#pragma unroll
            for (int j = 0; j < D; ++j) x[b][j] = v[b][j] >= 0 ? app.ld(v[b][j]) : 0.0f;
    }
#pragma unroll
    for (int b = 0; b < kRowBatch; ++b) {
        if (dummy_slots<D>() ? rs0 + b * kWideThreads >= rows : v[b][0] < 0) continue;  // past the layer
        float q[D];
        float m1 = FLT_MAX, m2 = FLT_MAX;
        int idx = 0;
        unsigned neg = 0;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            q[j] = 0.0f;
            if (used(b, j)) {
                const float qj = __fsub_rn(x[b][j], rebuild(o1[b], o2[b], om[b], j));
                q[j] = qj;
                neg |= (qj < 0.0f) ? (1u << j) : 0u;
                const float a = fabsf(qj);
                idx = (a < m1) ? j : idx;
                m2 = fminf(m2, fmaxf(m1, a));
                m1 = fminf(m1, a);
            }
        }
        const unsigned tot = static_cast<unsigned>(__popc(neg)) & 1u;
        const float n1 = nms_mag(p.alpha, p.beta, m1);
        const float n2 = nms_mag(p.alpha, p.beta, m2);
        const unsigned nm = ((neg ^ (0u - tot)) & 0x07FFFFFFu) | (static_cast<unsigned>(idx) << 27);
#pragma unroll
        for (int j = 0; j < D; ++j) {
            if (used(b, j)) {
                const unsigned sg = (nm >> j) & 1u;
                const float mag = (j == idx) ? n2 : n1;
                app.st(v[b][j], __fadd_rn(q[j], sg ? -mag : mag));
            }
        }
        const int ridx = first + rs0 + b * kWideThreads;
        r1[ridx] = n1;
        r2[ridx] = n2;
        meta[ridx] = nm;
    }
}

// Unsatisfied checks among the same rows under hard(app).
template <int D, int kRowBatch = row_batch<D>()>
__device__ __forceinline__ int wide_parity(const LayeredView& cv, int L, int rs0, int rows, const SplitApp& app,
                                           int dummy)
{
    int v[kRowBatch][D];
#pragma unroll
    for (int b = 0; b < kRowBatch; ++b) {
        const int rs = rs0 + b * kWideThreads;
        const bool live = rs < rows;
        const int* vp = cv.vars + (L * cv.maxdeg) * cv.width + rs;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            const int vj = (live && j < cv.maxdeg) ? __ldg(vp + j * cv.width) : -1;
            v[b][j] = (vj >= 0 || !dummy_slots<D>()) ? vj : dummy;
        }
    }
    int cnt = 0;
#pragma unroll
    for (int b = 0; b < kRowBatch; ++b) {
        if (dummy_slots<D>() && rs0 + b * kWideThreads >= rows) continue;  // past the layer
        unsigned par = 0;
#pragma unroll
        for (int j = 0; j < D; ++j)
            if (dummy_slots<D>() ? j < cv.maxdeg : v[b][j] >= 0) par ^= (app.ld(v[b][j]) < 0.0f) ? 1u : 0u;
        cnt += static_cast<int>(par);
    }
    return cnt;
}

}  // namespace

template <int D>
__global__ void __launch_bounds__(kWideThreads, 1)
bp_layered_wide_kernel(LayeredView cv, BpParams p, BpIO io, float* scratch, long long slice, int split,
                       int track_best)
{
    extern __shared__ __align__(16) float s_app[];
    __shared__ int s_red[kWideWarps];
    __shared__ int s_next, s_slot;
    const int tid = threadIdx.x;
    const int n = cv.n, n_pad = (n + 3) & ~3;
    const int mp = cv.m;  // messages of the rows in layer order, packed
    float* g = scratch + static_cast<size_t>(blockIdx.x) * static_cast<size_t>(slice);
    // posteriors [0, split) in shared memory.  The dummy posterior (index n_pad, +inf) takes the
    // empty edge slots of short rows: with split > n_pad it and every posterior are in shared
    // memory, else the slice starts with n_pad posteriors and the dummy (4 floats).
    const bool all_smem = split > n_pad;
    const SplitApp app{s_app, g, split};
    const int dummy = n_pad;
    float* best = all_smem ? g : g + n_pad + 4;
    float* r1 = best + (track_best ? n_pad : 0);
    float* r2 = r1 + mp;
    unsigned* meta = reinterpret_cast<unsigned*>(r2 + mp);

    auto syndrome = [&]() -> int {
        int cnt = 0;
        for (int L = 0; L < cv.num_layers; ++L) {
            const int first = __ldg(cv.layer_start + L), rows = __ldg(cv.layer_start + L + 1) - first;
            for (int rs0 = tid; rs0 < rows; rs0 += row_batch<D>() * kWideThreads)
                cnt += wide_parity<D>(cv, L, rs0, rows, app, dummy);
        }
        return cta_sum(cnt, s_red);
    };

    if (tid == 0) app.st(dummy, __int_as_float(0x7f800000));  // +inf, before the first __syncthreads
    for (int c = blockIdx.x; c < io.count; c = wide_next(io, &s_next)) {
        const float* src = io.llr + static_cast<size_t>(c) * n;
        for (int i = tid; i < n; i += kWideThreads) {
            const float v = __ldcs(src + i);
            app.st(i, v);
            if (track_best) best[i] = v;
        }
        for (int r = tid; r < mp; r += kWideThreads) {
            r1[r] = 0.0f;
            r2[r] = 0.0f;
            meta[r] = 0u;
        }
        __syncthreads();
        int best_w = syndrome();
        int iter = 0, w = 0;
        for (;;) {
            for (int L = 0; L < cv.num_layers; ++L) {
                const int first = __ldg(cv.layer_start + L), rows = __ldg(cv.layer_start + L + 1) - first;
                for (int rs0 = tid; rs0 < rows; rs0 += row_batch<D>() * kWideThreads)
                    wide_rows<D>(cv, p, L, rs0, rows, first, app, dummy, r1, r2, meta);
                __syncthreads();
            }
            w = syndrome();
            ++iter;
            if (track_best && (w < best_w || (w == 0 && best_w == 0))) {
                for (int i = tid; i < n; i += kWideThreads) best[i] = app.ld(i);
                __syncthreads();  // copied before the next layer rewrites the posteriors
            }
            if (w < best_w) best_w = w;
            if (w == 0 || iter >= p.max_iter) break;
        }
        wide_finish(p, io, c, n, w, iter, app, best, track_best != 0, s_red, &s_slot);
    }
}

// Plain posterior array for the flooding kernel's finish step.
struct PlainApp {
    const float* a;
    __device__ __forceinline__ float ld(int v) const { return a[v]; }
};

__global__ void __launch_bounds__(kWideThreads, 1)
bp_flooding_wide_kernel(FloodView cv, BpParams p, BpIO io, float* scratch, long long slice, int app_smem,
                        int track_best)
{
    extern __shared__ __align__(16) float s_app[];
    __shared__ int s_red[kWideWarps];
    __shared__ int s_next, s_slot;
    const int tid = threadIdx.x;
    const int n = cv.n, m = cv.m, E = cv.edges;
    const int n_pad = (n + 3) & ~3, m_pad = (m + 3) & ~3, e_pad = (E + 3) & ~3;
    float* g = scratch + static_cast<size_t>(blockIdx.x) * static_cast<size_t>(slice);
    float* llr = g;
    float* best = llr + n_pad;
    float* q = best + n_pad;
    float* r1 = q + e_pad;
    float* r2 = r1 + m_pad;
    unsigned* meta = reinterpret_cast<unsigned*>(r2 + m_pad);
    float* app = app_smem ? s_app : reinterpret_cast<float*>(meta + m_pad);
    const float keep = __fsub_rn(1.0f, p.damping);

    auto syndrome = [&](const float* x) {
        int cnt = 0;
        for (int r = tid; r < m; r += kWideThreads) {
            unsigned par = 0;
            for (int e = __ldg(cv.row_ptr + r); e < __ldg(cv.row_ptr + r + 1); ++e)
                par ^= (x[__ldg(cv.col_ind + e)] < 0.0f) ? 1u : 0u;
            cnt += static_cast<int>(par);
        }
        return cta_sum(cnt, s_red);
    };
    auto edge_msg = [&](int e) {
        const int r = __ldg(cv.edge_row + e);
        return rebuild(r1[r], r2[r], meta[r], e - __ldg(cv.row_ptr + r));
    };

    for (int c = blockIdx.x; c < io.count; c = wide_next(io, &s_next)) {
        const float* src = io.llr + static_cast<size_t>(c) * n;
        for (int i = tid; i < n; i += kWideThreads) {
            const float v = __ldcs(src + i);
            llr[i] = v;
            app[i] = v;
            if (track_best) best[i] = v;
        }
        __syncthreads();
        for (int e = tid; e < E; e += kWideThreads) q[e] = llr[__ldg(cv.col_ind + e)];
        __syncthreads();
        int best_w = syndrome(llr);
        int iter = 0, w = 0;
        for (;;) {
            // check nodes (L:3033-3060)
            for (int r = tid; r < m; r += kWideThreads) {
                const int e0 = __ldg(cv.row_ptr + r), e1 = __ldg(cv.row_ptr + r + 1);
                float m1 = FLT_MAX, m2 = FLT_MAX;
                int idx = 0;
                unsigned neg = 0;
                for (int e = e0; e < e1; ++e) {
                    const float v = q[e];
                    neg |= (v < 0.0f) ? (1u << (e - e0)) : 0u;
                    const float a = fabsf(v);
                    if (a < m1) {
                        m2 = m1;
                        m1 = a;
                        idx = e - e0;
                    } else if (a < m2) {
                        m2 = a;
                    }
                }
                const unsigned tot = static_cast<unsigned>(__popc(neg)) & 1u;
                unsigned nm = static_cast<unsigned>(idx) << 27;
                for (int j = 0; j < e1 - e0; ++j) nm |= (tot ^ ((neg >> j) & 1u)) << j;
                r1[r] = nms_mag(p.alpha, p.beta, m1);
                r2[r] = nms_mag(p.alpha, p.beta, m2);
                meta[r] = nm;
            }
            __syncthreads();
            // variable nodes (L:3062-3069): llr + sum of messages in row order
            for (int v = tid; v < n; v += kWideThreads) {
                float acc = llr[v];
                for (int j = __ldg(cv.col_ptr + v); j < __ldg(cv.col_ptr + v + 1); ++j)
                    acc = __fadd_rn(acc, edge_msg(__ldg(cv.col_edge + j)));
                app[v] = acc;
            }
            __syncthreads();
            w = syndrome(app);
            ++iter;
            if (track_best && (w < best_w || (w == 0 && best_w == 0))) {
                for (int i = tid; i < n; i += kWideThreads) best[i] = app[i];
            }
            if (w < best_w) best_w = w;
            if (w == 0 || iter >= p.max_iter) break;
            // next variable-to-check messages (L:3076-3081), optional damping
            for (int v = tid; v < n; v += kWideThreads) {
                for (int j = __ldg(cv.col_ptr + v); j < __ldg(cv.col_ptr + v + 1); ++j) {
                    const int e = __ldg(cv.col_edge + j);
                    const float fresh = __fsub_rn(app[v], edge_msg(e));
                    q[e] = (p.damping == 0.0f) ? fresh
                                                : __fadd_rn(__fmul_rn(keep, fresh), __fmul_rn(p.damping, q[e]));
                }
            }
            __syncthreads();
        }
        wide_finish(p, io, c, n, w, iter, PlainApp{app}, best, track_best != 0, s_red, &s_slot);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

namespace {

// Grid of the wide kernels: up to `per_sm` CTAs per SM, no more CTAs than codewords, and
// no more slices than keep the grid's scratch within `l2_budget` bytes (at least one CTA
// per SM).
int wide_grid(int count, int per_sm, size_t slice_bytes)
{
    constexpr size_t l2_budget = size_t(96) << 20;
    const int sms = device_sm_count();
    int ctas = std::max(1, per_sm) * sms;
    const size_t fit = slice_bytes > 0 ? l2_budget / slice_bytes : static_cast<size_t>(ctas);
    ctas = std::min<long long>(ctas, std::max<long long>(sms, static_cast<long long>(fit)));
    return std::max(1, std::min(ctas, count));
}

template <class K, class Launch>
void launch_wide(K kernel, size_t app_bytes, long long slice_floats, int count, cudaStream_t st, Launch&& go)
{
    // posteriors in shared memory when they fit beside the static arrays
    const bool app_smem = app_bytes <= 200 * 1024;
    const size_t smem = app_smem ? app_bytes : 0;
    check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(kernel), smem), "cudaFuncSetAttribute(bp wide)");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWideThreads, smem) != cudaSuccess || per_sm <= 0)
        per_sm = 1;
    const size_t slice_bytes = static_cast<size_t>(slice_floats) * sizeof(float);
    const int ctas = wide_grid(count, per_sm, slice_bytes);
    int device = 0;
    check_cuda(cudaGetDevice(&device), "cudaGetDevice");
    void* scratch = nullptr;
    check_cuda(cudaMallocFromPoolAsync(&scratch, std::max<size_t>(slice_bytes * ctas, 16), scratch_pool(device), st),
               "cudaMallocFromPoolAsync(bp wide)");
    go(ctas, smem, static_cast<float*>(scratch), app_smem ? 1 : 0);
    const cudaError_t err = cudaGetLastError();
    const cudaError_t ferr = cudaFreeAsync(scratch, st);
    check_cuda(err, "bp wide kernel launch");
    check_cuda(ferr, "cudaFreeAsync(bp wide)");
}

template <int D>
void launch_layered_wide_t(const LayeredView& cv, const BpParams& p, const BpIO& io, bool track_best, cudaStream_t st)
{
    const long long n_pad = (cv.n + 3) & ~3;
    const long long mp = cv.m;
    // the posteriors and the dummy posterior (index n_pad, padded to 4 floats)
    const size_t app_bytes = static_cast<size_t>(n_pad + 4) * sizeof(float);
    // posteriors in shared memory: all of them up to 200 KB, else the first 56,320 (220 KB;
    // variables beyond and the dummy stay in the slice)
    constexpr size_t kSmemApp = 200 * 1024, kSplitApp = 220 * 1024;
    const bool all_smem = app_bytes <= kSmemApp;
    const int split = all_smem ? static_cast<int>(n_pad + 4) : static_cast<int>(kSplitApp / sizeof(float));
    const size_t smem = all_smem ? app_bytes : kSplitApp;
    long long slice = (all_smem ? 0 : n_pad + 4) + (track_best ? n_pad : 0) + 3 * mp;
    slice = (slice + 31) & ~31LL;  // 128-byte aligned slices
    const auto kernel = bp_layered_wide_kernel<D>;
    check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(kernel), smem), "cudaFuncSetAttribute(bp wide)");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWideThreads, smem) != cudaSuccess || per_sm <= 0)
        per_sm = 1;
    const size_t slice_bytes = static_cast<size_t>(slice) * sizeof(float);
    const int ctas = wide_grid(io.count, per_sm, slice_bytes);
    int device = 0;
    check_cuda(cudaGetDevice(&device), "cudaGetDevice");
    void* scratch = nullptr;
    check_cuda(cudaMallocFromPoolAsync(&scratch, std::max<size_t>(slice_bytes * ctas, 16), scratch_pool(device), st),
               "cudaMallocFromPoolAsync(bp wide)");
    kernel<<<ctas, kWideThreads, smem, st>>>(cv, p, io, static_cast<float*>(scratch), slice, split, track_best ? 1 : 0);
    const cudaError_t err = cudaGetLastError();
    const cudaError_t ferr = cudaFreeAsync(scratch, st);
    check_cuda(err, "bp wide kernel launch");
    check_cuda(ferr, "cudaFreeAsync(bp wide)");
}

}  // namespace

bool layered_needs_wide(const LayeredView& cv, bool track_best)
{
    const int step = std::max(1, 32 / cv.group);
    return layered_smem_bytes(cv, step, track_best, nullptr) > 227 * 1024;
}

bool flooding_needs_wide(const FloodView& cv) { return flooding_smem_bytes(cv, 1, nullptr) > 227 * 1024; }

void launch_bp_layered_wide(const LayeredView& cv, const BpParams& p, const BpIO& io, cudaStream_t st)
{
    if (io.count <= 0) return;
    const bool track_best = p.route_failures_to_osd && io.osd_llr != nullptr;
    check_cuda(cudaMemsetAsync(io.work_counter, 0, sizeof(int), st), "reset work counter");
    if (cv.maxdeg <= 6) launch_layered_wide_t<6>(cv, p, io, track_best, st);
    else if (cv.maxdeg <= 8) launch_layered_wide_t<8>(cv, p, io, track_best, st);
    else if (cv.maxdeg <= 10) launch_layered_wide_t<10>(cv, p, io, track_best, st);
    else if (cv.maxdeg <= 12) launch_layered_wide_t<12>(cv, p, io, track_best, st);
    else if (cv.maxdeg <= 16) launch_layered_wide_t<16>(cv, p, io, track_best, st);
    else launch_layered_wide_t<27>(cv, p, io, track_best, st);
}

void launch_bp_flooding_wide(const FloodView& cv, const BpParams& p, const BpIO& io, cudaStream_t st)
{
    if (io.count <= 0) return;
    if (cv.maxdeg > 27) throw InvalidArgument("flooding schedule supports row degree <= 27");
    const bool track_best = p.route_failures_to_osd && io.osd_llr != nullptr;
    check_cuda(cudaMemsetAsync(io.work_counter, 0, sizeof(int), st), "reset work counter");
    const long long n_pad = (cv.n + 3) & ~3, m_pad = (cv.m + 3) & ~3, e_pad = (cv.edges + 3) & ~3;
    const size_t app_bytes = static_cast<size_t>(n_pad) * sizeof(float);
    const bool app_smem = app_bytes <= 200 * 1024;
    long long slice = 2 * n_pad + e_pad + 3 * m_pad + (app_smem ? 0 : n_pad);
    slice = (slice + 31) & ~31LL;
    launch_wide(bp_flooding_wide_kernel, app_bytes, slice, io.count, st,
                [&](int ctas, size_t smem, float* scratch, int in_smem) {
                    bp_flooding_wide_kernel<<<ctas, kWideThreads, smem, st>>>(cv, p, io, scratch, slice, in_smem,
                                                                              track_best ? 1 : 0);
                });
}

}  // namespace sicc
