// Normalized min-sum belief-propagation kernels for sm_103a.
//
// Layered kernel (schedules 2, 3): a group of G lanes (G = power of two <= 32)
// owns one codeword at a time.  Lane g handles row slots g, g+G, ... of every
// layer.  The posterior LLRs live in shared memory; each check row keeps its
// messages in compressed form (alpha*min1, alpha*min2, first-argmin position,
// message sign bits), from which the previous message of any edge is rebuilt
// exactly.  Groups run persistently: when a codeword stops (zero syndrome or
// iteration cap) the group writes its outputs, takes the next codeword index
// from a global counter and starts over, so uneven iteration counts never
// leave lanes idle until the queue drains.
//
// Flooding kernel (schedules 0, 1): one warp per codeword, performing the
// operations of the reference CPU decoder (uhd_ldpc_ofdm_link.cpp:3013-3094)
// in the same order, extended with MB-style damping (cpu_bp_osd_decode.m:
// 180-183) and best-syndrome tracking (cpu_bp_osd_decode.m:160-171).
//
// Every floating-point step uses explicit round-to-nearest intrinsics so no
// multiply-add contraction changes a result: the kernels reproduce the
// single-precision oracle (oracle/sicc_oracle.c) bit for bit.
#include "bp_device.cuh"
#include "bp_kernels.h"

#include <algorithm>
#include <cfloat>

namespace sicc {

namespace {

// Group-local syndrome weight of hard(app) under the layered tables; a row's
// D slots are loaded together (no chain of dependent loads per slot).  Empty
// slots hold the dummy posterior's index (+inf: never flips a parity).
template <int D>
__device__ __forceinline__ int layered_syndrome(const LayeredView& cv, const int* s_vars, const float* app,
                                                int gl, int G, unsigned gmask, int dummy)
{
    int cnt = 0;
    for (int L = 0; L < cv.num_layers; ++L) {
        for (int rr = 0; rr < cv.rows_per_lane; ++rr) {
            const int rs = gl + rr * G;
            const int* vp = s_vars + (L * cv.maxdeg) * cv.width + rs;
            unsigned par = 0;
#pragma unroll
            for (int j0 = 0; j0 < D; j0 += 8) {  // groups of 8 slots bound the registers held
                int v[8];
#pragma unroll
                for (int x = 0; x < 8; ++x) {
                    const int j = j0 + x;
                    v[x] = (j < D && j < cv.maxdeg) ? vp[j * cv.width] : dummy;
                }
#pragma unroll
                for (int x = 0; x < 8; ++x)
                    if (j0 + x < D) par ^= (app[v[x]] < 0.0f) ? 1u : 0u;
            }
            cnt += static_cast<int>(par);
        }
    }
    return static_cast<int>(__reduce_add_sync(gmask, static_cast<unsigned>(cnt)));
}

}  // namespace

template <int D>
__global__ void __launch_bounds__(kBpThreads, 3)
bp_layered_kernel(LayeredView cv, BpParams p, BpIO io, int slots_per_cta, int slot_floats, int track_best)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int table = cv.num_layers * cv.maxdeg * cv.width;
    // Empty edge slots (short rows, row slots past a layer's last row) point at a dummy
    // posterior held at +inf behind each slot's posteriors: such an edge never sets a row's
    // minima, argmin or sign and never flips a parity, and its update leaves it at +inf, so
    // the row loops need no per-edge test.
    const int dummy = (cv.n + 3) & ~3;
    int* s_vars = reinterpret_cast<int*>(smem);
    for (int i = threadIdx.x; i < table; i += blockDim.x) {
        const int v = cv.vars[i];
        s_vars[i] = v >= 0 ? v : dummy;
    }
    __syncthreads();

    const int G = cv.group;
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const int sub = lane / G;
    const int slot = threadIdx.x / G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (sub * G));
    const int leader = sub * G;

    const int n = cv.n;
    const int n_pad = (n + 3) & ~3;
    const int mp = cv.num_layers * cv.width;
    float* app = reinterpret_cast<float*>(smem) + ((table + 3) & ~3) + static_cast<size_t>(slot) * slot_floats;
    float* best = app + n_pad + 4;  // only when track_best (app[n_pad] is the dummy)
    float* r1 = app + (track_best ? 2 : 1) * n_pad + 4;
    float* r2 = r1 + mp;
    unsigned* meta = reinterpret_cast<unsigned*>(r2 + mp);

    const int total_groups = gridDim.x * slots_per_cta;
    int c = blockIdx.x * slots_per_cta + slot;
    bool active = c < io.count;
    int iter = 0, best_w = 0;

    auto init = [&](int cw) {
        const float* src = io.llr + static_cast<size_t>(cw) * n;
        if ((n & 3) == 0) {
            const float4* s4 = reinterpret_cast<const float4*>(src);
            for (int i = gl; i < (n >> 2); i += G) {
                const float4 v = __ldcs(s4 + i);
                reinterpret_cast<float4*>(app)[i] = v;
                if (track_best) reinterpret_cast<float4*>(best)[i] = v;
            }
        } else {
            for (int i = gl; i < n; i += G) {
                const float v = __ldcs(src + i);
                app[i] = v;
                if (track_best) best[i] = v;
            }
        }
        for (int r = gl; r < mp; r += G) {
            r1[r] = 0.0f;
            r2[r] = 0.0f;
            meta[r] = 0u;
        }
        __syncwarp(gmask);
        best_w = layered_syndrome<D>(cv, s_vars, app, gl, G, gmask, dummy);
        iter = 0;
    };

    if (gl == 0) app[dummy] = __int_as_float(0x7f800000);  // +inf, before init's __syncwarp
    if (active) init(c);

    while (__any_sync(0xffffffffu, active)) {
        if (active) {
            // ---- one layered iteration ----
            for (int L = 0; L < cv.num_layers; ++L) {
                for (int rr = 0; rr < cv.rows_per_lane; ++rr) {
                    const int rs = gl + rr * G;
                    const int ridx = L * cv.width + rs;
                    const int* vp = s_vars + (L * cv.maxdeg) * cv.width + rs;
                    int v[D];
#pragma unroll
                    for (int j = 0; j < D; ++j) v[j] = (j < cv.maxdeg) ? vp[j * cv.width] : dummy;
                    if (v[0] == dummy) continue;  // row slot past the layer's last row
                    const float o1 = r1[ridx], o2 = r2[ridx];
                    const unsigned om = meta[ridx];
                    float q[D];
                    float m1 = FLT_MAX, m2 = FLT_MAX;
                    int idx = 0;
                    unsigned neg = 0;
#pragma unroll
                    for (int j = 0; j < D; ++j) {
                        const float qj = __fsub_rn(app[v[j]], rebuild(o1, o2, om, j));
                        q[j] = qj;
                        neg |= (qj < 0.0f) ? (1u << j) : 0u;
                        const float a = fabsf(qj);
                        // first strict minimum and second minimum (magnitudes are >= +0)
                        idx = (a < m1) ? j : idx;
                        m2 = fminf(m2, fmaxf(m1, a));
                        m1 = fminf(m1, a);
                    }
                    const unsigned tot = static_cast<unsigned>(__popc(neg)) & 1u;
                    const float n1 = nms_mag(p.alpha, p.beta, m1);
                    const float n2 = nms_mag(p.alpha, p.beta, m2);
                    // new message signs (tot ^ sign of the input) for every slot in one step; bits of
                    // empty slots are never read back
                    const unsigned nm = ((neg ^ (0u - tot)) & 0x07FFFFFFu) | (static_cast<unsigned>(idx) << 27);
#pragma unroll
                    for (int j = 0; j < D; ++j) {
                        const unsigned s = (nm >> j) & 1u;
                        const float mag = (j == idx) ? n2 : n1;
                        app[v[j]] = __fadd_rn(q[j], s ? -mag : mag);
                    }
                    r1[ridx] = n1;
                    r2[ridx] = n2;
                    meta[ridx] = nm;
                }
                __syncwarp(gmask);
            }
            const int w = layered_syndrome<D>(cv, s_vars, app, gl, G, gmask, dummy);
            ++iter;
            if (track_best && (w < best_w || (w == 0 && best_w == 0))) {
                for (int i = gl; i < n; i += G) best[i] = app[i];
                __syncwarp(gmask);
            }
            if (w < best_w) best_w = w;
            if (w == 0 || iter >= p.max_iter) {
                // ---- finalize ----
                bool accept = (w == 0);
                if (accept && p.min_abs_accept > 0.0f) {
                    unsigned mn = 0x7f800000u;
                    for (int i = gl; i < n; i += G) mn = min(mn, __float_as_uint(fabsf(app[i])));
                    mn = __reduce_min_sync(gmask, mn);
                    accept = __uint_as_float(mn) >= p.min_abs_accept;
                }
                const bool route = !accept && p.route_failures_to_osd && io.osd_llr != nullptr;
                if (gl == 0) {
                    if (io.success) io.success[c] = accept ? 1 : 0;
                    if (io.iterations) io.iterations[c] = static_cast<uint8_t>(iter);
                    if (io.used_osd) io.used_osd[c] = 0;
                }
                if (io.out_bits) {
                    uint8_t* dst = io.out_bits + static_cast<size_t>(c) * io.out_stride;
                    for (int i = gl; i < io.out_len; i += G) dst[i] = app[i] < 0.0f ? 1 : 0;
                }
                if (io.app_out) {
                    float* dst = io.app_out + static_cast<size_t>(c) * n;
                    for (int i = gl; i < n; i += G) dst[i] = app[i];
                }
                if (route) {
                    int s = 0;
                    if (gl == 0) s = atomicAdd(io.osd_count, 1);
                    s = __shfl_sync(gmask, s, leader);
                    const float* b = track_best ? best : app;
                    float* dst = io.osd_llr + static_cast<size_t>(s) * n;
                    for (int i = gl; i < n; i += G) dst[i] = b[i];
                    if (gl == 0) io.osd_index[s] = c;
                }
                int nxt = 0;
                if (gl == 0) nxt = total_groups + atomicAdd(io.work_counter, 1);
                c = __shfl_sync(gmask, nxt, leader);
                active = c < io.count;
                __syncwarp(gmask);
                if (active) init(c);
            }
        }
    }
}

// Layered kernel for codes whose group lane owns at most NL rows in all
// (num_layers x rows_per_lane <= NL, the (128,64) code: 4): the lane's row
// tables (variable indices) stay in registers for the whole launch and its
// rows' compressed messages in registers for the codeword, so the row updates
// and the syndrome go to shared memory only for the posteriors.  Rows, order
// and arithmetic are those of bp_layered_kernel.  A row shorter than D (and a
// row slot past its layer's last row) points its missing edges at a dummy
// posterior held at +inf behind the slot's posteriors: such an edge never sets
// the row's minima, argmin or sign and never flips a parity, and its update
// leaves it at +inf, so the row loops need no per-edge test.
template <int D, int NL>
__global__ void __launch_bounds__(kBpThreads, 3)
bp_layered_reg_kernel(LayeredView cv, BpParams p, BpIO io, int slots_per_cta, int slot_floats, int track_best)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int G = cv.group;
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const int sub = lane / G;
    const int slot = threadIdx.x / G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (sub * G));
    const int leader = sub * G;

    const int n = cv.n;
    const int n_pad = (n + 3) & ~3;
    const int rpl = cv.rows_per_lane;
    const int nrows = cv.num_layers * rpl;
    float* app = reinterpret_cast<float*>(smem) + static_cast<size_t>(slot) * slot_floats;
    const int dummy = n_pad;           // app[dummy] = +inf for the whole launch
    float* best = app + n_pad + 4;     // only when track_best

    // row t of this lane: layer t / rpl, slot gl + (t mod rpl) G
    int vr[NL][D];
    unsigned real_rows = 0;  // bit t: row t of this lane exists
#pragma unroll
    for (int t = 0; t < NL; ++t) {
        const int L = t / rpl, rs = gl + (t - L * rpl) * G;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            const int v = (t < nrows && j < cv.maxdeg) ? __ldg(cv.vars + (L * cv.maxdeg + j) * cv.width + rs) : -1;
            vr[t][j] = v >= 0 ? v : dummy;
        }
        real_rows |= (vr[t][0] != dummy) ? (1u << t) : 0u;
    }
    float m1r[NL], m2r[NL];
    unsigned mr[NL];

    auto syndrome = [&]() -> int {
        int cnt = 0;
#pragma unroll
        for (int t = 0; t < NL; ++t) {
            unsigned par = 0;
#pragma unroll
            for (int j = 0; j < D; ++j) par ^= (app[vr[t][j]] < 0.0f) ? 1u : 0u;
            cnt += static_cast<int>(par);
        }
        return static_cast<int>(__reduce_add_sync(gmask, static_cast<unsigned>(cnt)));
    };

    const int total_groups = gridDim.x * slots_per_cta;
    int c = blockIdx.x * slots_per_cta + slot;
    bool active = c < io.count;
    int iter = 0, best_w = 0;

    auto init = [&](int cw) {
        const float* src = io.llr + static_cast<size_t>(cw) * n;
        if ((n & 3) == 0) {
            const float4* s4 = reinterpret_cast<const float4*>(src);
            for (int i = gl; i < (n >> 2); i += G) {
                const float4 v = __ldcs(s4 + i);
                reinterpret_cast<float4*>(app)[i] = v;
                if (track_best) reinterpret_cast<float4*>(best)[i] = v;
            }
        } else {
            for (int i = gl; i < n; i += G) {
                const float v = __ldcs(src + i);
                app[i] = v;
                if (track_best) best[i] = v;
            }
        }
#pragma unroll
        for (int t = 0; t < NL; ++t) {
            m1r[t] = 0.0f;
            m2r[t] = 0.0f;
            mr[t] = 0u;
        }
        __syncwarp(gmask);
        best_w = syndrome();
        iter = 0;
    };

    if (gl == 0) app[dummy] = __int_as_float(0x7f800000);  // +inf, before init's __syncwarp
    if (active) init(c);

    while (__any_sync(0xffffffffu, active)) {
        if (active) {
            // ---- one layered iteration ----
#pragma unroll
            for (int t = 0; t < NL; ++t) {
                if ((real_rows >> t) & 1u) {
                    float q[D];
                    float m1 = FLT_MAX, m2 = FLT_MAX;
                    int idx = 0;
                    unsigned neg = 0;
#pragma unroll
                    for (int j = 0; j < D; ++j) {
                        const float qj = __fsub_rn(app[vr[t][j]], rebuild(m1r[t], m2r[t], mr[t], j));
                        q[j] = qj;
                        neg |= (qj < 0.0f) ? (1u << j) : 0u;
                        const float a = fabsf(qj);
                        idx = (a < m1) ? j : idx;
                        m2 = fminf(m2, fmaxf(m1, a));
                        m1 = fminf(m1, a);
                    }
                    const unsigned tot = static_cast<unsigned>(__popc(neg)) & 1u;
                    const float n1 = nms_mag(p.alpha, p.beta, m1);
                    const float n2 = nms_mag(p.alpha, p.beta, m2);
                    const unsigned nm = ((neg ^ (0u - tot)) & 0x07FFFFFFu) | (static_cast<unsigned>(idx) << 27);
#pragma unroll
                    for (int j = 0; j < D; ++j) {
                        const unsigned sg = (nm >> j) & 1u;
                        const float mag = (j == idx) ? n2 : n1;
                        app[vr[t][j]] = __fadd_rn(q[j], sg ? -mag : mag);
                    }
                    m1r[t] = n1;
                    m2r[t] = n2;
                    mr[t] = nm;
                }
                if ((t + 1) % rpl == 0) __syncwarp(gmask);  // end of a layer
            }
            const int w = syndrome();
            ++iter;
            // The best posterior so far (a zero syndrome always is).  A zero syndrome's is app
            // itself, so its copy is skipped where that costs no spill (D = 8 would spill).
            const bool last = w == 0 || iter >= p.max_iter;
            const bool zero_in_app = D <= 6 && w == 0;
            if (track_best && (w < best_w || (w == 0 && best_w == 0)) && !zero_in_app) {
                for (int i = gl; i < n; i += G) best[i] = app[i];
                __syncwarp(gmask);
            }
            if (w < best_w) best_w = w;
            if (last) {
                // ---- finalize (bp_layered_kernel's) ----
                bool accept = (w == 0);
                if (accept && p.min_abs_accept > 0.0f) {
                    unsigned mn = 0x7f800000u;
                    for (int i = gl; i < n; i += G) mn = min(mn, __float_as_uint(fabsf(app[i])));
                    mn = __reduce_min_sync(gmask, mn);
                    accept = __uint_as_float(mn) >= p.min_abs_accept;
                }
                const bool route = !accept && p.route_failures_to_osd && io.osd_llr != nullptr;
                if (gl == 0) {
                    if (io.success) io.success[c] = accept ? 1 : 0;
                    if (io.iterations) io.iterations[c] = static_cast<uint8_t>(iter);
                    if (io.used_osd) io.used_osd[c] = 0;
                }
                if (io.out_bits) {
                    uint8_t* dst = io.out_bits + static_cast<size_t>(c) * io.out_stride;
                    for (int i = gl; i < io.out_len; i += G) dst[i] = app[i] < 0.0f ? 1 : 0;
                }
                if (io.app_out) {
                    float* dst = io.app_out + static_cast<size_t>(c) * n;
                    for (int i = gl; i < n; i += G) dst[i] = app[i];
                }
                if (route) {
                    int s = 0;
                    if (gl == 0) s = atomicAdd(io.osd_count, 1);
                    s = __shfl_sync(gmask, s, leader);
                    const float* b = (track_best && !zero_in_app) ? best : app;
                    float* dst = io.osd_llr + static_cast<size_t>(s) * n;
                    for (int i = gl; i < n; i += G) dst[i] = b[i];
                    if (gl == 0) io.osd_index[s] = c;
                }
                int nxt = 0;
                if (gl == 0) nxt = total_groups + atomicAdd(io.work_counter, 1);
                c = __shfl_sync(gmask, nxt, leader);
                active = c < io.count;
                __syncwarp(gmask);
                if (active) init(c);
            }
        }
    }
}

__global__ void __launch_bounds__(kBpThreads)
bp_flooding_kernel(FloodView cv, BpParams p, BpIO io, int slot_floats, int track_best)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int n = cv.n, m = cv.m, E = cv.edges;
    const int n_pad = (n + 3) & ~3, m_pad = (m + 3) & ~3;
    float* llr = reinterpret_cast<float*>(smem) + static_cast<size_t>(warp) * slot_floats;
    float* app = llr + n_pad;
    float* best = app + n_pad;
    float* q = best + n_pad;
    float* r1 = q + ((E + 3) & ~3);
    float* r2 = r1 + m_pad;
    unsigned* meta = reinterpret_cast<unsigned*>(r2 + m_pad);
    const float keep = __fsub_rn(1.0f, p.damping);

    auto syndrome = [&](const float* x) {
        int cnt = 0;
        for (int r = lane; r < m; r += 32) {
            unsigned par = 0;
            for (int e = __ldg(cv.row_ptr + r); e < __ldg(cv.row_ptr + r + 1); ++e)
                par ^= (x[__ldg(cv.col_ind + e)] < 0.0f) ? 1u : 0u;
            cnt += static_cast<int>(par);
        }
        return static_cast<int>(__reduce_add_sync(0xffffffffu, static_cast<unsigned>(cnt)));
    };
    auto edge_msg = [&](int e) {
        const int r = __ldg(cv.edge_row + e);
        return rebuild(r1[r], r2[r], meta[r], e - __ldg(cv.row_ptr + r));
    };

    const int warps_total = gridDim.x * (blockDim.x >> 5);
    for (int c = blockIdx.x * (blockDim.x >> 5) + warp; c < io.count; c += warps_total) {
        const float* src = io.llr + static_cast<size_t>(c) * n;
        for (int i = lane; i < n; i += 32) {
            const float v = __ldcs(src + i);
            llr[i] = v;
            app[i] = v;
            if (track_best) best[i] = v;
        }
        __syncwarp();
        for (int e = lane; e < E; e += 32) q[e] = llr[__ldg(cv.col_ind + e)];
        __syncwarp();
        int best_w = syndrome(llr);
        int iter = 0, w = 0;
        while (true) {
            // check nodes (L:3033-3060)
            for (int r = lane; r < m; r += 32) {
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
            __syncwarp();
            // variable nodes (L:3062-3069): llr + sum of messages in row order
            for (int v = lane; v < n; v += 32) {
                float acc = llr[v];
                for (int j = __ldg(cv.col_ptr + v); j < __ldg(cv.col_ptr + v + 1); ++j)
                    acc = __fadd_rn(acc, edge_msg(__ldg(cv.col_edge + j)));
                app[v] = acc;
            }
            __syncwarp();
            w = syndrome(app);
            ++iter;
            if (track_best && (w < best_w || (w == 0 && best_w == 0))) {
                for (int i = lane; i < n; i += 32) best[i] = app[i];
                __syncwarp();
            }
            if (w < best_w) best_w = w;
            if (w == 0 || iter >= p.max_iter) break;
            // next variable-to-check messages (L:3076-3081), optional damping
            for (int v = lane; v < n; v += 32) {
                for (int j = __ldg(cv.col_ptr + v); j < __ldg(cv.col_ptr + v + 1); ++j) {
                    const int e = __ldg(cv.col_edge + j);
                    const float fresh = __fsub_rn(app[v], edge_msg(e));
                    q[e] = (p.damping == 0.0f) ? fresh
                                                : __fadd_rn(__fmul_rn(keep, fresh), __fmul_rn(p.damping, q[e]));
                }
            }
            __syncwarp();
        }
        bool accept = (w == 0);
        if (accept && p.min_abs_accept > 0.0f) {
            unsigned mn = 0x7f800000u;
            for (int i = lane; i < n; i += 32) mn = min(mn, __float_as_uint(fabsf(app[i])));
            mn = __reduce_min_sync(0xffffffffu, mn);
            accept = __uint_as_float(mn) >= p.min_abs_accept;
        }
        const bool route = !accept && p.route_failures_to_osd && io.osd_llr != nullptr;
        if (lane == 0) {
            if (io.success) io.success[c] = accept ? 1 : 0;
            if (io.iterations) io.iterations[c] = static_cast<uint8_t>(iter);
            if (io.used_osd) io.used_osd[c] = 0;
        }
        if (io.out_bits) {
            uint8_t* dst = io.out_bits + static_cast<size_t>(c) * io.out_stride;
            for (int i = lane; i < io.out_len; i += 32) dst[i] = app[i] < 0.0f ? 1 : 0;
        }
        if (io.app_out) {
            float* dst = io.app_out + static_cast<size_t>(c) * n;
            for (int i = lane; i < n; i += 32) dst[i] = app[i];
        }
        if (route) {
            int s = 0;
            if (lane == 0) s = atomicAdd(io.osd_count, 1);
            s = __shfl_sync(0xffffffffu, s, 0);
            const float* b = track_best ? best : app;
            float* dst = io.osd_llr + static_cast<size_t>(s) * n;
            for (int i = lane; i < n; i += 32) dst[i] = b[i];
            if (lane == 0) io.osd_index[s] = c;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

size_t layered_smem_bytes(const LayeredView& cv, int slots, bool track_best, int* slot_floats_out)
{
    const int n_pad = (cv.n + 3) & ~3;
    const int mp = cv.num_layers * cv.width;
    // posteriors, the dummy edge's +inf (padded to 4 floats), the best posteriors, messages
    int slot_floats = ((track_best ? 2 : 1) * n_pad + 4 + 3 * mp + 3) & ~3;
    slot_floats = pad_slot_stride(slot_floats, cv.group);
    if (slot_floats_out) *slot_floats_out = slot_floats;
    const int table = (cv.num_layers * cv.maxdeg * cv.width + 3) & ~3;
    return (static_cast<size_t>(table) + static_cast<size_t>(slots) * slot_floats) * sizeof(float);
}

int layered_default_slots(const LayeredView& cv, bool track_best)
{
    int slots = kBpThreads / cv.group;
    while (slots > 32 / cv.group && layered_smem_bytes(cv, slots, track_best, nullptr) > 112 * 1024)
        slots -= 32 / cv.group;
    return slots;
}

// Register-resident variant: codes whose lane owns at most kRegRows rows (num_layers x
// rows_per_lane), row degree <= 8.
constexpr int kRegRows = 4;

template <int D>
static void launch_layered_reg_t(const LayeredView& cv, const BpParams& p, const BpIO& io, int slots, int ctas,
                                 bool track_best, cudaStream_t st)
{
    const int n_pad = (cv.n + 3) & ~3;
    // posteriors, the dummy edge's +inf (padded to 4 floats), then the best posteriors
    int slot_floats = (track_best ? 2 : 1) * n_pad + 4;
    slot_floats = pad_slot_stride(slot_floats, cv.group);
    const size_t smem = static_cast<size_t>(slots) * slot_floats * sizeof(float);
    const auto kernel = bp_layered_reg_kernel<D, kRegRows>;
    check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(kernel), smem), "cudaFuncSetAttribute(bp_layered_reg)");
    if (ctas <= 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, slots * cv.group, smem) != cudaSuccess ||
            per_sm <= 0)
            per_sm = 1;
        ctas = per_sm * device_sm_count();
        ctas = std::max(1, std::min(ctas, (io.count + slots - 1) / slots));
    }
    kernel<<<ctas, slots * cv.group, smem, st>>>(cv, p, io, slots, slot_floats, track_best ? 1 : 0);
    check_cuda(cudaGetLastError(), "bp_layered_reg_kernel launch");
}

template <int D>
static void launch_layered_t(const LayeredView& cv, const BpParams& p, const BpIO& io, int slots, int ctas,
                             bool track_best, cudaStream_t st)
{
    if constexpr (D <= 8) {
        if (cv.num_layers * cv.rows_per_lane <= kRegRows) {
            launch_layered_reg_t<D>(cv, p, io, slots, ctas, track_best, st);
            return;
        }
    }
    int slot_floats = 0;
    const size_t smem = layered_smem_bytes(cv, slots, track_best, &slot_floats);
    check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(bp_layered_kernel<D>), smem),
               "cudaFuncSetAttribute(bp_layered)");
    if (ctas <= 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bp_layered_kernel<D>, slots * cv.group, smem) !=
                cudaSuccess ||
            per_sm <= 0)
            per_sm = 1;
        ctas = per_sm * device_sm_count();
        ctas = std::max(1, std::min(ctas, (io.count + slots - 1) / slots));
    }
    bp_layered_kernel<D><<<ctas, slots * cv.group, smem, st>>>(cv, p, io, slots, slot_floats, track_best ? 1 : 0);
    check_cuda(cudaGetLastError(), "bp_layered_kernel launch");
}

void launch_bp_layered(const LayeredView& cv, const BpParams& p, const BpIO& io, const BpLaunch& shape,
                       cudaStream_t st)
{
    if (io.count <= 0) return;
    const bool track_best = p.route_failures_to_osd && io.osd_llr != nullptr;
    if (layered_needs_wide(cv, track_best)) {
        launch_bp_layered_wide(cv, p, io, st);
        return;
    }
    const int step = std::max(1, 32 / cv.group);
    int slots = shape.slots_per_cta > 0 ? shape.slots_per_cta : layered_default_slots(cv, track_best);
    slots = std::max(step, slots - slots % step);
    if (slots * cv.group > kBpThreads) slots = kBpThreads / cv.group;
    while (slots > step && layered_smem_bytes(cv, slots, track_best, nullptr) > 227 * 1024) slots -= step;
    check_cuda(cudaMemsetAsync(io.work_counter, 0, sizeof(int), st), "reset work counter");
    // the row loops are unrolled to D slots: the closest D above the code's row degree
    if (cv.maxdeg <= 6) launch_layered_t<6>(cv, p, io, slots, shape.ctas, track_best, st);
    else if (cv.maxdeg <= 8) launch_layered_t<8>(cv, p, io, slots, shape.ctas, track_best, st);
    else if (cv.maxdeg <= 10) launch_layered_t<10>(cv, p, io, slots, shape.ctas, track_best, st);
    else if (cv.maxdeg <= 12) launch_layered_t<12>(cv, p, io, slots, shape.ctas, track_best, st);
    else if (cv.maxdeg <= 14) launch_layered_t<14>(cv, p, io, slots, shape.ctas, track_best, st);
    else if (cv.maxdeg <= 16) launch_layered_t<16>(cv, p, io, slots, shape.ctas, track_best, st);
    else launch_layered_t<27>(cv, p, io, slots, shape.ctas, track_best, st);
}

size_t flooding_smem_bytes(const FloodView& cv, int warps, int* slot_floats_out)
{
    const int n_pad = (cv.n + 3) & ~3, m_pad = (cv.m + 3) & ~3, e_pad = (cv.edges + 3) & ~3;
    const int slot_floats = 3 * n_pad + e_pad + 3 * m_pad;
    if (slot_floats_out) *slot_floats_out = slot_floats;
    return static_cast<size_t>(warps) * slot_floats * sizeof(float);
}

void launch_bp_flooding(const FloodView& cv, const BpParams& p, const BpIO& io, cudaStream_t st)
{
    if (io.count <= 0) return;
    if (flooding_needs_wide(cv)) {
        launch_bp_flooding_wide(cv, p, io, st);
        return;
    }
    const bool track_best = p.route_failures_to_osd && io.osd_llr != nullptr;
    int warps = kBpThreads / 32;
    int slot_floats = 0;
    while (warps > 1 && flooding_smem_bytes(cv, warps, &slot_floats) > 160 * 1024) --warps;
    const size_t smem = flooding_smem_bytes(cv, warps, &slot_floats);
    check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(bp_flooding_kernel), smem),
               "cudaFuncSetAttribute(bp_flooding)");
    const int per_sm = std::max(1, static_cast<int>((227 * 1024) / std::max<size_t>(smem, 1)));
    int ctas = std::min(per_sm, 8) * device_sm_count();
    ctas = std::max(1, std::min(ctas, (io.count + warps - 1) / warps));
    bp_flooding_kernel<<<ctas, warps * 32, smem, st>>>(cv, p, io, slot_floats, track_best ? 1 : 0);
    check_cuda(cudaGetLastError(), "bp_flooding_kernel launch");
}

template __global__ void bp_layered_kernel<6>(LayeredView, BpParams, BpIO, int, int, int);
template __global__ void bp_layered_kernel<8>(LayeredView, BpParams, BpIO, int, int, int);
template __global__ void bp_layered_kernel<10>(LayeredView, BpParams, BpIO, int, int, int);
template __global__ void bp_layered_kernel<12>(LayeredView, BpParams, BpIO, int, int, int);
template __global__ void bp_layered_kernel<14>(LayeredView, BpParams, BpIO, int, int, int);
template __global__ void bp_layered_kernel<16>(LayeredView, BpParams, BpIO, int, int, int);
template __global__ void bp_layered_kernel<27>(LayeredView, BpParams, BpIO, int, int, int);

}  // namespace sicc
