// Ordered-statistics decoding (OSD) for sm_103a: one warp per codeword.
//
// Restates cpu_bp_osd_decode.m:187-305 (the reference's MATLAB BP-OSD):
//   1. stable descending sort of |llr| (ties: lower index first);
//   2. systematic form of the column-permuted generator G = [I_k | P]: the
//      pivots are the first k linearly independent positions in reliability
//      order (the most reliable basis), found by a column scan over a
//      bit-packed row-reduced copy of G held in registers (64-bit XOR rows);
//   3. base candidate = hard decisions on the basis; flip candidates over the
//      weakest basis positions in the enumeration order of MATLAB nchoosek;
//   4. metric = sum of |llr| over positions where the candidate differs from
//      the hard decision, accumulated in decreasing-reliability order in
//      single precision; the first candidate with the smallest metric wins
//      (strict <, cpu_bp_osd_decode.m:222), realised as a minimum over
//      (metric bits, test index) keys.
// Candidates are evaluated by all 32 lanes in parallel; each candidate's
// difference vector is the base difference XOR at most three reduced rows.
// A lane stops summing a candidate once its partial metric exceeds the best
// metric it knows; the warp exchanges its best every `share_rounds` rounds of
// 32 candidates (a launch parameter, chosen by the autotuner).  Pruning only
// drops candidates that cannot win, so the winner is the same for any value.
#include "bp_kernels.h"

#include <algorithm>
#include <type_traits>

namespace sicc {

namespace {

constexpr int kOsdWarps = 8;

// Small shapes also keep the reduced rows in flip-pool order, so a candidate reads its
// flipped rows without the rank lookup (the larger shapes would lose occupancy to it).
template <int NW, int KR>
constexpr bool kFlipRows = NW * KR <= 4;

template <int NW, int KR>
struct OsdSmem {
    float rel_sorted[NW * 64];
    int16_t perm[NW * 64];
    int16_t rowpiv[KR * 32];  // row id -> pivot index
    int16_t flip[KR * 32];    // weakness rank -> pivot index
    uint32_t hard_orig[NW * 2];
    unsigned long long rows[KR * 32][NW];  // reduced rows by pivot index
    unsigned long long frows[kFlipRows<NW, KR> ? KR * 32 : 1][NW];  // the same rows by flip-pool rank
    int16_t mrb_pos[KR * 32];
    float prel[KR * 32];      // flip-pool rank -> |llr| of its position (non-decreasing)
    int16_t rstart[KR * 32];  // order-2 rows: first surviving pair of row a in the compact list
};

__device__ __forceinline__ unsigned long long shfl_u64(unsigned long long v, int src)
{
    const unsigned lo = __shfl_sync(0xffffffffu, static_cast<unsigned>(v), src);
    const unsigned hi = __shfl_sync(0xffffffffu, static_cast<unsigned>(v >> 32), src);
    return (static_cast<unsigned long long>(hi) << 32) | lo;
}

// Word `w` of a register array, selected without dynamic indexing (which
// would move the array to local memory).
template <int NW>
__device__ __forceinline__ unsigned long long pick(const unsigned long long (&a)[NW], int w)
{
    unsigned long long r = 0ull;
#pragma unroll
    for (int i = 0; i < NW; ++i)
        if (i == w) r = a[i];
    return r;
}

__device__ __forceinline__ unsigned long long shfl_xor_u64(unsigned long long v, int m)
{
    const unsigned lo = __shfl_xor_sync(0xffffffffu, static_cast<unsigned>(v), m);
    const unsigned hi = __shfl_xor_sync(0xffffffffu, static_cast<unsigned>(v >> 32), m);
    return (static_cast<unsigned long long>(hi) << 32) | lo;
}

}  // namespace

template <int NW, int KR>
__global__ void __launch_bounds__(kOsdWarps * 32)
osd_kernel(OsdView ov0, OsdIO io)
{
    constexpr int KW = (KR + 1) / 2;
    __shared__ OsdSmem<NW, KR> sm_all[kOsdWarps];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    OsdSmem<NW, KR>& s = sm_all[warp];
    const int count = io.count_ptr ? *io.count_ptr : io.count;
    const int total_warps = gridDim.x * kOsdWarps;

    auto next_item = [&](int prev) -> int {  // the warp's next work item
        if (!io.work) return prev < 0 ? static_cast<int>(blockIdx.x) * kOsdWarps + warp : prev + total_warps;
        int it = 0;
        if (lane == 0) it = atomicAdd(io.work, 1);
        return __shfl_sync(0xffffffffu, it, 0);
    };
    for (int item = next_item(-1); item < count; item = next_item(item)) {
        const int cw = io.index ? io.index[item] : item;
        const OsdView ov = io.views ? io.views[io.code_of[cw]] : ov0;
        if (ov.n == 0) continue;  // code without warp-kernel tables (uniform over the warp)
        const int n = ov.n, k = ov.k;
        const float* src = io.row_off   ? io.llr + io.row_off[item]
                           : io.llr_off ? io.llr + io.llr_off[cw]
                                        : io.llr + static_cast<size_t>(item) * n;
        uint8_t* info_dst = io.out_info ? (io.info_off ? io.out_info + io.info_off[cw]
                                                       : io.out_info + static_cast<size_t>(cw) * io.info_stride)
                                        : nullptr;
        // ---- 1. reliabilities, hard decisions, stable descending sort ----
        // Bitonic sort of 64-bit keys in registers (element q*32 + lane in v[q]):
        // ascending key = descending |llr|, ties by ascending index (the order of
        // MATLAB's stable sort, cpu_bp_osd_decode.m:194).
        constexpr int NP = NW * 64, KPL = NP / 32;
        unsigned long long v[KPL];
#pragma unroll
        for (int q = 0; q < KPL; ++q) {
            const int i = q * 32 + lane;
            const float x = (i < n) ? src[i] : 0.0f;
            v[q] = (i < n) ? ((static_cast<unsigned long long>(0x7fffffffu - __float_as_uint(fabsf(x))) << 32) |
                              static_cast<unsigned>(i))
                           : ~0ull;
            const unsigned hb = __ballot_sync(0xffffffffu, (i < n) && (x < 0.0f));
            if (lane == 0) s.hard_orig[q] = hb;
        }
#pragma unroll
        for (int k2 = 2; k2 <= NP; k2 <<= 1) {
#pragma unroll
            for (int j2 = k2 >> 1; j2 > 0; j2 >>= 1) {
                if (j2 >= 32) {  // partner in this lane
#pragma unroll
                    for (int q = 0; q < KPL; ++q) {
                        if (q & (j2 >> 5)) continue;
                        const int q2 = q | (j2 >> 5);
                        const bool asc = ((q * 32 + lane) & k2) == 0;
                        const unsigned long long a = v[q], b = v[q2];
                        if ((a > b) == asc) {
                            v[q] = b;
                            v[q2] = a;
                        }
                    }
                } else {  // partner in lane ^ j2
#pragma unroll
                    for (int q = 0; q < KPL; ++q) {
                        const unsigned long long o = shfl_xor_u64(v[q], j2);
                        const bool asc = ((q * 32 + lane) & k2) == 0;
                        const bool take_min = ((lane & j2) == 0) == asc;
                        v[q] = take_min ? (o < v[q] ? o : v[q]) : (o > v[q] ? o : v[q]);
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < KPL; ++q) {
            const int r = q * 32 + lane;
            if (r < n) {
                s.perm[r] = static_cast<int16_t>(v[q] & 0xffffffffull);
                s.rel_sorted[r] = __uint_as_float(0x7fffffffu - static_cast<unsigned>(v[q] >> 32));
            }
        }
        __syncwarp();
        // hard decisions in sorted order
        unsigned long long hard_sorted[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            unsigned lo, hi;
            {
                const int j = w * 64 + lane;
                const int o = (j < n) ? s.perm[j] : 0;
                lo = __ballot_sync(0xffffffffu, (j < n) && ((s.hard_orig[o >> 5] >> (o & 31)) & 1u));
            }
            {
                const int j = w * 64 + 32 + lane;
                const int o = (j < n) ? s.perm[j] : 0;
                hi = __ballot_sync(0xffffffffu, (j < n) && ((s.hard_orig[o >> 5] >> (o & 31)) & 1u));
            }
            hard_sorted[w] = (static_cast<unsigned long long>(hi) << 32) | lo;
        }
        // ---- 2. permuted generator rows via ballots over column vectors ----
        unsigned long long rows[KR][NW];
#pragma unroll
        for (int a = 0; a < KR; ++a)
#pragma unroll
            for (int w = 0; w < NW; ++w) rows[a][w] = 0ull;
#pragma unroll
        for (int q = 0; q < NW * 2; ++q) {
            const int j = q * 32 + lane;
            unsigned long long col[KW];
#pragma unroll
            for (int x = 0; x < KW; ++x) col[x] = 0ull;
            if (j < n) {
                const int o = s.perm[j];
                if (o < k) {
                    col[o >> 6] = 1ull << (o & 63);
                } else {
#pragma unroll
                    for (int x = 0; x < KW; ++x)  // the code's own words (kw <= KW)
                        col[x] = x < ov.kw ? ov.pcols[static_cast<size_t>(o - k) * ov.kw + x] : 0ull;
                }
            }
            // 32 x 32 bit transposes (butterfly over lane ^ j): lane j's bits a*32.. of its
            // column become lane r's bits q*32.. of row a*32 + r
#pragma unroll
            for (int a = 0; a < KR; ++a) {
                unsigned x = static_cast<unsigned>(col[a >> 1] >> ((a & 1) * 32));
                unsigned msk = 0x0000FFFFu;
#pragma unroll
                for (int jj = 16; jj > 0; jj >>= 1) {
                    const unsigned y = __shfl_xor_sync(0xffffffffu, x, jj);
                    x = (lane & jj) ? ((x & ~msk) | ((y & ~msk) >> jj)) : ((x & msk) | ((y & msk) << jj));
                    msk ^= msk << (jj >> 1);
                }
                if (a * 32 + lane < k) rows[a][q >> 1] |= static_cast<unsigned long long>(x) << ((q & 1) * 32);
            }
        }
        // ---- 3. column-scan elimination: pivots = most reliable basis ----
        // Column j lives in bit j % 32 of 32-bit half (j / 32) % 2 of word j / 64 of every row:
        // the scan runs half-word by half-word, so the column's half is a register known at
        // compile time and each row test is one 32-bit operation.
        unsigned avail = 0;  // bit a: my row in slot a exists (r < k) and is not yet a pivot row
#pragma unroll
        for (int a = 0; a < KR; ++a) avail |= (a * 32 + lane < k) ? 1u << a : 0u;
        int rank = 0;
#pragma unroll
        for (int W = 0; W < NW; ++W) {
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                for (int b = 0; b < 32 && rank < k; ++b) {
                    const int j = W * 64 + hh * 32 + b;
                    if (j >= n) break;
                    const unsigned bm = 1u << b;
                    auto has = [&](int a) { return (static_cast<unsigned>(rows[a][W] >> (hh * 32)) & bm) != 0u; };
                    int ps = -1, pl = 0;
#pragma unroll
                    for (int a = 0; a < KR; ++a) {
                        const unsigned bal = __ballot_sync(0xffffffffu, ((avail >> a) & 1u) && has(a));
                        if (ps < 0 && bal) {
                            ps = a;
                            pl = __ffs(bal) - 1;
                        }
                    }
                    if (ps < 0) continue;  // dependent position
                    unsigned long long pw[NW];
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        unsigned long long mine = 0ull;
#pragma unroll
                        for (int a = 0; a < KR; ++a)
                            if (a == ps) mine = rows[a][w];
                        pw[w] = shfl_u64(mine, pl);
                    }
#pragma unroll
                    for (int a = 0; a < KR; ++a) {
                        const bool is_p = (a == ps) && (lane == pl);
                        if (!is_p && has(a)) {
#pragma unroll
                            for (int w = 0; w < NW; ++w) rows[a][w] ^= pw[w];
                        }
                        if (is_p) avail &= ~(1u << a);
                    }
                    if (lane == 0) {
                        s.rowpiv[ps * 32 + pl] = static_cast<int16_t>(rank);
                        s.mrb_pos[rank] = static_cast<int16_t>(j);
                    }
                    ++rank;
                }
            }
        }
        __syncwarp();
        if (rank < k) {  // generator not full rank: cannot happen for a valid code table
            if (lane == 0 && io.out_metric) io.out_metric[cw] = -1.0f;
            continue;
        }
        // ---- 4. reduced rows by pivot index; base difference vector ----
        unsigned long long acc[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) acc[w] = 0ull;
#pragma unroll
        for (int a = 0; a < KR; ++a) {
            const int r = a * 32 + lane;
            if (r < k) {
                const int t = s.rowpiv[r];
#pragma unroll
                for (int w = 0; w < NW; ++w) s.rows[t][w] = rows[a][w];
                const int pj = s.mrb_pos[t];
                if ((pick<NW>(hard_sorted, pj >> 6) >> (pj & 63)) & 1ull) {
#pragma unroll
                    for (int w = 0; w < NW; ++w) acc[w] ^= rows[a][w];
                }
            }
        }
#pragma unroll
        for (int w = 0; w < NW; ++w) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[w] ^= shfl_xor_u64(acc[w], o);
            acc[w] ^= hard_sorted[w];  // base difference from the hard decision
        }
        // ---- 5. flip pool: basis positions, weakest first (stable) ----
        // Pivots come in sorted-position order, so |llr| does not increase with the pivot
        // index t: t's rank is the count of later runs plus its place in its run of equal
        // |llr| (the run found by binary search).
        // |llr| compared as bit patterns, the order the sort used (a permutation whatever the values)
        auto relbits = [&](int t) -> unsigned { return __float_as_uint(s.rel_sorted[s.mrb_pos[t]]); };
        for (int t = lane; t < k; t += 32) {
            const unsigned bt = relbits(t);
            int lo = 0, hi = t;  // first index with |llr| <= bt
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (relbits(mid) > bt) lo = mid + 1;
                else hi = mid;
            }
            const int a = lo;
            lo = t + 1;
            hi = k;  // first index with |llr| < bt
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (relbits(mid) < bt) hi = mid;
                else lo = mid + 1;
            }
            const int r = (k - lo) + (t - a);
            if (r < ov.pool) {
                s.flip[r] = static_cast<int16_t>(t);
                s.prel[r] = s.rel_sorted[s.mrb_pos[t]];
                if (kFlipRows<NW, KR>)
#pragma unroll
                    for (int w = 0; w < NW; ++w) s.frows[kFlipRows<NW, KR> ? r : 0][w] = s.rows[t][w];
            }
        }
        __syncwarp();
        // ---- 6. all candidates in parallel ----
        // A candidate's metric is a sum of non-negative terms in a fixed order, so
        // its partial sums never decrease: once one exceeds the smallest metric
        // already found the candidate cannot win and its sum stops.  Ties are not
        // pruned (strict >), so the first minimum in test order still wins.
        unsigned long long best_key = ~0ull;
        float thr = INFINITY;
        const int share = io.share_rounds > 0 ? io.share_rounds : 2;
        // The metric of test q, whose flips are pool ranks f0, f1, f2, pruned against thr.  The
        // first `kSure` flips are known to exist (no test); the others may be -1 (none).
        auto evaluate = [&](auto sure, int q, int f0, int f1, int f2) {
            constexpr int kSure = decltype(sure)::value;
            unsigned long long d[NW];
#pragma unroll
            for (int w = 0; w < NW; ++w) d[w] = acc[w];
            const int fl[3] = {f0, f1, f2};
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                const int fi = fl[f];
                if (f < kSure || fi >= 0) {
                    if (kFlipRows<NW, KR>) {
#pragma unroll
                        for (int w = 0; w < NW; ++w) d[w] ^= s.frows[kFlipRows<NW, KR> ? fi : 0][w];
                    } else {
                        const int t = s.flip[fi];
#pragma unroll
                        for (int w = 0; w < NW; ++w) d[w] ^= s.rows[t][w];
                    }
                }
            }
            float metric = 0.0f;
            bool pruned = false;
#pragma unroll
            for (int h = 0; h < 2 * NW; ++h) {
                unsigned bits = static_cast<unsigned>(d[h >> 1] >> ((h & 1) * 32));
                const float* rel = s.rel_sorted + h * 32;
                while (bits && !pruned) {
                    const int b = __ffs(bits) - 1;
                    metric = __fadd_rn(metric, rel[b]);
                    bits &= bits - 1;
                    pruned = metric > thr;
                }
            }
            if (!pruned) {
                const unsigned long long key =
                    (static_cast<unsigned long long>(__float_as_uint(metric)) << 32) | static_cast<unsigned>(q);
                if (key < best_key) {
                    best_key = key;
                    thr = fminf(thr, metric);
                }
            }
        };
        auto share_best = [&]() {  // the best metric so far, to every lane
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long other = shfl_xor_u64(best_key, o);
                best_key = other < best_key ? other : best_key;
            }
            if (best_key != ~0ull) thr = __uint_as_float(static_cast<unsigned>(best_key >> 32));
        };
        auto flips_of = [&](int q, int& f0, int& f1, int& f2) {
            f0 = f1 = f2 = -1;
            if (q > 0) {
                const uint32_t cmb = ov.combos[q - 1];
                const uint32_t a = cmb & 0x3FFu, b = (cmb >> 10) & 0x3FFu, c = (cmb >> 20) & 0x3FFu;
                f0 = a != 0x3FFu ? static_cast<int>(a) : -1;
                f1 = b != 0x3FFu ? static_cast<int>(b) : -1;
                f2 = c != 0x3FFu ? static_cast<int>(c) : -1;
            }
        };
        const int P = ov.pool;
        const bool complete2 = P >= 2 && ov.num_tests == 1 + P + P * (P - 1) / 2;
        if (complete2) {
            // The tests are the base, the P single flips, then every pair (a, b), a < b, in
            // lexicographic order (test 1 + P + a (2P - a - 1) / 2 + b - a - 1).  A candidate
            // differs from the hard decision at its flipped positions, and the metric, summed in
            // position order, is at least those terms summed alone (each rounded partial sum of
            // a sum of non-negative terms is at least that of any of its subsequences): a pair
            // whose two |llr| already add up above the best metric of the base and single-flip
            // tests cannot win.  The pool is weakest first, so within row a the bound grows
            // with b and each row keeps a prefix (binary search); only those pairs are
            // evaluated, 32 at a time from a compact list.
            const int single = 1 + P;
            for (int rd = 0; rd * 32 < single; ++rd) {
                const int q = rd * 32 + lane;
                if (q < single) evaluate(std::integral_constant<int, 0>(), q, q > 0 ? q - 1 : -1, -1, -1);
            }
            share_best();
            const int R = (P - 1 + 31) / 32;  // rows a = 0 .. P-2, R consecutive rows per lane
            int mine = 0;
            for (int i = 0; i < R; ++i) {
                const int a = lane * R + i;
                int cnt = 0;
                if (a < P - 1) {
                    const float ra = s.prel[a];
                    int lo = a + 1, hi = P;  // first b with bound > thr
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (__fadd_rn(ra, s.prel[mid]) > thr) hi = mid;
                        else lo = mid + 1;
                    }
                    cnt = lo - (a + 1);
                }
                if (a < P - 1) s.rstart[a] = static_cast<int16_t>(mine);  // lane-local offset for now
                mine += cnt;
            }
            int incl = mine;  // inclusive scan of the lanes' pair counts
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int up = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += up;
            }
            const int base = incl - mine, total = __shfl_sync(0xffffffffu, incl, 31);
            for (int i = 0; i < R; ++i) {
                const int a = lane * R + i;
                if (a < P - 1) s.rstart[a] = static_cast<int16_t>(s.rstart[a] + base);
            }
            __syncwarp();
            int rd = 0, a = 0;  // a: the last row with rstart[a] <= idx (idx only grows: walk forward)
            for (int i0 = 0; i0 < total; i0 += 32, ++rd) {
                const int idx = i0 + lane;
                if (idx < total) {
                    while (a < P - 2 && s.rstart[a + 1] <= idx) ++a;
                    const int b = a + 1 + (idx - s.rstart[a]);
                    evaluate(std::integral_constant<int, 2>(), single + a * (2 * P - a - 1) / 2 + (b - a - 1), a, b, -1);
                }
                if (rd % share == share - 1) share_best();
            }
        } else {
            const int rounds = (ov.num_tests + 31) / 32;
            for (int rd = 0; rd < rounds; ++rd) {
                const int q = rd * 32 + lane;
                if (q < ov.num_tests) {
                    int f0, f1, f2;
                    flips_of(q, f0, f1, f2);
                    evaluate(std::integral_constant<int, 0>(), q, f0, f1, f2);
                }
                if (rd % share == share - 1) share_best();
            }
        }
        share_best();
        // ---- 7. winner -> original positions ----
        const int qbest = static_cast<int>(best_key & 0xffffffffull);
        unsigned long long d[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) d[w] = acc[w];
        if (qbest > 0) {
            const uint32_t cmb = ov.combos[qbest - 1];
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                const uint32_t fi = (cmb >> (10 * f)) & 0x3FFu;
                if (fi != 0x3FFu) {
                    const int t = s.flip[fi];
#pragma unroll
                    for (int w = 0; w < NW; ++w) d[w] ^= s.rows[t][w];
                }
            }
        }
#pragma unroll
        for (int w = 0; w < NW; ++w) d[w] ^= hard_sorted[w];  // decoded codeword in sorted order
        for (int j = lane; j < n; j += 32) {
            const int o = s.perm[j];
            const uint8_t bit = static_cast<uint8_t>((pick<NW>(d, j >> 6) >> (j & 63)) & 1ull);
            if (info_dst && o < k) info_dst[o] = bit;
            if (io.out_code) io.out_code[static_cast<size_t>(cw) * n + o] = bit;
        }
        if (lane == 0) {
            if (io.out_metric) io.out_metric[cw] = __uint_as_float(static_cast<unsigned>(best_key >> 32));
            if (io.used_osd) io.used_osd[cw] = 1;
        }
        __syncwarp();
    }
}

template <int NW, int KR>
static void launch_osd_t(const OsdView& ov, const OsdIO& io, int max_items, cudaStream_t st, int ctas)
{
    if (ctas <= 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, osd_kernel<NW, KR>, kOsdWarps * 32, 0) !=
                cudaSuccess ||
            per_sm <= 0)
            per_sm = 1;
        ctas = per_sm * device_sm_count();
        ctas = std::max(1, std::min(ctas, (max_items + kOsdWarps - 1) / kOsdWarps));
    }
    osd_kernel<NW, KR><<<ctas, kOsdWarps * 32, 0, st>>>(ov, io);
    check_cuda(cudaGetLastError(), "osd_kernel launch");
}

void launch_osd(const OsdView& ov, const OsdIO& io, int max_items, cudaStream_t st, int warps_per_cta, int ctas)
{
    (void)warps_per_cta;
    if (max_items <= 0) return;
    if (io.work) check_cuda(cudaMemsetAsync(io.work, 0, sizeof(int), st), "reset OSD work counter");
    // for a mixed-code batch `ov` carries the largest n and k of its codes
    const int nw = (ov.n + 63) / 64;
    const int kr = (ov.k + 31) / 32;
    const int NW = nw <= 1 ? 1 : (nw <= 2 ? 2 : 4);
    const int KR = kr <= 1 ? 1 : (kr <= 2 ? 2 : 4);
    if (nw > 4 || kr > 4) throw InvalidArgument("OSD kernel supports n <= 256 and k <= 128");
#define SICC_OSD_CASE(A, B) \
    if (NW == A && KR == B) { launch_osd_t<A, B>(ov, io, max_items, st, ctas); return; }
    SICC_OSD_CASE(1, 1) SICC_OSD_CASE(1, 2) SICC_OSD_CASE(2, 1) SICC_OSD_CASE(2, 2)
    SICC_OSD_CASE(2, 4) SICC_OSD_CASE(4, 2) SICC_OSD_CASE(4, 4) SICC_OSD_CASE(4, 1) SICC_OSD_CASE(1, 4)
#undef SICC_OSD_CASE
    throw InvalidArgument("unsupported OSD shape");
}

}  // namespace sicc
