// Ordered-statistics decoding for codes beyond the warp kernel (n > 256 or
// k > 128): one CTA per codeword, elimination on the parity-check matrix.
//
// The decoder is cpu_bp_osd_decode.m:187-305 (the reference's MATLAB BP-OSD)
// with the same result, candidate order and tie rule as the warp kernel; only
// the way the most reliable basis (MRB) and the re-encoding are obtained
// differs, because the k x n generator of a long code (up to 1536 x 2048 bits)
// does not fit in shared memory:
//   * the MRB -- the first k independent positions of G in decreasing
//     reliability, found by the column-pivoted elimination of
//     generator_to_systematic (MB:270-305) -- is the complement of the first
//     m independent positions of H in increasing reliability (the bases of a
//     code's matroid are the complements of the bases of its dual, and the
//     greedy scan gives the extreme basis in either order);
//   * those m columns are found by Gauss-Jordan elimination on H: the
//     accumulated row operations T (m x m bits, 128 KiB at m = 1024) live in
//     shared memory, and column c's reduced form is T h_c, the XOR of the few
//     columns of T that h_c selects (column weight <= 16);
//   * with T H in reduced form on those columns, a candidate that keeps the
//     hard decisions on the MRB except a flip set F differs from the hard
//     decisions at the pivot positions selected by T s XOR (XOR over f in F of
//     T h_f), s = H * hard.  Only T s and the flip-pool columns are built.
// The metric sums |llr| over the differing positions in increasing sorted
// position (decreasing reliability) in single precision, exactly as MB:247-250.
#include "bp_kernels.h"

#include <algorithm>
#include <climits>

namespace sicc {

namespace {

constexpr int kOsdHThreads = 512;
constexpr int kOsdHWarps = kOsdHThreads / 32;
constexpr int kOsdHMaxPool = 128;

struct OsdHLayout {
    int np;       // sort length: power of two >= the longest n
    int nmax;
    int mw;       // words per row of T for the largest m
    int ts;       // row stride of T in words (odd: a warp reading one word of 32 rows hits 32 banks)
    int poolmax;
};

struct OsdHSmem {
    uint32_t* T;             // [32*mw][ts]
    unsigned long long* keys;// [np]; reused as the flip-pool scratch after the sort
    float* rel;              // [nmax] |llr| by sorted position j
    int16_t* perm;           // [nmax] code position at sorted position j
    int16_t* row_of_col;     // [nmax] pivot row of a code position, -1 for the MRB
    uint32_t* hard;          // [nmax/32+1] hard decisions by code position
    uint32_t* vw;            // [mw] reduced column of the position being scanned
    uint32_t* syn;           // [mw] s = H * hard by row of H
    int16_t* pivj;           // [32*mw] sorted position of each pivot row's column
    float* relq;             // [32*mw] |llr| of each pivot row's column
    int16_t* mrb;            // [nmax] dependent positions met during the scan (descending j)
    int16_t* pool_j;         // [poolmax] flip pool (sorted positions, weakest first)
    uint32_t* avec;          // [poolmax][mw] T h_f for the pool
    uint32_t* aug;           // [mw] T s
};

__host__ __device__ inline size_t a16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline size_t carve(const OsdHLayout& l, unsigned char* base, OsdHSmem* s)
{
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base ? base + o : nullptr;
        o = a16(o + bytes);
        return p;
    };
    const size_t rows = 32 * static_cast<size_t>(l.mw);
    OsdHSmem t{};
    t.T = reinterpret_cast<uint32_t*>(take(rows * l.ts * 4));
    t.keys = reinterpret_cast<unsigned long long*>(take(static_cast<size_t>(l.np) * 8));
    t.rel = reinterpret_cast<float*>(take(static_cast<size_t>(l.nmax) * 4));
    t.perm = reinterpret_cast<int16_t*>(take(static_cast<size_t>(l.nmax) * 2));
    t.row_of_col = reinterpret_cast<int16_t*>(take(static_cast<size_t>(l.nmax) * 2));
    t.hard = reinterpret_cast<uint32_t*>(take((static_cast<size_t>(l.nmax) / 32 + 1) * 4));
    t.vw = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(l.mw) * 4));
    t.syn = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(l.mw) * 4));
    t.pivj = reinterpret_cast<int16_t*>(take(rows * 2));
    t.relq = reinterpret_cast<float*>(take(rows * 4));
    t.mrb = reinterpret_cast<int16_t*>(take(static_cast<size_t>(l.nmax) * 2));
    t.pool_j = reinterpret_cast<int16_t*>(take(static_cast<size_t>(l.poolmax) * 2));
    t.avec = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(l.poolmax) * l.mw * 4));
    t.aug = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(l.mw) * 4));
    if (s) *s = t;
    return o;
}

__device__ __forceinline__ unsigned tbit(const uint32_t* row, int q) { return (row[q >> 5] >> (q & 31)) & 1u; }

// Reduced column T h_c, bit of row r.
__device__ __forceinline__ unsigned reduced_bit(const uint32_t* Trow, const int* __restrict__ col_rows, int e0, int e1)
{
    unsigned v = 0;
    for (int e = e0; e < e1; ++e) v ^= tbit(Trow, col_rows[e]);
    return v;
}

}  // namespace

__global__ void __launch_bounds__(kOsdHThreads, 1)
osd_h_kernel(OsdHView hv0, OsdHLayout lay, OsdIO io)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    OsdHSmem s;
    carve(lay, smem_raw, &s);
    __shared__ int s_piv[3];
    __shared__ int s_nd;
    __shared__ unsigned long long s_best;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int TS = lay.ts;
    const int count = io.count_ptr ? *io.count_ptr : io.count;

    for (int item = blockIdx.x; item < count; item += gridDim.x) {
        const int cw = io.index ? io.index[item] : item;
        const OsdHView hv = io.hviews ? io.hviews[io.code_of[cw]] : hv0;
        if (hv.n == 0) continue;  // not a large-code item (uniform over the CTA)
        const int n = hv.n, m = hv.m, k = hv.k, MW = hv.mw, rows = 32 * hv.mw;
        const float* src = io.row_off   ? io.llr + io.row_off[item]
                           : io.llr_off ? io.llr + io.llr_off[cw]
                                        : io.llr + static_cast<size_t>(item) * n;
        uint8_t* info_dst = io.out_info ? (io.info_off ? io.out_info + io.info_off[cw]
                                                       : io.out_info + static_cast<size_t>(cw) * io.info_stride)
                                        : nullptr;

        // ---- 1. sort keys (descending |llr|, ties by position), hard decisions ----
        const int np = 1 << (32 - __clz(n - 1));
        for (int i = tid; i < np; i += kOsdHThreads) {
            const float x = (i < n) ? src[i] : 0.0f;
            s.keys[i] = (i < n) ? ((static_cast<unsigned long long>(0x7fffffffu - __float_as_uint(fabsf(x))) << 32) |
                                   static_cast<unsigned>(i))
                                : ~0ull;
        }
        for (int i = tid; i < ((n + 31) & ~31); i += kOsdHThreads) {
            const bool neg = (i < n) && (src[i] < 0.0f);
            const unsigned b = __ballot_sync(0xffffffffu, neg);
            if (lane == 0) s.hard[i >> 5] = b;
        }
        for (int i = tid; i < n; i += kOsdHThreads) s.row_of_col[i] = -1;
        __syncthreads();
        for (int k2 = 2; k2 <= np; k2 <<= 1) {
            for (int j2 = k2 >> 1; j2 > 0; j2 >>= 1) {
                for (int pr = tid; pr < np / 2; pr += kOsdHThreads) {
                    const int i = (pr / j2) * 2 * j2 + (pr % j2);
                    const int ixj = i + j2;
                    const bool asc = (i & k2) == 0;
                    const unsigned long long a = s.keys[i], b = s.keys[ixj];
                    if ((a > b) == asc) {
                        s.keys[i] = b;
                        s.keys[ixj] = a;
                    }
                }
                __syncthreads();
            }
        }
        for (int j = tid; j < n; j += kOsdHThreads) {
            const unsigned long long key = s.keys[j];
            s.perm[j] = static_cast<int16_t>(key & 0xffffffffull);
            s.rel[j] = __uint_as_float(0x7fffffffu - static_cast<unsigned>(key >> 32));
        }
        // ---- 2. T = identity, syndrome of the hard decisions ----
        for (int i = tid; i < rows * TS; i += kOsdHThreads) {
            const int r = i / TS, w = i - r * TS;
            s.T[i] = (r < m && w == (r >> 5)) ? (1u << (r & 31)) : 0u;
        }
        for (int r = tid; r < rows; r += kOsdHThreads) {
            unsigned par = 0;
            if (r < m)
                for (int e = hv.row_ptr[r]; e < hv.row_ptr[r + 1]; ++e) par ^= tbit(s.hard, hv.col_ind[e]);
            const unsigned b = __ballot_sync(0xffffffffu, par);
            if (lane == 0) s.syn[r >> 5] = b;
        }
        if (tid == 0) {
            s_piv[0] = s_piv[1] = s_piv[2] = INT_MAX;
            s_nd = 0;
        }
        __syncthreads();

        // ---- 3. Gauss-Jordan scan of H's columns in increasing reliability ----
        int t = 0, jstop = -1, it = 0;
        for (int j = n - 1; j >= 0; --j, ++it) {
            const int c = s.perm[j];
            const int e0 = hv.col_ptr[c], e1 = hv.col_ptr[c + 1];
            const int cur = it % 3;
            for (int r = tid; r < rows; r += kOsdHThreads) {
                const unsigned v = reduced_bit(s.T + static_cast<size_t>(r) * TS, hv.col_rows, e0, e1);
                const unsigned b = __ballot_sync(0xffffffffu, v);
                const int r0 = r & ~31;
                unsigned cand = b;
                if (r0 + 32 <= t) cand = 0u;
                else if (r0 < t) cand &= ~0u << (t - r0);
                if (lane == 0) {
                    s.vw[r >> 5] = b;
                    if (cand) atomicMin(&s_piv[cur], r0 + __ffs(cand) - 1);
                }
            }
            __syncthreads();
            const int p = s_piv[cur];
            // buffer (it+2)%3 was last read before this iteration's barrier and is next
            // written after the following one
            if (tid == 0) s_piv[(it + 2) % 3] = INT_MAX;
            if (p == INT_MAX) {  // dependent on the pivots so far: an MRB position
                if (tid == 0) s.mrb[s_nd++] = static_cast<int16_t>(j);
                continue;
            }
            if (warp == 0) {
                if (p != t) {
                    for (int w = lane; w < MW; w += 32) {
                        const uint32_t a = s.T[static_cast<size_t>(t) * TS + w];
                        s.T[static_cast<size_t>(t) * TS + w] = s.T[static_cast<size_t>(p) * TS + w];
                        s.T[static_cast<size_t>(p) * TS + w] = a;
                    }
                }
                if (lane == 0) {
                    // after the swap row t holds the pivot and row p the former row t
                    const unsigned vt = (s.vw[t >> 5] >> (t & 31)) & 1u;
                    s.vw[p >> 5] = (s.vw[p >> 5] & ~(1u << (p & 31))) | (vt << (p & 31));
                    s.vw[t >> 5] &= ~(1u << (t & 31));
                    s.row_of_col[c] = static_cast<int16_t>(t);
                    s.pivj[t] = static_cast<int16_t>(j);
                }
            }
            __syncthreads();
            {
                const uint32_t* prow = s.T + static_cast<size_t>(t) * TS;
                for (int q = warp; q < MW; q += kOsdHWarps) {
                    unsigned bits = s.vw[q];
                    while (bits) {
                        const int b = __ffs(bits) - 1;
                        bits &= bits - 1;
                        uint32_t* row = s.T + static_cast<size_t>(q * 32 + b) * TS;
                        for (int w = lane; w < MW; w += 32) row[w] ^= prow[w];
                    }
                }
            }
            __syncthreads();
            if (++t == m) {
                jstop = j;
                break;
            }
        }
        if (t < m) {  // H rank deficient: leave the BP decision in place
            __syncthreads();
            continue;
        }

        // ---- 4. flip pool: the weakest MRB positions, (|llr| ascending, position ascending) ----
        if (tid == 0) {
            int16_t* taken = reinterpret_cast<int16_t*>(s.keys);
            const int nd = s_nd, total = nd + jstop, want = hv.pool;
            int cnt = 0;
            while (cnt < total) {
                const int jj = cnt < nd ? s.mrb[cnt] : jstop - 1 - (cnt - nd);  // descending position
                if (cnt >= want && (cnt == 0 || s.rel[jj] != s.rel[taken[cnt - 1]])) break;
                taken[cnt++] = static_cast<int16_t>(jj);
            }
            for (int a = 0; a < cnt;) {  // runs of equal |llr| come in descending position: reverse them
                int b = a + 1;
                while (b < cnt && s.rel[taken[b]] == s.rel[taken[a]]) ++b;
                for (int x = a, y = b - 1; x < y; ++x, --y) {
                    const int16_t z = taken[x];
                    taken[x] = taken[y];
                    taken[y] = z;
                }
                a = b;
            }
            for (int i = 0; i < want; ++i) s.pool_j[i] = taken[i];
            s_best = ~0ull;
        }
        __syncthreads();

        // ---- 5. T s and the reduced pool columns, by pivot row ----
        const int pool = hv.pool;
        for (int r = tid; r < rows; r += kOsdHThreads) {
            const uint32_t* Tr = s.T + static_cast<size_t>(r) * TS;
            unsigned par = 0;
            for (int w = 0; w < MW; ++w) par ^= __popc(Tr[w] & s.syn[w]);
            unsigned b = __ballot_sync(0xffffffffu, par & 1u);
            if (lane == 0) s.aug[r >> 5] = b;
            for (int i = 0; i < pool; ++i) {
                const int c = s.perm[s.pool_j[i]];
                const unsigned v = reduced_bit(Tr, hv.col_rows, hv.col_ptr[c], hv.col_ptr[c + 1]);
                b = __ballot_sync(0xffffffffu, v);
                if (lane == 0) s.avec[i * MW + (r >> 5)] = b;
            }
            s.relq[r] = r < m ? s.rel[s.pivj[r]] : 0.0f;
        }
        __syncthreads();

        // ---- 6. candidates: metric in increasing sorted position, exact pruning ----
        for (int ti = tid; ti < hv.num_tests; ti += kOsdHThreads) {
            int fl[3], fj[3], nf = 0;
            if (ti > 0) {
                const uint32_t pk = hv.combos[ti - 1];
                for (int q = 0; q < 3; ++q) {
                    const int f = (pk >> (10 * q)) & 1023;
                    if (f != 1023) fl[nf++] = f;
                }
            }
            for (int q = 0; q < nf; ++q) fj[q] = s.pool_j[fl[q]];
            for (int a = 1; a < nf; ++a)  // flip positions ascending
                for (int b = a; b > 0 && fj[b - 1] > fj[b]; --b) {
                    const int z = fj[b];
                    fj[b] = fj[b - 1];
                    fj[b - 1] = z;
                }
            float acc = 0.0f;
            int fi = 0;
            bool pruned = false;
            // pivot rows in descending index hold the pivot positions in ascending order
            for (int w = MW - 1; w >= 0 && !pruned; --w) {
                unsigned word = s.aug[w];
                for (int q = 0; q < nf; ++q) word ^= s.avec[fl[q] * MW + w];
                while (word) {
                    const int b = 31 - __clz(word);
                    word &= ~(1u << b);
                    const int r = w * 32 + b;
                    const int jr = s.pivj[r];
                    while (fi < nf && fj[fi] < jr) acc = __fadd_rn(acc, s.rel[fj[fi++]]);
                    acc = __fadd_rn(acc, s.relq[r]);
                }
                const unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(&s_best);
                if (cur != ~0ull && acc > __uint_as_float(static_cast<unsigned>(cur >> 32))) pruned = true;
            }
            if (pruned) continue;
            while (fi < nf) acc = __fadd_rn(acc, s.rel[fj[fi++]]);
            atomicMin(&s_best, (static_cast<unsigned long long>(__float_as_uint(acc)) << 32) | static_cast<unsigned>(ti));
        }
        __syncthreads();

        // ---- 7. the winning codeword ----
        const unsigned long long best = s_best;
        const int bt = static_cast<int>(best & 0xffffffffull);
        int fl[3], fpos[3], nf = 0;
        if (bt > 0) {
            const uint32_t pk = hv.combos[bt - 1];
            for (int q = 0; q < 3; ++q) {
                const int f = (pk >> (10 * q)) & 1023;
                if (f != 1023) {
                    fl[nf] = f;
                    fpos[nf] = s.perm[s.pool_j[f]];
                    ++nf;
                }
            }
        }
        auto bit_at = [&](int i) -> uint8_t {
            unsigned bit = tbit(s.hard, i);
            const int r = s.row_of_col[i];
            if (r >= 0) {
                unsigned word = s.aug[r >> 5];
                for (int q = 0; q < nf; ++q) word ^= s.avec[fl[q] * MW + (r >> 5)];
                bit ^= (word >> (r & 31)) & 1u;
            } else {
                for (int q = 0; q < nf; ++q) bit ^= (fpos[q] == i) ? 1u : 0u;
            }
            return static_cast<uint8_t>(bit);
        };
        if (info_dst)
            for (int i = tid; i < k; i += kOsdHThreads) info_dst[i] = bit_at(i);
        if (io.out_code)
            for (int i = tid; i < n; i += kOsdHThreads) io.out_code[static_cast<size_t>(cw) * n + i] = bit_at(i);
        if (tid == 0) {
            if (io.used_osd) io.used_osd[cw] = 1;
            if (io.out_metric) io.out_metric[cw] = __uint_as_float(static_cast<unsigned>(best >> 32));
        }
        __syncthreads();  // shared memory is rewritten by the next item
    }
}

size_t osd_h_smem_bytes(int nmax, int mmax, int poolmax)
{
    OsdHLayout l{};
    l.nmax = nmax;
    l.np = 1;
    while (l.np < nmax) l.np <<= 1;
    l.mw = (mmax + 31) / 32;
    l.ts = l.mw | 1;
    l.poolmax = std::max(poolmax, 1);
    return carve(l, nullptr, nullptr);
}

void launch_osd_h(const OsdHView& hv, int nmax, int mmax, int poolmax, const OsdIO& io, int max_items,
                  cudaStream_t st)
{
    if (max_items <= 0) return;
    if (nmax > 32767 || poolmax > kOsdHMaxPool) throw InvalidArgument("large-code OSD: n <= 32767, pool <= 128");
    OsdHLayout l{};
    l.nmax = nmax;
    l.np = 1;
    while (l.np < nmax) l.np <<= 1;
    l.mw = (mmax + 31) / 32;
    l.ts = l.mw | 1;
    l.poolmax = std::max(poolmax, 1);
    const size_t smem = carve(l, nullptr, nullptr);
    if (smem > 227 * 1024) throw InvalidArgument("large-code OSD tables exceed shared memory (m <= 1024, n <= 4096)");
    check_cuda(cudaFuncSetAttribute(osd_h_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)),
               "cudaFuncSetAttribute(osd_h)");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, osd_h_kernel, kOsdHThreads, smem) != cudaSuccess ||
        per_sm <= 0)
        per_sm = 1;
    const int ctas = std::max(1, std::min(max_items, per_sm * device_sm_count()));
    osd_h_kernel<<<ctas, kOsdHThreads, smem, st>>>(hv, l, io);
    check_cuda(cudaGetLastError(), "osd_h_kernel launch");
}

}  // namespace sicc
