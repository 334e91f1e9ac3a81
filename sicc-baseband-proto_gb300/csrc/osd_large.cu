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
//     shared memory column-major, column c's reduced form is T h_c, the XOR
//     of the few columns of T that h_c selects (column weight <= 16).  The
//     pivots are taken 8 at a time; their combined row operation is linear in
//     a column's 8 pivot-row bits (a -> a + sum_r a_{p_r} U_r), so each
//     column of T takes it in one pass, and one warp picks the next round's
//     pivots while the others apply the current round to T;
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

constexpr int kOsdHClassThreads[kOsdHClasses] = {256, 256, 512};  // CTA size by class
constexpr int kOsdHMaxPool = 128;
constexpr int kRound = 8;  // columns of H per elimination round
constexpr int kHitsPerWarp = 96;  // a worker's list of touched columns (applied whenever it fills)
constexpr int kTabStride = 33;  // words per table entry: lanes reading different entries hit different banks

struct OsdHLayout {
    int np;       // sort length: power of two >= the longest n
    int nmax;
    int mw;       // words per row of T for the largest m
    int ts;       // column stride of T in words (odd: a warp reading one word of 32 columns hits 32 banks)
    int poolmax;
    int nnzmax;   // > 0: the columns' row lists are staged in shared memory (16-bit rows)
    int warps;    // warps per CTA
    int mlo, mhi; // the launch decodes the items of codes with mlo < m <= mhi
};

struct OsdHSmem {
    uint32_t* T;             // [32*mw + 2*kRound][ts] column-major: column i of the row-operation matrix,
                             // then two buffers of kRound reduced candidate columns
    unsigned long long* keys;// [np] sort keys; shares T's space
    int* colinfo;            // [nmax] first edge << 8 | weight of the column at each sorted position
    float* rel;              // [nmax] |llr| by sorted position j
    int16_t* perm;           // [nmax] code position at sorted position j
    int16_t* row_of_col;     // [nmax] pivot rank of a code position, -1 for the MRB
    uint32_t* hard;          // [nmax/32+1] hard decisions by code position
    uint32_t* tab;           // [2][32][kTabStride] by round parity: entry g < 16 the XOR of U_0..3 selected by g, entry
                             // 16 + g that of U_4..7; aliases vs..relq, which are first written after the
                             // elimination
    uint32_t* wv;            // [2][kRound][32] by round parity: the round's basis U_r (0 for a dependent candidate)
    uint32_t* hits;          // [warps][kHitsPerWarp] per warp: the columns a round changes, word offset in T
                             // (16 bits) | pivot-row index << 16
    uint32_t* piv;           // [mw] pivoted rows
    int16_t* order;          // [32*mw] row of the t-th pivot
    uint32_t* vs;            // [poolmax+1][32] T s and T h_f by row (before reordering)
    uint32_t* syn;           // [mw] s = H * hard by row of H
    int16_t* pivj;           // [32*mw] sorted position of the t-th pivot's column
    float* relq;             // [32*mw] |llr| of the t-th pivot's column
    int16_t* mrb;            // [nmax] dependent positions met during the scan (descending j)
    int16_t* pool_j;         // [poolmax] flip pool (sorted positions, weakest first)
    uint32_t* avec;          // [poolmax][mw] T h_f for the pool, bit t = pivot rank t
    uint32_t* aug;           // [mw] T s, bit t = pivot rank t
    int16_t* rows;           // [nnzmax] rows of H's columns (when staged)
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
    {  // the sort keys, then T (the keys are dead once the sorted order is extracted)
        const size_t bt = (rows + 2 * kRound) * l.ts * 4, bk = static_cast<size_t>(l.np) * 8;
        unsigned char* g = take(bt > bk ? bt : bk);
        t.T = reinterpret_cast<uint32_t*>(g);
        t.keys = reinterpret_cast<unsigned long long*>(g);
    }
    t.colinfo = reinterpret_cast<int*>(take(static_cast<size_t>(l.nmax) * 4));
    t.rel = reinterpret_cast<float*>(take(static_cast<size_t>(l.nmax) * 4));
    t.perm = reinterpret_cast<int16_t*>(take(static_cast<size_t>(l.nmax) * 2));
    t.row_of_col = reinterpret_cast<int16_t*>(take(static_cast<size_t>(l.nmax) * 2));
    t.hard = reinterpret_cast<uint32_t*>(take((static_cast<size_t>(l.nmax) / 32 + 1) * 4));
    t.wv = reinterpret_cast<uint32_t*>(take(2 * kRound * 32 * 4));
    t.hits = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(l.warps) * kHitsPerWarp * 4));
    t.piv = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(l.mw) * 4));
    t.order = reinterpret_cast<int16_t*>(take(rows * 2));
    t.syn = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(l.mw) * 4));
    t.pivj = reinterpret_cast<int16_t*>(take(rows * 2));
    t.mrb = reinterpret_cast<int16_t*>(take(static_cast<size_t>(l.nmax) * 2));
    t.pool_j = reinterpret_cast<int16_t*>(take(static_cast<size_t>(l.poolmax) * 2));
    {  // the tables of the elimination, then the vectors of the candidate search
        const size_t b_vs = a16((static_cast<size_t>(l.poolmax) + 1) * 32 * 4);
        const size_t b_avec = a16(static_cast<size_t>(l.poolmax) * l.mw * 4);
        const size_t b_aug = a16(static_cast<size_t>(l.mw) * 4);
        const size_t b_relq = a16(rows * 4);
        const size_t b_vec = b_vs + b_avec + b_aug + b_relq, b_tab = 2 * 32 * 33 * 4;
        unsigned char* g = take(b_vec > b_tab ? b_vec : b_tab);
        t.tab = reinterpret_cast<uint32_t*>(g);
        t.vs = reinterpret_cast<uint32_t*>(g);
        t.avec = reinterpret_cast<uint32_t*>(g ? g + b_vs : nullptr);
        t.aug = reinterpret_cast<uint32_t*>(g ? g + b_vs + b_avec : nullptr);
        t.relq = reinterpret_cast<float*>(g ? g + b_vs + b_avec + b_aug : nullptr);
    }
    t.rows = reinterpret_cast<int16_t*>(take(static_cast<size_t>(l.nnzmax) * 2));
    if (s) *s = t;
    return o;
}

__device__ __forceinline__ unsigned tbit(const uint32_t* row, int q) { return (row[q >> 5] >> (q & 31)) & 1u; }

// Slot of column q of T.  The columns a pivot touches come in runs of
// consecutive rows (the parity part of these codes is a chain); a transposed
// placement spreads a run over the 32-column chunks, hence over the warps
// that apply the pivot, instead of loading one warp with the whole run.
__device__ __forceinline__ int tslot(int q, int mw) { return (q & 31) * mw + (q >> 5); }

}  // namespace

template <int kThreads>
__global__ void __launch_bounds__(kThreads, kThreads == 256 ? 2 : 1)
osd_h_kernel(OsdHView hv0, OsdHLayout lay, OsdIO io)
{
    constexpr int kWarps = kThreads / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    OsdHSmem s;
    carve(lay, smem_raw, &s);
    __shared__ int s_rp[2][kRound];
    __shared__ int s_np[2], s_used[2], s_jstop[2];
    __shared__ unsigned long long s_best;
    __shared__ int s_item;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int TS = lay.ts;
    const int count = io.count_ptr ? *io.count_ptr : io.count;

    auto next_item = [&](int prev) -> int {  // the CTA's next work item (all threads get it)
        if (!io.work_h) return prev < 0 ? static_cast<int>(blockIdx.x) : prev + static_cast<int>(gridDim.x);
        __syncthreads();  // every thread has read the previous one
        if (tid == 0) s_item = atomicAdd(io.work_h, 1);
        __syncthreads();
        return s_item;
    };
    for (int item = next_item(-1); item < count; item = next_item(item)) {
        const int cw = io.index ? io.index[item] : item;
        const OsdHView hv = io.hviews ? io.hviews[io.code_of[cw]] : hv0;
        if (hv.n == 0 || hv.m <= lay.mlo || hv.m > lay.mhi) continue;  // another kernel's item (uniform over the CTA)
        const int n = hv.n, m = hv.m, k = hv.k, MW = hv.mw, rows = 32 * hv.mw;
        const float* src = io.row_off   ? io.llr + io.row_off[item]
                           : io.llr_off ? io.llr + io.llr_off[cw]
                                        : io.llr + static_cast<size_t>(item) * n;
        uint8_t* info_dst = io.out_info ? (io.info_off ? io.out_info + io.info_off[cw]
                                                       : io.out_info + static_cast<size_t>(cw) * io.info_stride)
                                        : nullptr;

        // ---- 1. sort keys (descending |llr|, ties by position), hard decisions ----
        const int np = 1 << (32 - __clz(n - 1));
        for (int i = tid; i < np; i += kThreads) {
            const float x = (i < n) ? src[i] : 0.0f;
            s.keys[i] = (i < n) ? ((static_cast<unsigned long long>(0x7fffffffu - __float_as_uint(fabsf(x))) << 32) |
                                   static_cast<unsigned>(i))
                                : ~0ull;
        }
        for (int i = tid; i < ((n + 31) & ~31); i += kThreads) {
            const bool neg = (i < n) && (src[i] < 0.0f);
            const unsigned b = __ballot_sync(0xffffffffu, neg);
            if (lane == 0) s.hard[i >> 5] = b;
        }
        for (int i = tid; i < n; i += kThreads) s.row_of_col[i] = -1;
        __syncthreads();
        // bitonic sort (np >= 32): compare-exchange distances j2 >= 32 through shared memory, one
        // barrier each; the distances below 32 of each merge level on registers within a warp
        // (lane = element index mod 32), one barrier per level
        auto warp_stages = [&](int k2lo, int k2hi, int j2top) {
            for (int b0 = warp * 32; b0 < np; b0 += kThreads) {
                const int i = b0 + lane;
                unsigned long long v = s.keys[i];
                for (int k2 = k2lo; k2 <= k2hi; k2 <<= 1) {
                    const bool asc = (i & k2) == 0;
                    for (int j2 = min(k2 >> 1, j2top); j2 > 0; j2 >>= 1) {
                        const unsigned long long o =
                            (static_cast<unsigned long long>(__shfl_xor_sync(0xffffffffu, static_cast<unsigned>(v >> 32), j2)) << 32) |
                            __shfl_xor_sync(0xffffffffu, static_cast<unsigned>(v), j2);
                        const bool take_min = ((i & j2) == 0) == asc;
                        v = take_min ? (o < v ? o : v) : (o > v ? o : v);
                    }
                }
                s.keys[i] = v;
            }
            __syncthreads();
        };
        warp_stages(2, 32, 16);
        for (int k2 = 64; k2 <= np; k2 <<= 1) {
            for (int j2 = k2 >> 1; j2 >= 32; j2 >>= 1) {
                for (int pr = tid; pr < np / 2; pr += kThreads) {
                    const int i = ((pr & ~(j2 - 1)) << 1) | (pr & (j2 - 1));  // j2 is a power of two
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
            warp_stages(k2, k2, 16);
        }
        for (int j = tid; j < n; j += kThreads) {
            const unsigned long long key = s.keys[j];
            s.perm[j] = static_cast<int16_t>(key & 0xffffffffull);
            s.rel[j] = __uint_as_float(0x7fffffffu - static_cast<unsigned>(key >> 32));
        }
        __syncthreads();  // T overwrites the keys
        // ---- 2. T = identity (column-major), syndrome of the hard decisions ----
        for (int i = tid; i < rows * TS; i += kThreads) s.T[i] = 0u;
        __syncthreads();
        for (int col = tid; col < m; col += kThreads)
            s.T[static_cast<size_t>(tslot(col, MW)) * TS + (col >> 5)] = 1u << (col & 31);
        for (int r = tid; r < rows; r += kThreads) {
            unsigned par = 0;
            if (r < m)
                for (int e = hv.row_ptr[r]; e < hv.row_ptr[r + 1]; ++e) par ^= tbit(s.hard, hv.col_ind[e]);
            const unsigned b = __ballot_sync(0xffffffffu, par);
            if (lane == 0) s.syn[r >> 5] = b;
        }
        for (int w = tid; w < MW; w += kThreads) s.piv[w] = 0u;
        // column of H at each sorted position: first edge << 8 | weight
        const bool staged = lay.nnzmax > 0;
        if (staged)
            for (int e = tid; e < hv.col_ptr[n]; e += kThreads) s.rows[e] = static_cast<int16_t>(hv.col_rows[e]);
        int* colinfo = s.colinfo;
        for (int j = tid; j < n; j += kThreads) {
            const int c = s.perm[j];
            const int e0 = hv.col_ptr[c];
            colinfo[j] = (e0 << 8) | (hv.col_ptr[c + 1] - e0);
        }
        __syncthreads();

        // ---- 3. Gauss-Jordan scan of H's columns in increasing reliability ----
        // A column c's reduced form is v = T h_c (the XOR of the columns of T that
        // h_c selects); its pivot is the lowest unpivoted row p with v_p = 1, and
        // the pivot's row operation T <- (I + W e_p^T) T, W = v + e_p, turns
        // column c into e_p and leaves earlier pivot columns alone.
        // Columns are taken kRound at a time, in rounds pipelined over one
        // barrier each.  In the barrier interval of round k:
        //   * warp 0 takes round k's candidates (reduced against T before
        //     round k-1), applies round k-1's operation to them, and picks
        //     their pivots in order; each pivot's operation is applied at once
        //     to the later candidates and to the round's basis,
        //       a -> a + sum_r a_{p_r} U_r,  U_r <- U_r + U_r[p] W for a new pivot p
        //     (a_{p_r} a column's bits before the round, U_r = 0 for a dependent
        //     candidate);
        //   * warps 1..15 tabulate round k-1's basis by index nibble, and the
        //     worker warps apply round k-1's operation to the columns of T they
        //     own (the pivot-row bits of a column form its index; columns with a
        //     nonzero index take its two table entries), meet on a named
        //     barrier, and kRound of them reduce round k+1's candidates against
        //     T.  In 512-thread CTAs (m > 640, the update bounds the round) the
        //     workers are warps 1..15; in 256-thread CTAs (the selection bounds
        //     it) warp 0 keeps its scheduler (warps w = 0 mod 4) to itself and
        //     the workers are the warps w != 0 mod 4.
        auto rows_of = [&](int jj, int& e0, int& cnt) -> int {  // one row of column jj per lane
            const int ci = colinfo[jj];
            e0 = ci >> 8;
            cnt = ci & 255;
            return lane < cnt ? (staged ? static_cast<int>(s.rows[e0 + lane]) : hv.col_rows[e0 + lane]) : -1;
        };
        auto reduce_column = [&](int myrow, int e0, int cnt) -> unsigned {  // T h_c, word `lane`
            unsigned v = 0u;
            for (int e = 0; e < cnt && e < 32; e += 8) {  // groups of 8 loads in flight together
                unsigned part[8];
#pragma unroll
                for (int x = 0; x < 8; ++x) {
                    const int q = __shfl_sync(0xffffffffu, myrow, (e + x) & 31);
                    part[x] = (e + x < cnt && lane < MW) ? s.T[static_cast<size_t>(tslot(q, MW)) * TS + lane] : 0u;
                }
                v ^= (part[0] ^ part[1]) ^ (part[2] ^ part[3]) ^ (part[4] ^ part[5]) ^ (part[6] ^ part[7]);
            }
            for (int e = 32; e < cnt; ++e)  // columns heavier than 32
                if (lane < MW) v ^= s.T[static_cast<size_t>(tslot(hv.col_rows[e0 + e], MW)) * TS + lane];
            return v;
        };
        // candidate slot r of buffer b: rows + b * kRound + r
        auto reduce_candidate = [&](int jj, int slot) {
            unsigned v = 0u;
            if (jj >= 0) {
                int e0, cnt;
                const int rw = rows_of(jj, e0, cnt);
                v = reduce_column(rw, e0, cnt);
            }
            if (lane < MW) s.T[static_cast<size_t>(slot) * TS + lane] = v;
        };
        for (int c = warp; c < kRound; c += kWarps) reduce_candidate(n - 1 - c, rows + c);
        __syncthreads();
        const int lg = MW <= 1 ? 0 : 32 - __clz(MW - 1);  // table words per entry: 2^lg >= MW
        uint32_t* seg = s.hits + warp * kHitsPerWarp;
        constexpr bool narrow = kThreads < 512;  // the small-T classes: selection-bound
        const int nworkers = narrow ? kWarps - kWarps / 4 : kWarps - 1;
        const bool worker = warp != 0 && (!narrow || (warp & 3) != 0);
        const int wi = narrow ? warp - (warp >> 2) - 1 : warp - 1;  // worker index
        int t = 0, j = n - 1, nd = 0, jstop = -1;          // after the rounds selected so far
        int pt = 0, pj = 0, pnd = 0, pnp = 0, pused = 0;   // the round whose update is pending
        bool pending = false;
        unsigned pivw = 0u;  // warp 0: pivoted rows, word `lane`
        unsigned Up[kRound];  // warp 0: the pending round's basis, and its pivot rows as word offset + bit
        int pwo[kRound];
        unsigned pwb[kRound];
#pragma unroll
        for (int r = 0; r < kRound; ++r) {
            Up[r] = 0u;
            pwo[r] = 0;
            pwb[r] = 0u;
        }
        for (int k = 0;; ++k) {
            const bool select = j >= 0 && t < m;
            if (!select && !pending) break;
            const int cb = k & 1;
            if (warp == 0) {
                if (select) {
                    // branch-free, so that the loads and the candidates' chains overlap
                    unsigned v[kRound], U[kRound];
                    int P[kRound];
#pragma unroll
                    for (int r = 0; r < kRound; ++r) {
                        v[r] = lane < MW ? s.T[static_cast<size_t>(rows + cb * kRound + r) * TS + lane] : 0u;
                        U[r] = 0u;
                        P[r] = -1;
                    }
                    {  // the previous round's operation, not yet in the reduced candidates (a no-op in round 0)
                        // lane l: candidate l mod kRound's bits at that round's pivot rows
                        const uint32_t* col = s.T + static_cast<size_t>(rows + cb * kRound + (lane & (kRound - 1))) * TS;
                        unsigned idx = 0u;
#pragma unroll
                        for (int i = 0; i < kRound; ++i)
                            if (col[pwo[i]] & pwb[i]) idx |= 1u << i;
#pragma unroll
                        for (int r = 0; r < kRound; ++r) {
                            const unsigned ir = __shfl_sync(0xffffffffu, idx, r);
#pragma unroll
                            for (int i = 0; i < kRound; ++i) v[r] ^= ((ir >> i) & 1u) ? Up[i] : 0u;
                        }
                    }
                    int np = 0, used = 0, js = -1;
                    int pl[kRound];  // the pivot's position on its lane, -1 elsewhere
#pragma unroll
                    for (int r = 0; r < kRound; ++r) {
                        const bool valid = j - r >= 0 && t + np < m;  // warp-uniform
                        // each lane: its lowest unpivoted set row (as a mask); the lowest such lane
                        // holds the pivot.  The later candidates (c > r) and the basis (c < r) at
                        // each lane's row are balloted at once, before the pivot lane is known, so
                        // the chain from one candidate to the next is one ballot deep: the pivot
                        // lane's bit of each ballot is that vector's bit at the pivot row.
                        const unsigned x = valid ? (v[r] & ~pivw) : 0u;
                        const unsigned lb = x & (0u - x);
                        const unsigned bx = __ballot_sync(0xffffffffu, x != 0u);
                        unsigned bc[kRound];
#pragma unroll
                        for (int c = 0; c < kRound; ++c)
                            bc[c] = c > r   ? __ballot_sync(0xffffffffu, (v[c] & lb) != 0u)
                                    : c < r ? __ballot_sync(0xffffffffu, (U[c] & lb) != 0u)
                                            : 0u;
                        const bool piv = bx != 0u;
                        const unsigned sel = bx & (0u - bx);  // the pivot lane's bit (0: no pivot)
                        const bool me = (sel >> lane) & 1u;
                        const unsigned W = me ? (v[r] ^ lb) : v[r];
#pragma unroll
                        for (int c = 0; c < kRound; ++c) {
                            if (c > r) v[c] ^= (bc[c] & sel) ? W : 0u;
                            if (c < r) U[c] ^= (bc[c] & sel) ? W : 0u;
                        }
                        U[r] = piv ? W : 0u;
                        pl[r] = me ? lane * 32 + __ffs(lb) - 1 : -1;
                        pivw |= me ? lb : 0u;
                        np += piv ? 1 : 0;
                        js = (piv && t + np == m) ? j - r : js;
                        used = valid ? r + 1 : used;
                    }
#pragma unroll
                    for (int r = 0; r < kRound; ++r)
                        P[r] = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(pl[r] + 1))) - 1;
#pragma unroll
                    for (int r = 0; r < kRound; ++r) {  // every lane stores (same values): no divergence
                        s.wv[(cb * kRound + r) * 32 + lane] = U[r];
                        s_rp[cb][r] = P[r];
                        Up[r] = U[r];
                        pwo[r] = P[r] >= 0 ? P[r] >> 5 : 0;
                        pwb[r] = P[r] >= 0 ? 1u << (P[r] & 31) : 0u;
                    }
                    s_np[cb] = np;
                    s_used[cb] = used;
                    s_jstop[cb] = js;
                }
            } else {
                if (pending) {
                    const int pb = cb ^ 1;
                    if (pnp > 0) {  // tables of the pending round's basis (entries 0 and 16 are 0)
                        uint32_t* tb = s.tab + pb * 32 * kTabStride;
                        const uint32_t* U = s.wv + pb * kRound * 32;
                        for (int q = tid - 32; q < (32 << lg); q += kThreads - 32) {
                            const int e = q >> lg, w = q & ((1 << lg) - 1), h = (e >> 4) * 4;
                            unsigned acc = 0u;
#pragma unroll
                            for (int b = 0; b < 4; ++b)
                                if ((e >> b) & 1) acc ^= U[(h + b) * 32 + w];
                            tb[e * kTabStride + w] = acc;
                        }
                        asm volatile("bar.sync 1, %0;" ::"r"(kThreads - 32) : "memory");
                    }
                    int P[kRound];
#pragma unroll
                    for (int r = 0; r < kRound; ++r) P[r] = s_rp[pb][r];
                    if (warp == kWarps - 1 && lane < pused) {  // pivot ranks and dependent positions
                        int bp = 0, bd = 0, pr = -1;
#pragma unroll
                        for (int r = 0; r < kRound; ++r) {
                            if (r < lane) {
                                if (P[r] >= 0) ++bp;
                                else ++bd;
                            }
                            if (r == lane) pr = P[r];
                        }
                        if (pr >= 0) {
                            s.order[pt + bp] = static_cast<int16_t>(pr);
                            s.row_of_col[s.perm[pj - lane]] = static_cast<int16_t>(pt + bp);
                            s.pivj[pt + bp] = static_cast<int16_t>(pj - lane);
                        } else {
                            s.mrb[pnd + bd] = static_cast<int16_t>(pj - lane);  // dependent: an MRB position
                        }
                    }
                    if (pnp > 0 && worker) {
                        // gather: one thread per owned column, the touched ones listed; then one
                        // thread per listed column walks its MW words (three loads, one store each)
                        const uint32_t* tb = s.tab + pb * 32 * kTabStride;
                        int woff[kRound];
                        unsigned wbit[kRound];
#pragma unroll
                        for (int r = 0; r < kRound; ++r) {
                            woff[r] = P[r] >= 0 ? P[r] >> 5 : 0;
                            wbit[r] = P[r] >= 0 ? 1u << (P[r] & 31) : 0u;
                        }
                        auto walk = [&](int nh) {
                            __syncwarp();
                            for (int h = lane; h < nh; h += 32) {
                                const unsigned e = seg[h];
                                uint32_t* c = s.T + (e & 0xffffu);
                                const unsigned idx = e >> 16;
                                const uint32_t* lo = tb + (idx & 15u) * kTabStride;
                                const uint32_t* hi = tb + (16u + (idx >> 4)) * kTabStride;
                                int w = 0;
                                for (; w + 4 <= MW; w += 4) {
                                    const unsigned a0 = c[w] ^ lo[w] ^ hi[w];
                                    const unsigned a1 = c[w + 1] ^ lo[w + 1] ^ hi[w + 1];
                                    const unsigned a2 = c[w + 2] ^ lo[w + 2] ^ hi[w + 2];
                                    const unsigned a3 = c[w + 3] ^ lo[w + 3] ^ hi[w + 3];
                                    c[w] = a0;
                                    c[w + 1] = a1;
                                    c[w + 2] = a2;
                                    c[w + 3] = a3;
                                }
                                for (; w < MW; ++w) c[w] ^= lo[w] ^ hi[w];
                            }
                            __syncwarp();  // the list is rewritten next
                        };
                        int nh = 0;
                        for (int b0 = wi * 32; b0 < rows; b0 += nworkers * 32) {
                            if (nh > kHitsPerWarp - 32) {  // the list is full: apply it first
                                walk(nh);
                                nh = 0;
                            }
                            const int slot = b0 + lane;
                            unsigned idx = 0u;
                            if (slot < rows) {
                                const uint32_t* col = s.T + slot * TS;
#pragma unroll
                                for (int r = 0; r < kRound; ++r)
                                    if (col[woff[r]] & wbit[r]) idx |= 1u << r;
                            }
                            const unsigned bal = __ballot_sync(0xffffffffu, idx != 0u);
                            if (idx) seg[nh + __popc(bal & ((1u << lane) - 1u))] = static_cast<unsigned>(slot * TS) | (idx << 16);
                            nh += __popc(bal);
                        }
                        walk(nh);
                    }
                }
                // T is final for the pending round before the next candidates read it
                asm volatile("bar.sync 1, %0;" ::"r"(kThreads - 32) : "memory");
                if (select && worker)
                    for (int c = wi; c < kRound; c += nworkers)
                        reduce_candidate(j - kRound - c, rows + (cb ^ 1) * kRound + c);
            }
            __syncthreads();
            pending = select;
            if (select) {
                pnp = s_np[cb];
                pused = s_used[cb];
                pt = t;
                pj = j;
                pnd = nd;
                t += pnp;
                if (t == m) jstop = s_jstop[cb];
                nd += pused - pnp;
                j -= pused;
            }
        }
        if (t < m) {  // H rank deficient: leave the BP decision in place
            __syncthreads();
            continue;
        }

        // ---- 4. flip pool: the weakest MRB positions, (|llr| ascending, position ascending) ----
        // The MRB positions in descending sorted position -- the dependent ones met during the
        // scan, then jstop-1 .. 0 -- come in ascending |llr|; ties come in descending position,
        // so the pool entry i is taken from the mirror image of i within its run of equal |llr|
        // (the runs found by binary search: |llr| is non-decreasing along that order).
        {
            const int total = nd + jstop, want = hv.pool;  // nd and jstop: the same in every thread
            auto mrb_at = [&](int c) -> int { return c < nd ? s.mrb[c] : jstop - 1 - (c - nd); };
            // |llr| compared as bit patterns, the order the sort used (a permutation whatever the values)
            auto relbits = [&](int c) -> unsigned { return __float_as_uint(s.rel[mrb_at(c)]); };
            for (int i = tid; i < want; i += kThreads) {
                const unsigned ri = relbits(i);
                int lo = 0, hi = i;  // first index with |llr| >= ri
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (relbits(mid) < ri) lo = mid + 1;
                    else hi = mid;
                }
                const int a = lo;
                lo = i + 1;
                hi = total;  // first index with |llr| > ri
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (relbits(mid) > ri) hi = mid;
                    else lo = mid + 1;
                }
                s.pool_j[i] = static_cast<int16_t>(mrb_at(a + lo - 1 - i));
            }
            if (tid == 0) s_best = ~0ull;
        }
        __syncthreads();

        // ---- 5. T s and the reduced pool columns, then in pivot order ----
        const int pool = hv.pool;
        for (int i = tid; i < (pool + 1) * 32; i += kThreads) s.vs[i] = 0u;
        __syncthreads();
        {
            // T s: XOR of the columns of T selected by s, spread over the warps
            unsigned acc = 0u;
            for (int q = warp; q < m; q += kWarps)
                if (lane < MW && tbit(s.syn, q)) acc ^= s.T[static_cast<size_t>(tslot(q, MW)) * TS + lane];
            if (lane < MW && acc) atomicXor(&s.vs[lane], acc);
            // T h_f for the flip pool, one warp per column
            for (int i = warp; i < pool; i += kWarps) {
                const int c = s.perm[s.pool_j[i]];
                unsigned v = 0u;
                if (lane < MW)
                    for (int e = hv.col_ptr[c]; e < hv.col_ptr[c + 1]; ++e)
                        v ^= s.T[static_cast<size_t>(tslot(hv.col_rows[e], MW)) * TS + lane];
                if (lane < MW) s.vs[(i + 1) * 32 + lane] = v;
            }
        }
        __syncthreads();
        // bit t of an ordered vector = bit order[t] of the row-indexed one (8 vectors' loads in flight)
        for (int r = tid; r < rows; r += kThreads) {
            const int q = r < m ? s.order[r] : -1;
            const int qw = q >= 0 ? q >> 5 : 0;
            const unsigned qb = q >= 0 ? 1u << (q & 31) : 0u;
            for (int v0 = 0; v0 <= pool; v0 += 8) {
                unsigned bits[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) bits[u] = v0 + u <= pool ? s.vs[(v0 + u) * 32 + qw] & qb : 0u;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const unsigned b = __ballot_sync(0xffffffffu, bits[u] != 0u);
                    const int vi = v0 + u;
                    if (lane == 0 && vi <= pool) (vi == 0 ? s.aug : s.avec + (vi - 1) * MW)[r >> 5] = b;
                }
            }
        }
        for (int r = tid; r < rows; r += kThreads) s.relq[r] = r < m ? s.rel[s.pivj[r]] : 0.0f;
        __syncthreads();

        // ---- 6. candidates: metric in increasing sorted position, exact pruning ----
        // Bit t of T s (+ T h_f) marks a differing pivot position; pivot ranks in descending
        // order hold the positions in ascending order, so the metric walks the bits from the
        // top.  A flipped position f joins the sum before the first rank t < cut(f), the
        // number of pivots after it.  Four set bits are taken at a time, their |llr| loaded
        // together; the additions stay in order.
        for (int ti = tid; ti < hv.num_tests; ti += kThreads) {
            int fa = -1, fb = -1, fc = -1;  // pool indices of the flips
            if (ti > 0) {
                const uint32_t pk = hv.combos[ti - 1];
                const int f0 = pk & 1023, f1 = (pk >> 10) & 1023, f2 = (pk >> 20) & 1023;
                fa = f0 != 1023 ? f0 : -1;
                fb = f1 != 1023 ? f1 : -1;
                fc = f2 != 1023 ? f2 : -1;
            }
            // flip positions ascending (absent: INT_MAX), their |llr| and cuts
            int j0 = fa >= 0 ? s.pool_j[fa] : INT_MAX, j1 = fb >= 0 ? s.pool_j[fb] : INT_MAX,
                j2 = fc >= 0 ? s.pool_j[fc] : INT_MAX;
            if (j0 > j1) { const int z = j0; j0 = j1; j1 = z; }
            if (j1 > j2) { const int z = j1; j1 = j2; j2 = z; }
            if (j0 > j1) { const int z = j0; j0 = j1; j1 = z; }
            auto cut_of = [&](int jf) -> int {  // pivots at positions above jf (pivj decreases with rank)
                if (jf == INT_MAX) return -1;
                int lo = 0, hi = m;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (s.pivj[mid] > jf) lo = mid + 1;
                    else hi = mid;
                }
                return lo;
            };
            const int c0 = cut_of(j0), c1 = cut_of(j1), c2 = cut_of(j2);
            const float r0 = j0 != INT_MAX ? s.rel[j0] : 0.0f, r1 = j1 != INT_MAX ? s.rel[j1] : 0.0f,
                        r2 = j2 != INT_MAX ? s.rel[j2] : 0.0f;
            {  // the flipped positions' own sum (in position order) bounds the metric from below
                const float lb = __fadd_rn(__fadd_rn(r0, r1), r2);
                const unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(&s_best);
                if (cur != ~0ull && lb > __uint_as_float(static_cast<unsigned>(cur >> 32))) continue;
            }
            int fi = 0;  // flips added so far
            int ncut = c0;
            float nrel = r0;
            const uint32_t* va = fa >= 0 ? s.avec + fa * MW : nullptr;
            const uint32_t* vb = fb >= 0 ? s.avec + fb * MW : nullptr;
            const uint32_t* vc = fc >= 0 ? s.avec + fc * MW : nullptr;
            float acc = 0.0f;
            bool pruned = false;
            for (int w = MW - 1; w >= 0 && !pruned; --w) {
                unsigned word = s.aug[w];
                if (va) word ^= va[w];
                if (vb) word ^= vb[w];
                if (vc) word ^= vc[w];
                while (word) {
                    int bq[4];
                    float rq[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        bq[u] = word ? 31 - __clz(word) : -1;
                        if (bq[u] >= 0) word &= ~(1u << bq[u]);
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) rq[u] = bq[u] >= 0 ? s.relq[w * 32 + bq[u]] : 0.0f;
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        if (bq[u] < 0) break;
                        const int t = w * 32 + bq[u];
                        while (t < ncut) {  // flipped positions below this pivot's
                            acc = __fadd_rn(acc, nrel);
                            ++fi;
                            ncut = fi == 1 ? c1 : fi == 2 ? c2 : -1;
                            nrel = fi == 1 ? r1 : r2;
                        }
                        acc = __fadd_rn(acc, rq[u]);
                    }
                }
                const unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(&s_best);
                if (cur != ~0ull && acc > __uint_as_float(static_cast<unsigned>(cur >> 32))) pruned = true;
            }
            if (pruned) continue;
            while (ncut >= 0) {  // flipped positions above every differing pivot position
                acc = __fadd_rn(acc, nrel);
                ++fi;
                ncut = fi == 1 ? c1 : fi == 2 ? c2 : -1;
                nrel = fi == 1 ? r1 : r2;
            }
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
            for (int i = tid; i < k; i += kThreads) info_dst[i] = bit_at(i);
        if (io.out_code)
            for (int i = tid; i < n; i += kThreads) io.out_code[static_cast<size_t>(cw) * n + i] = bit_at(i);
        if (tid == 0) {
            if (io.used_osd) io.used_osd[cw] = 1;
            if (io.out_metric) io.out_metric[cw] = __uint_as_float(static_cast<unsigned>(best >> 32));
        }
        __syncthreads();  // shared memory is rewritten by the next item
    }
}

namespace {

OsdHLayout osd_h_layout(const OsdHBounds& bd, int threads, int mlo, int mhi)
{
    OsdHLayout l{};
    l.nmax = bd.nmax;
    l.np = 1;
    while (l.np < bd.nmax) l.np <<= 1;
    l.mw = (bd.mmax + 31) / 32;
    l.ts = l.mw | 1;
    l.poolmax = std::max(bd.poolmax, 1);
    l.warps = threads / 32;
    l.mlo = mlo;
    l.mhi = mhi;
    l.nnzmax = 0;
    return l;
}

template <int kThreads>
void launch_osd_h_class(const OsdHBounds& bd, int mlo, int mhi, const OsdIO& io_all, int max_items, cudaStream_t st,
                        int cls)
{
    OsdIO io = io_all;  // the class's own work counter
    io.work_h = io_all.work_h ? io_all.work_h + cls : nullptr;
    OsdHLayout l = osd_h_layout(bd, kThreads, mlo, mhi);
    size_t smem = carve(l, nullptr, nullptr);
    if (smem > 227 * 1024) throw InvalidArgument("large-code OSD tables exceed shared memory (m <= 1024, n <= 4096)");
    // stage the columns' row lists when they fit as well, and keep the class's CTAs per SM
    const size_t per_sm_bytes = kThreads == 512 ? 227 * 1024 : 112 * 1024;  // two 256-thread CTAs per SM
    l.nnzmax = bd.nnzmax;
    if (bd.nnzmax <= 0 || carve(l, nullptr, nullptr) > (smem <= per_sm_bytes ? per_sm_bytes : 227 * 1024)) l.nnzmax = 0;
    smem = carve(l, nullptr, nullptr);
    // the two 256-thread classes share this kernel with different sizes: the limit only grows
    check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(osd_h_kernel<kThreads>), smem),
               "cudaFuncSetAttribute(osd_h)");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, osd_h_kernel<kThreads>, kThreads, smem) != cudaSuccess ||
        per_sm <= 0)
        per_sm = 1;
    const int ctas = std::max(1, std::min(max_items, per_sm * device_sm_count()));
    osd_h_kernel<kThreads><<<ctas, kThreads, smem, st>>>(OsdHView{}, l, io);
    check_cuda(cudaGetLastError(), "osd_h_kernel launch");
}

}  // namespace

void OsdHBounds::add(int n, int m, int pool, int nnz)
{
    nmax = std::max(nmax, n);
    mmax = std::max(mmax, m);
    poolmax = std::max(poolmax, pool);
    nnzmax = std::max(nnzmax, nnz);
}

size_t osd_h_smem_bytes(int nmax, int mmax, int poolmax)
{  // without the staged row lists
    OsdHBounds bd;
    bd.add(nmax, mmax, poolmax, 0);
    const int c = osd_h_class(mmax);
    const OsdHLayout l = osd_h_layout(bd, kOsdHClassThreads[c], 0, 1024);
    return carve(l, nullptr, nullptr);
}

void launch_osd_h(const OsdHBounds* cls, const OsdIO& io, int max_items, cudaStream_t st, const cudaStream_t* side,
                  cudaEvent_t fork, const cudaEvent_t* join)
{
    if (max_items <= 0) return;
    int present = 0;
    for (int c = 0; c < kOsdHClasses; ++c) {
        if (cls[c].empty()) continue;
        ++present;
        if (cls[c].nmax > 32767 || cls[c].poolmax > kOsdHMaxPool)
            throw InvalidArgument("large-code OSD: n <= 32767, pool <= 128");
        if (cls[c].mmax > kOsdHClassMaxM[c]) throw InvalidArgument("large-code OSD: code in the wrong class (m <= 1024)");
    }
    if (present == 0) return;
    if (io.work_h) check_cuda(cudaMemsetAsync(io.work_h, 0, kOsdHClasses * sizeof(int), st), "reset OSD work counters");
    // the classes run side by side: the first present one on st, the others on side streams
    const bool fan = present > 1 && side && fork && join;
    if (fan) check_cuda(cudaEventRecord(fork, st), "cudaEventRecord(osd fork)");
    int used = 0;
    for (int c = kOsdHClasses - 1; c >= 0; --c) {
        if (cls[c].empty()) continue;
        cudaStream_t cs = st;
        if (fan && used > 0) {
            cs = side[used - 1];
            check_cuda(cudaStreamWaitEvent(cs, fork, 0), "cudaStreamWaitEvent(osd fork)");
        }
        const int mlo = c == 0 ? 0 : kOsdHClassMaxM[c - 1];
        if (kOsdHClassThreads[c] == 256) launch_osd_h_class<256>(cls[c], mlo, kOsdHClassMaxM[c], io, max_items, cs, c);
        else launch_osd_h_class<512>(cls[c], mlo, kOsdHClassMaxM[c], io, max_items, cs, c);
        if (fan && used > 0) {
            check_cuda(cudaEventRecord(join[used - 1], cs), "cudaEventRecord(osd join)");
            check_cuda(cudaStreamWaitEvent(st, join[used - 1], 0), "cudaStreamWaitEvent(osd join)");
        }
        ++used;
    }
}

}  // namespace sicc
