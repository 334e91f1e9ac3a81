// OFDM receive kernels for sm_103a.
//
// sync_kernel (one CTA per frame and pass of 4352 candidates) restates the CPU receiver's frame search
// (uhd_ldpc_ofdm_link.cpp:5123-5329): Schmidl-Cox metric
//   P(d) = sum_{i<L} conj(x[d+i]) x[d+i+L],  E1 = sum |x[d+i]|^2,  E2 = sum |x[d+i+L]|^2,
//   metric(d) = |P|^2 / max(E1*E2, 1e-18);
// the earliest candidate over the threshold (or the global maximum), then a
// full-preamble cross-correlation refinement within +-radius, then the CFO
// arg(sum conj(x[s+i]) x[s+i+L]) * fs / (2 pi L).  Candidates are scanned in
// passes of 256 x 17 from a shared-memory copy of the samples: each pass
// computes the window sums at 256 chunk starts warp-cooperatively and slides
// them 17 candidates per thread (the odd chunk keeps shared-memory reads on
// distinct banks).  Every pass publishes its result to global scratch and the
// last pass of a frame to finish resolves the frame.
//
// demod_kernel (grid = frames x data-symbol groups) fuses the demodulator of
// gpu_ofdm_pipeline.cu:566-672 / uhd_ldpc_ofdm_link.cpp:5350-5521: CFO
// derotation and CP strip while loading, a shared-memory Stockham FFT
// (radix 4, plus one radix-2 stage for odd log2 N), LS pilot estimates with
// linear interpolation, MMSE equalisation and max-log LLRs.  The max-log
// search runs per constellation axis: for Gray square QAM the minimum of
// fl(dI^2) + fl(dQ^2) over a bit-constrained set splits into the two axis
// minima (single-precision addition is monotone in each argument), so the
// result equals the exhaustive 2^bps search of the reference bit for bit
// given the same equalised symbol.
#include "ofdm_kernels.h"

#include <algorithm>
#include <cfloat>

#include <cstdint>

namespace sicc {

namespace {

constexpr int kSyncThreads = 256;
constexpr int kSyncChunk = 17;
constexpr int kSyncPass = kSyncThreads * kSyncChunk;
constexpr int kMaxRefine = 1024;  // 2 * radius + 1
constexpr int kMaxRadius = 511;

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                       __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

__device__ __forceinline__ float2 cmulconj(float2 a, float2 b)  // a * conj(b)
{
    return make_float2(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                       __fsub_rn(__fmul_rn(a.y, b.x), __fmul_rn(a.x, b.y)));
}

__device__ __forceinline__ float cnorm(float2 a) { return __fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)); }

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace

// One search result per pass, published to global scratch for the CTA that
// resolves the frame.
struct PassResult {
    int key;      // mode 0: earliest successful candidate (INT_MAX: none); mode 1: position of the maximum (-1: none)
    int start;    // mode 0: refined start
    float fine;   // mode 0: refined metric; mode 1: the maximum coarse metric
    float coarse; // mode 0: coarse metric at the candidate
};

// Full-preamble correlation metric of candidate dd, one warp: lane-strided
// products accumulated per lane with fused multiply-adds, then a butterfly
// sum.  Samples come from the shared window when it covers them
// (win[i] = x[wbase + i]).
__device__ __forceinline__ float fine_metric(const float2* __restrict__ x, const float2* win, int wbase, int wlen, int dd,
                                             const float2* __restrict__ preamble, int pre, float pre_energy, int lane)
{
    float cr = 0.f, ci = 0.f, eng = 0.f;
    const bool local = dd >= wbase && dd + pre <= wbase + wlen;
    for (int i = lane; i < pre; i += 32) {
        const float2 y = local ? win[dd - wbase + i] : x[dd + i];
        const float2 q = preamble[i];
        cr = fmaf(y.x, q.x, fmaf(y.y, q.y, cr));    // Re(y conj(q))
        ci = fmaf(y.y, q.x, fmaf(-y.x, q.y, ci));   // Im(y conj(q))
        eng = fmaf(y.x, y.x, fmaf(y.y, y.y, eng));  // |y|^2
    }
    cr = warp_sum(cr);
    ci = warp_sum(ci);
    eng = warp_sum(eng);
    return (cr * cr + ci * ci) / fmaxf(eng * pre_energy, 1e-18f);
}

// Shared-memory working set of a frame search by one CTA.
struct SyncShared {
    float2* win;      // [kSyncPass + pre_len] the pass's samples (rounded up to an even count: the
                      // float4 chunk sums after the metric stay 16-byte aligned)
    float* metric;    // [kSyncPass] coarse metric
    float4* chunk;    // [kSyncThreads] window sums at chunk starts: P.re, P.im, E1, E2
    float* memo;      // [kSyncPass + 2 * kMaxRadius] fine metric around crossings
    float* red;       // [4][kSyncThreads / 32] reductions
    float* rmetric;   // [kMaxRefine] mode-1 refinement
    int* s_key;       // [kSyncThreads / 32]
    PassResult* s_res;
};

__device__ __forceinline__ SyncShared sync_shared(unsigned char* smem_raw, int pre_len, float* red, float* rmetric,
                                                  int* s_key, PassResult* s_res)
{
    SyncShared sh;
    sh.win = reinterpret_cast<float2*>(smem_raw);
    sh.metric = reinterpret_cast<float*>(sh.win + ((kSyncPass + pre_len + 1) & ~1));
    sh.chunk = reinterpret_cast<float4*>(sh.metric + kSyncPass);
    sh.memo = reinterpret_cast<float*>(sh.chunk + kSyncThreads);
    sh.red = red;
    sh.rmetric = rmetric;
    sh.s_key = s_key;
    sh.s_res = s_res;
    return sh;
}

// One pass of the frame search over candidates [4352 pass, 4352 (pass + 1)) of x
// (avail samples, limit candidates), by the whole CTA.  Mode 0: *sh.s_res takes the
// pass's earliest successful crossing (key stays INT_MAX when none); mode 1: the
// pass maximum is folded into *sh.s_res.  Ends with a barrier.
__device__ void sync_scan_pass(const float2* __restrict__ x, int avail, int limit, int pass,
                               const float2* __restrict__ preamble, const SyncParams& p, const SyncShared& sh)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int L = p.half_len, pre = p.pre_len, R = p.radius;
    const int base = pass * kSyncPass;
    const int span = min(kSyncPass + pre, avail - base);
    for (int i = tid; i < kSyncPass + pre; i += kSyncThreads) sh.win[i] = (i < span) ? x[base + i] : make_float2(0.f, 0.f);
    __syncthreads();
    // chunks holding candidates below the limit (the rest only hold -1)
    const int nchunks = min(kSyncThreads, (limit - base + kSyncChunk - 1) / kSyncChunk);
    // window sums at chunk starts, one warp per chunk
    for (int t = warp; t < nchunks; t += kSyncThreads / 32) {
        const int d0 = t * kSyncChunk;
        float pr = 0.f, pi = 0.f, e1 = 0.f, e2 = 0.f;
        for (int i = lane; i < L; i += 32) {
            const float2 a = sh.win[d0 + i], b = sh.win[d0 + i + L];
            const float2 c = cmulconj(b, a);  // conj(a) * b
            pr += c.x;
            pi += c.y;
            e1 += cnorm(a);
            e2 += cnorm(b);
        }
        pr = warp_sum(pr);
        pi = warp_sum(pi);
        e1 = warp_sum(e1);
        e2 = warp_sum(e2);
        if (lane == 0) sh.chunk[t] = make_float4(pr, pi, e1, e2);
    }
    __syncthreads();
    if (tid >= nchunks) {
        for (int c = 0; c < kSyncChunk; ++c) sh.metric[tid * kSyncChunk + c] = -1.0f;
    } else {
        float4 w = sh.chunk[tid];
        const int d0 = tid * kSyncChunk;
        for (int c = 0; c < kSyncChunk; ++c) {
            const int d = d0 + c;
            const float den = fmaxf(w.z * w.w, 1e-18f);
            sh.metric[d] = (base + d < limit) ? (w.x * w.x + w.y * w.y) / den : -1.0f;
            const float2 x0 = sh.win[d], x1 = sh.win[d + L], x2 = sh.win[d + pre];
            const float2 add = cmulconj(x2, x1), sub = cmulconj(x1, x0);
            w.x += add.x - sub.x;
            w.y += add.y - sub.y;
            w.z += cnorm(x1) - cnorm(x0);
            w.w += cnorm(x2) - cnorm(x1);
        }
    }
    __syncthreads();
    if (p.mode == 1) {
        // maximum of the pass, first occurrence (strict >)
        float bm = -1.0f;
        int bd = 0x7fffffff;
        for (int c = 0; c < kSyncChunk; ++c) {
            const int d = tid * kSyncChunk + c;
            const float m = sh.metric[d];
            if (m > bm) { bm = m; bd = d; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float om = __shfl_xor_sync(0xffffffffu, bm, o);
            const int od = __shfl_xor_sync(0xffffffffu, bd, o);
            if (om > bm || (om == bm && od < bd)) { bm = om; bd = od; }
        }
        if (lane == 0) { sh.red[warp] = bm; sh.red[8 + warp] = __int_as_float(bd); }
        __syncthreads();
        if (tid == 0) {
            for (int w = 0; w < kSyncThreads / 32; ++w) {
                const float m = sh.red[w];
                const int d = __float_as_int(sh.red[8 + w]);
                if (d == 0x7fffffff) continue;  // no valid candidate in that warp's chunks
                if (m > sh.s_res->fine || (m == sh.s_res->fine && base + d < sh.s_res->key)) {
                    sh.s_res->fine = m;
                    sh.s_res->key = base + d;
                }
            }
        }
    } else {
        // positions within +-R of a crossing of this pass: memo index i <-> sample x = base - R + i
        const int mspan = kSyncPass + 2 * R;
        {
            const int seg = (mspan + kSyncThreads - 1) / kSyncThreads;
            const int i0 = tid * seg, i1 = min(mspan, i0 + seg);
            auto crossing = [&](int y) -> int {  // memo index y holds candidate d = y - R
                const int d = y - R;
                return (d >= 0 && d < kSyncPass && sh.metric[d] >= p.threshold) ? 1 : 0;
            };
            int cnt = 0;
            if (i0 < i1)
                for (int y = i0 - R; y <= i0 + R; ++y) cnt += crossing(y);
            for (int i = i0; i < i1; ++i) {
                const int xs = base - R + i;
                sh.memo[i] = (cnt > 0 && xs >= 0 && xs <= avail - pre) ? -2.0f : -1.0f;
                cnt += crossing(i + R + 1) - crossing(i - R);
            }
        }
        __syncthreads();
        for (int i = warp; i < mspan; i += kSyncThreads / 32) {
            if (sh.memo[i] != -2.0f) continue;
            const float m = fine_metric(x, sh.win, base, kSyncPass + pre, base - R + i, preamble, pre, p.pre_energy, lane);
            if (lane == 0) sh.memo[i] = m;
        }
        __syncthreads();
        // earliest crossing of the pass whose window maximum reaches the threshold
        int first = 0x7fffffff, fstart = -1;
        float fbm = 0.0f;
        for (int c = 0; c < kSyncChunk; ++c) {
            const int d = tid * kSyncChunk + c;
            if (!(sh.metric[d] >= p.threshold)) continue;
            const int cand = base + d;
            const int lo = max(0, cand - R);
            const int hi = min(avail - pre, cand + R);
            float bm = 0.0f;
            int bd = cand;
            for (int dd = lo; dd <= hi; ++dd) {
                const float m = sh.memo[dd - base + R];
                if (m > bm) { bm = m; bd = dd; }
            }
            if (bm >= p.threshold) { first = d; fstart = bd; fbm = bm; break; }
        }
        const int wmin = __reduce_min_sync(0xffffffffu, static_cast<unsigned>(first));
        if (lane == 0) sh.s_key[warp] = wmin;
        __syncthreads();
        int bmin = 0x7fffffff;
        for (int w = 0; w < kSyncThreads / 32; ++w) bmin = min(bmin, sh.s_key[w]);
        if (bmin != 0x7fffffff && first == bmin) {
            sh.s_res->key = base + first;
            sh.s_res->start = fstart;
            sh.s_res->fine = fbm;
            sh.s_res->coarse = sh.metric[first];
                    }
    }
    __syncthreads();
}

// The record of a frame search from its resolved result `fin` (mode 1: refined
// first), with the CFO of the start found; valid in thread 0.  All threads call it.
__device__ SyncOut sync_finish(const float2* __restrict__ x, int avail, int limit, const PassResult fin,
                               const float2* __restrict__ preamble, const SyncParams& p, const SyncShared& sh)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int L = p.half_len, pre = p.pre_len, R = p.radius;

    SyncOut res{0, -1, 0.0f, 0.0f, 0.0f, -1};
    if (p.mode == 0) {
        if (fin.key != 0x7fffffff) {
            res.coarse_start = fin.key;
            res.coarse = fin.coarse >= 0.0f ? fin.coarse : 0.0f;
            res.start = fin.start;
            res.fine = fin.fine;
            res.found = (p.frame_len > 0 && res.start + p.frame_len > avail) ? 2 : 1;
        }
    } else if (fin.key >= 0 && fin.fine >= p.threshold) {
        const int cand = fin.key;
        const int lo = max(0, cand - R);
        const int hi = min(limit - 1, cand + R);
        for (int dd = lo + warp; dd <= hi; dd += kSyncThreads / 32) {
            const float m = fine_metric(x, sh.win, 0, 0, dd, preamble, pre, p.pre_energy, lane);
            if (lane == 0) sh.rmetric[dd - lo] = m;
        }
        __syncthreads();
        if (tid == 0) {
            float bm = 0.0f;
            int bd = cand;
            for (int dd = lo; dd <= hi; ++dd)
                if (sh.rmetric[dd - lo] > bm) { bm = sh.rmetric[dd - lo]; bd = dd; }
            sh.s_res->start = bd;
            sh.s_res->fine = bm;
        }
        __syncthreads();
        res.coarse_start = cand;
        res.coarse = fin.fine;
        res.fine = sh.s_res->fine;
        if (sh.s_res->fine >= p.threshold) {
            res.start = sh.s_res->start;
            res.found = 1;
        }
    }

    if (res.found == 1 || res.found == 2) {  // an incomplete frame also gets its CFO (for one-frame buffers)
        const int s0 = res.start;
        float ar = 0.f, ai = 0.f;
        for (int i = tid; i < L; i += kSyncThreads) {
            const float2 c = cmulconj(x[s0 + i + L], x[s0 + i]);  // conj(x[s0+i]) * x[s0+i+L]
            ar += c.x;
            ai += c.y;
        }
        ar = warp_sum(ar);
        ai = warp_sum(ai);
        if (lane == 0) { sh.red[16 + warp] = ar; sh.red[24 + warp] = ai; }
        __syncthreads();
        if (tid == 0) {
            float sr = 0.f, si = 0.f;
            for (int w = 0; w < kSyncThreads / 32; ++w) { sr += sh.red[16 + w]; si += sh.red[24 + w]; }
            res.cfo_hz = atan2f(si, sr) * p.sample_rate / (2.0f * 3.14159265358979323846f * static_cast<float>(L));
        }
    }
    return res;
}

// Frame search, one CTA per (pass, frame): pass q scans candidates
// [4352 q, 4352 (q + 1)).  Within a pass every threshold crossing is refined
// at once: the fine metric of each position within +-radius of any crossing is
// computed once (one warp per position), then each crossing takes the first
// maximum over its window (starting from 0, strict >) and the earliest
// crossing whose maximum reaches the threshold wins -- the outcome of the CPU
// receiver's sequential retry loop.  Mode 0 wants the earliest success, so a
// pass that starts after an earlier pass of its frame succeeded skips its
// scan (`ticket[frames + f]` holds passes - earliest successful pass, 0 for
// none).  Each pass stores its result in `pres`, and the CTA that takes the
// frame's last ticket (`ticket[f]`) takes the earliest result (mode 0) or the
// first global maximum (mode 1), refines it (mode 1), computes the CFO and
// writes the record.  `ticket` starts zeroed.
__global__ void __launch_bounds__(kSyncThreads)
sync_kernel(const float2* __restrict__ samples, long long stride, const long long* __restrict__ frame_off,
            const int* __restrict__ counts, int count, int frames, int passes, const float2* __restrict__ preamble,
            SyncParams p, PassResult* __restrict__ pres, int* __restrict__ ticket, SyncOut* __restrict__ out,
            const int* __restrict__ frames_ptr)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float red[4 * (kSyncThreads / 32)];
    __shared__ float rmetric[kMaxRefine];
    __shared__ int s_key[kSyncThreads / 32];
    __shared__ PassResult s_res;
    __shared__ int s_flag;
    const SyncShared sh = sync_shared(smem_raw, p.pre_len, red, rmetric, s_key, &s_res);

    // pass-major order: the first passes of all frames run first, so later
    // passes of a frame found early skip their scans
    const int pass = blockIdx.x / frames;
    const int f = blockIdx.x - pass * frames;
    // a grid sized for `frames` over a batch of *frames_ptr frames: the CTAs of absent frames
    // leave at once (uniform over the CTA, before any barrier)
    if (frames_ptr && f >= *frames_ptr) return;
    const int tid = threadIdx.x;
    const float2* x = samples + (frame_off ? frame_off[f] : static_cast<long long>(f) * stride);
    const int avail = counts ? counts[f] : count;
    int limit = avail - p.pre_len + 1;
    if (p.max_search > 0) limit = min(limit, p.max_search + 1);
    int* done = ticket + frames;

    if (tid == 0) {
        s_res.key = p.mode == 1 ? -1 : 0x7fffffff;
        s_res.start = -1;
        s_res.fine = -1.0f;
        s_res.coarse = 0.0f;
        s_flag = p.mode == 0 && *reinterpret_cast<volatile int*>(done + f) > passes - pass;
    }
    __syncthreads();

    const int base = pass * kSyncPass;
    if (!s_flag && base < limit) sync_scan_pass(x, avail, limit, pass, preamble, p, sh);
    __syncthreads();
    if (tid == 0 && p.mode == 0 && s_res.key != 0x7fffffff) atomicMax(done + f, passes - pass);

    // publish this pass; the frame's last pass to finish resolves it
    if (tid == 0) {
        pres[static_cast<long long>(f) * passes + pass] = s_res;
        __threadfence();
        s_flag = atomicAdd(ticket + f, 1) == passes - 1;
    }
    __syncthreads();
    if (!s_flag) return;
    __threadfence();
    if (tid == 0) {
        const PassResult* fr = pres + static_cast<long long>(f) * passes;
        PassResult best;
        best.key = __ldcg(&fr[0].key);
        best.start = __ldcg(&fr[0].start);
        best.fine = __ldcg(&fr[0].fine);
        best.coarse = __ldcg(&fr[0].coarse);
        for (int q = 1; q < passes; ++q) {
            PassResult o;
            o.key = __ldcg(&fr[q].key);
            o.start = __ldcg(&fr[q].start);
            o.fine = __ldcg(&fr[q].fine);
            o.coarse = __ldcg(&fr[q].coarse);
            if (p.mode == 1) {
                if (o.key >= 0 && (o.fine > best.fine || (o.fine == best.fine && (best.key < 0 || o.key < best.key))))
                    best = o;
            } else if (o.key < best.key) {
                best = o;
            }
        }
        s_res = best;
    }
    __syncthreads();
    const SyncOut res = sync_finish(x, avail, limit, s_res, preamble, p, sh);
    if (tid == 0) out[f] = res;
}

// Frame extraction over one window (one CTA): the receive loop's sequence of
// searches, each over [base, base + window) with the tracking or acquisition
// window, the earliest crossing found by scanning passes in order (mode 0),
// then the miss / late-peak / incomplete rules of extract_device; a found frame
// is copied into the next free pool slot and the search continues after it.
__global__ void __launch_bounds__(kSyncThreads)
ingest_extract_kernel(const float2* __restrict__ window, int n, const float2* __restrict__ preamble, SyncParams p,
                      IngestParams ip, const int* __restrict__ slots, float2* __restrict__ pool,
                      IngestRecord* __restrict__ rec, IngestState* __restrict__ state)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float red[4 * (kSyncThreads / 32)];
    __shared__ float rmetric[kMaxRefine];
    __shared__ int s_key[kSyncThreads / 32];
    __shared__ PassResult s_res;
    __shared__ SyncOut s_out;
    __shared__ IngestState s_st;
    const SyncShared sh = sync_shared(smem_raw, p.pre_len, red, rmetric, s_key, &s_res);
    const int tid = threadIdx.x;
    if (tid == 0) {
        s_st = *state;
        s_st.base = 0;
        s_st.frames = 0;
    }
    __syncthreads();
    while (s_st.frames < ip.max_frames) {
        const int base = s_st.base;
        const int available = n - base;
        if (available < p.pre_len) break;
        const int count = min(available, s_st.tracking ? ip.track_window : ip.acq_window);
        const float2* x = window + base;
        const int limit = count - p.pre_len + 1;
        if (tid == 0) {
            s_res.key = 0x7fffffff;
            s_res.start = -1;
            s_res.fine = -1.0f;
            s_res.coarse = 0.0f;
        }
        __syncthreads();
        for (int pass = 0; pass * kSyncPass < limit; ++pass) {  // the earliest success ends the search
            sync_scan_pass(x, count, limit, pass, preamble, p, sh);
            if (s_res.key != 0x7fffffff) break;
        }
        const SyncOut r = sync_finish(x, count, limit, s_res, preamble, p, sh);
        if (tid == 0) s_out = r;
        __syncthreads();
        const SyncOut res = s_out;
        const bool late = s_st.tracking && ip.late_threshold > 0.0f && res.start > ip.strict_window &&
                          res.fine < ip.late_threshold;
        int outcome = 0;  // 0 miss, 1 incomplete, 2 no pool slot, 3 found
        if (res.found == 0 || res.fine < p.threshold || late) outcome = 0;
        else if (res.start + ip.frame_len > available) outcome = 1;
        else if (s_st.frames >= ip.free_slots) outcome = 2;
        else outcome = 3;
        if (outcome == 3) {  // copy the frame into its pool slot
            float2* dst = pool + static_cast<size_t>(slots[s_st.frames]) * ip.frame_len;
            const float2* src = x + res.start;
            for (int i = tid; i < ip.frame_len; i += kSyncThreads) dst[i] = src[i];
        }
        __syncthreads();
        if (tid == 0) {
            if (outcome == 0) {
                if (s_st.tracking) {
                    ++s_st.tracking_miss;
                    s_st.tracking = 0;
                } else {
                    ++s_st.miss;
                }
            } else if (outcome == 1) {
                ++s_st.incomplete;
            } else if (outcome == 2) {
                s_st.base = base + res.start + ip.frame_len;
                ++s_st.miss;
                ++s_st.pool_exhausted;
            } else {
                IngestRecord& o = rec[s_st.frames];
                o.slot = slots[s_st.frames];
                o.start = base + res.start;
                o.peak = res.fine;
                o.cfo_hz = res.cfo_hz;
                ++s_st.found;
                s_st.skipped_samples += static_cast<unsigned long long>(res.start);
                if (static_cast<unsigned long long>(res.start) > s_st.max_start) s_st.max_start = res.start;
                s_st.tracking = 1;
                s_st.base = base + res.start + ip.frame_len;
                ++s_st.frames;
            }
        }
        __syncthreads();
        if (outcome != 3) break;
    }
    if (tid == 0) *state = s_st;
}

static long long sync_passes(long long stride, const int* counts, int count, const SyncParams& p)
{
    // passes of the longest search: frames hold at most `stride` samples
    long long span = counts ? stride : std::min<long long>(count, stride);
    long long limit = span - p.pre_len + 1;
    if (p.max_search > 0) limit = std::min<long long>(limit, p.max_search + 1);
    return std::max<long long>(1, (limit + kSyncPass - 1) / kSyncPass);
}

SyncScratchLayout sync_scratch_layout(long long stride, const int* counts, int count, int frames, const SyncParams& p)
{
    const long long passes = sync_passes(stride, counts, count, p);
    SyncScratchLayout l;
    l.ticket_offset = (static_cast<size_t>(frames) * passes * sizeof(PassResult) + 15) & ~size_t(15);
    l.ticket_bytes = static_cast<size_t>(2) * frames * sizeof(int);
    l.bytes = l.ticket_offset + l.ticket_bytes;
    return l;
}

void launch_sync(const float2* samples, long long stride, const int* counts, int count, int frames,
                 const float2* preamble, const SyncParams& p, SyncOut* out, cudaStream_t st,
                 const long long* frame_off, const int* frames_ptr, void* caller_scratch, size_t caller_scratch_bytes)
{
    if (frames <= 0) return;
    const size_t smem = static_cast<size_t>((kSyncPass + p.pre_len + 1) & ~1) * sizeof(float2) +
                        static_cast<size_t>(kSyncPass) * sizeof(float) + kSyncThreads * sizeof(float4) +
                        static_cast<size_t>(kSyncPass + 2 * kMaxRadius) * sizeof(float);
    if (smem > 200 * 1024) throw InvalidArgument("preamble too long for the sync kernel");
    if (p.radius > kMaxRadius || p.radius < 0) throw InvalidArgument("refinement radius must be 0..511");
    const long long passes = sync_passes(stride, counts, count, p);
    if (passes * frames > 0x7fffffffLL) throw InvalidArgument("sync grid too large");
    const SyncScratchLayout l = sync_scratch_layout(stride, counts, count, frames, p);
    void* scratch = caller_scratch;
    const bool own = caller_scratch == nullptr;
    if (own) {
        int device = 0;
        check_cuda(cudaGetDevice(&device), "cudaGetDevice");
        check_cuda(cudaMallocFromPoolAsync(&scratch, l.bytes, scratch_pool(device), st), "cudaMallocFromPoolAsync(sync)");
    } else if (caller_scratch_bytes < l.bytes) {
        throw InvalidArgument("sync scratch smaller than the grid needs");
    }
    PassResult* pres = static_cast<PassResult*>(scratch);
    int* ticket = reinterpret_cast<int*>(static_cast<unsigned char*>(scratch) + l.ticket_offset);
    // caller scratch: the caller has zeroed the tickets in stream order before this launch
    cudaError_t err = own ? cudaMemsetAsync(ticket, 0, l.ticket_bytes, st) : cudaSuccess;
    if (err == cudaSuccess)
        err = grant_dynamic_smem(reinterpret_cast<const void*>(sync_kernel), smem);
    if (err == cudaSuccess) {
        sync_kernel<<<static_cast<unsigned>(passes * frames), kSyncThreads, smem, st>>>(
            samples, stride, frame_off, counts, count, frames, static_cast<int>(passes), preamble, p, pres, ticket, out,
            frames_ptr);
        err = cudaGetLastError();
    }
    const cudaError_t ferr = own ? cudaFreeAsync(scratch, st) : cudaSuccess;
    check_cuda(err, "sync_kernel launch");
    check_cuda(ferr, "cudaFreeAsync(sync)");
}

// ---------------------------------------------------------------------------
// demodulator
// ---------------------------------------------------------------------------

namespace {

constexpr int kDemodThreads = 256;

// Twiddle entries the FFT of nfft points reads (indices below 3 nfft / 4), rounded to an
// even count so the buffers after them stay 16-byte aligned.
__host__ __device__ constexpr int demod_twiddles(int nfft) { return ((3 * nfft / 4) + 1) & ~1; }

// Stockham autosort FFT of `nfft` points held in buf[0] (natural order in and
// out); returns the buffer that holds the result.
// `tw` in shared memory (kSharedTw) or read through the read-only cache.
template <bool kSharedTw = false>
__device__ __forceinline__ float2 twiddle_at(const float2* __restrict__ tw, int i)
{
    if constexpr (kSharedTw) return tw[i];
    else return __ldg(tw + i);
}

template <bool kSharedTw = false>
__device__ float2* fft_stockham(float2* a, float2* b, int nfft, const float2* __restrict__ tw)
{
    int ns = 1;
    const int q = nfft >> 2;
    while (ns * 4 <= nfft) {
        for (int j = threadIdx.x; j < q; j += blockDim.x) {
            const int k = j & (ns - 1);
            const int step = nfft / (4 * ns);
            float2 a0 = a[j], a1 = a[j + q], a2 = a[j + 2 * q], a3 = a[j + 3 * q];
            if (ns > 1) {
                a1 = cmul(a1, twiddle_at<kSharedTw>(tw, k * step));
                a2 = cmul(a2, twiddle_at<kSharedTw>(tw, 2 * k * step));
                a3 = cmul(a3, twiddle_at<kSharedTw>(tw, 3 * k * step));
            }
            const float2 b0 = make_float2(a0.x + a2.x, a0.y + a2.y);
            const float2 b1 = make_float2(a0.x - a2.x, a0.y - a2.y);
            const float2 b2 = make_float2(a1.x + a3.x, a1.y + a3.y);
            const float2 b3 = make_float2(a1.y - a3.y, a3.x - a1.x);  // -i (a1 - a3)
            const int o = (j / ns) * ns * 4 + k;
            b[o] = make_float2(b0.x + b2.x, b0.y + b2.y);
            b[o + ns] = make_float2(b1.x + b3.x, b1.y + b3.y);
            b[o + 2 * ns] = make_float2(b0.x - b2.x, b0.y - b2.y);
            b[o + 3 * ns] = make_float2(b1.x - b3.x, b1.y - b3.y);
        }
        __syncthreads();
        float2* t = a;
        a = b;
        b = t;
        ns *= 4;
    }
    if (ns < nfft) {  // one radix-2 stage
        const int h = nfft >> 1;
        for (int j = threadIdx.x; j < h; j += blockDim.x) {
            const int k = j & (ns - 1);
            const float2 a0 = a[j];
            const float2 a1 = cmul(a[j + h], twiddle_at<kSharedTw>(tw, k * (nfft / (2 * ns))));
            const int o = (j / ns) * ns * 2 + k;
            b[o] = make_float2(a0.x + a1.x, a0.y + a1.y);
            b[o + ns] = make_float2(a0.x - a1.x, a0.y - a1.y);
        }
        __syncthreads();
        a = b;
    }
    return a;
}

// ---- bulk-async staging of a symbol's samples (cp.async.bulk + mbarrier) ----

__device__ unsigned int g_demod_wait_timeouts = 0;  // waits that hit their iteration limit (never expected)
constexpr int kMaxWaitSpins = 1 << 22;

__device__ __forceinline__ unsigned smem_addr(const void* p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity)
{
    unsigned ok = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the barrier's phase `parity` with an iteration limit; on the limit the
// timeout is counted, one more bounded wait lets an in-flight copy land, and false
// is returned (the caller skips the symbol's data).
__device__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity)
{
    for (int i = 0; i < kMaxWaitSpins; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    if (threadIdx.x == 0) atomicAdd(&g_demod_wait_timeouts, 1u);
    for (int i = 0; i < kMaxWaitSpins; ++i)
        if (mbar_try_wait(bar, parity)) break;
    return false;
}

// Where symbol `sym` of the frame at x lies, and how its samples are staged: the
// 16-byte-aligned middle [s, s + len) by one bulk copy into stage[0 .. len), the
// samples before s and from s + len on (at most one each: the rows are 8-byte
// complex samples) by plain loads when they are used.
struct SymbolStage {
    const float2* src;  // first sample of the symbol (CP stripped)
    int s, len;
};

__device__ __forceinline__ SymbolStage symbol_stage(const DemodView& v, const float2* x, int sym)
{
    SymbolStage g;
    g.src = x + v.pre_len + sym * (v.nfft + v.cp) + v.cp;
    g.s = (reinterpret_cast<uintptr_t>(g.src) & 15u) ? 1 : 0;
    g.len = v.nfft - 2 * g.s;  // nfft is even: len * 8 bytes is a multiple of 16
    return g;
}

// Thread 0: arms `bar` for the symbol's bytes and starts its bulk copy into `stage`.
__device__ __forceinline__ void stage_symbol(const SymbolStage& g, float2* stage, uint64_t* bar)
{
    const unsigned bytes = static_cast<unsigned>(g.len) * 8u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier reads of `stage` come first
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(stage)),
                 "l"(g.src + g.s), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// CFO derotation and CP strip: work[i] = sample i of the symbol times
// exp(-j 2 pi cfo n / fs), n its index from the frame start; the samples come from
// the staged copy, the edge samples (and every sample if the copy did not land)
// from global memory.
__device__ __forceinline__ void derotate_symbol(const DemodView& v, const SymbolStage& g, const float2* stage,
                                                float2* work, float cfo_norm, int sym, bool staged)
{
    const int off = v.pre_len + sym * (v.nfft + v.cp) + v.cp;
    for (int i = threadIdx.x; i < v.nfft; i += blockDim.x) {
        const float2 smp = (!staged || i < g.s || i >= g.s + g.len) ? g.src[i] : stage[i - g.s];
        float sn, cs;
        // exp(-j 2 pi cfo n / fs) with cfo_norm = cfo / fs
        sincospif(-2.0f * cfo_norm * static_cast<float>(off + i), &sn, &cs);
        work[i] = cmul(smp, make_float2(cs, sn));
    }
    __syncthreads();
}

__device__ __forceinline__ float sq_dist(float x, float c)
{
    const float d = __fsub_rn(x, c);
    return __fmul_rn(d, d);
}

}  // namespace

__global__ void __launch_bounds__(kDemodThreads)
demod_kernel(DemodView v, const float2* __restrict__ samples, long long stride, const SyncOut* __restrict__ sync,
             float* __restrict__ llr, long long llr_stride, int symbols_per_cta, const long long* __restrict__ frame_off,
             const long long* __restrict__ llr_off, const int* __restrict__ frames_ptr)
{
    // a grid sized for more frames than the batch holds: the CTAs of absent frames leave at once
    if (frames_ptr && static_cast<int>(blockIdx.x) >= *frames_ptr) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* work = reinterpret_cast<float2*>(smem_raw);  // derotated symbol, FFT buffer
    // stage(b) = work + (1 + b) * nfft: staged raw symbols (two buffers), FFT buffer after use
    auto stage = [&](int b) { return work + static_cast<size_t>(1 + b) * v.nfft; };
    float2* tw = work + 3 * v.nfft;                       // twiddles 0 .. 3 nfft / 4 (all the FFT reads)
    float2* hp = tw + demod_twiddles(v.nfft);             // [max_pilots_per_cta][active_sc]
    __shared__ __align__(8) uint64_t s_bar[2];

    const int f = blockIdx.x;
    const int ds0 = blockIdx.y * symbols_per_cta;
    const int ds1 = min(v.num_data, ds0 + symbols_per_cta);
    if (ds0 >= ds1) return;
    int start = 0;
    float cfo = 0.0f;
    if (sync) {
        const SyncOut so = sync[f];
        if (so.found != 1) {
            // no frame: zero LLRs (the caller sees found != 1 in the sync result)
            float* dst = llr + (llr_off ? llr_off[f] : static_cast<long long>(f) * llr_stride);
            const int hi = min(ds1 * v.active_sc * v.bits_per_symbol, v.kept_bits);
            for (int i = ds0 * v.active_sc * v.bits_per_symbol + threadIdx.x; i < hi; i += blockDim.x) dst[i] = 0.0f;
            return;
        }
        start = so.start;
        cfo = so.cfo_hz;
    }
    const float2* x = samples + (frame_off ? frame_off[f] : static_cast<long long>(f) * stride) + start;
    const float cfo_norm = cfo / v.sample_rate;

    // pilots referenced by this CTA's data symbols
    int pmin = 0x7fffffff, pmax = -1;
    for (int d = ds0; d < ds1; ++d) {
        pmin = min(pmin, min(v.interp_p0[d], v.interp_p1[d]));
        pmax = max(pmax, max(v.interp_p0[d], v.interp_p1[d]));
    }
    const int npil = v.use_pilot_est ? min(pmax - pmin + 1, v.max_pilots_per_cta) : 0;
    const int nsym = npil + (ds1 - ds0);
    // the CTA's symbols in processing order: its pilots, then its data symbols
    auto sym_at = [&](int i) { return i < npil ? v.pilot_symbols[pmin + i] : v.data_symbols[ds0 + i - npil]; };

    // Symbol i+1's samples are copied into stage[(i+1)&1] by the bulk-copy engine while
    // symbol i is transformed; each buffer's barrier completes once per copy.
    if (threadIdx.x == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = threadIdx.x; i < demod_twiddles(v.nfft); i += blockDim.x) tw[i] = __ldg(v.twiddle + i);
    // the constellation's axis levels (at most 8: 64-QAM) in registers
    float lvl[8];
#pragma unroll
    for (int g = 0; g < 8; ++g) lvl[g] = (v.bits_per_symbol >= 2 && g < (1 << (v.bits_per_symbol >> 1))) ? __ldg(v.axis_levels + g) : 0.0f;
    __syncthreads();
    if (threadIdx.x == 0) stage_symbol(symbol_stage(v, x, sym_at(0)), stage(0), &s_bar[0]);
    unsigned phase = 0u;  // bit b: parity of buffer b's next completion

    const int bps = v.bits_per_symbol;
    const int abits = bps >> 1;
    const int levels = 1 << abits;
    float* out = llr + (llr_off ? llr_off[f] : static_cast<long long>(f) * llr_stride);
    for (int i = 0; i < nsym; ++i) {
        const int b = i & 1;
        const int sym = sym_at(i);
        if (threadIdx.x == 0 && i + 1 < nsym)
            stage_symbol(symbol_stage(v, x, sym_at(i + 1)), stage(b ^ 1), &s_bar[b ^ 1]);
        const SymbolStage g = symbol_stage(v, x, sym);
        const bool staged = mbar_wait_bounded(b ? &s_bar[1] : &s_bar[0], (phase >> b) & 1u);
        phase ^= 1u << b;
        derotate_symbol(v, g, stage(b), work, cfo_norm, sym, staged);
        const float2* Y = fft_stockham<true>(work, stage(b), v.nfft, tw);
        if (i < npil) {  // LS estimate at the pilot symbol
            const int p = pmin + i;
            for (int sc = threadIdx.x; sc < v.active_sc; sc += blockDim.x) {
                const float2 y = Y[v.used_bins[sc]];
                const float2 pil = v.pilot_grid[static_cast<size_t>(p) * v.active_sc + sc];
                const float den = fmaxf(cnorm(pil), 1e-9f);
                const float2 t = cmulconj(y, pil);
                hp[i * v.active_sc + sc] = make_float2(__fdiv_rn(t.x, den), __fdiv_rn(t.y, den));
            }
            __syncthreads();
            continue;
        }
        const int d = ds0 + i - npil;
        const int q0 = v.interp_p0[d] - pmin, q1 = v.interp_p1[d] - pmin;
        const float al = v.interp_alpha[d];
        const float w0 = __fsub_rn(1.0f, al);
        const int sc_end = min(v.active_sc, v.kept_bits / bps - d * v.active_sc);  // REs of whole codewords
        for (int sc = threadIdx.x; sc < sc_end; sc += blockDim.x) {
            const float2 y = Y[v.used_bins[sc]];
            float2 h = make_float2(1.0f, 0.0f);
            if (v.use_pilot_est) {
                const float2 h0 = hp[q0 * v.active_sc + sc], h1 = hp[q1 * v.active_sc + sc];
                h = make_float2(__fadd_rn(__fmul_rn(h0.x, w0), __fmul_rn(h1.x, al)),
                                __fadd_rn(__fmul_rn(h0.y, w0), __fmul_rn(h1.y, al)));
            }
            const float h2 = fmaxf(cnorm(h), 1e-9f);
            const float2 t = cmulconj(y, h);
            // eq = y conj(h) / (|h|^2 + N0) and LLR = (d1 - d0) / sigma^2 as products with the two
            // reciprocals (as the reference's GPU equaliser scales by 1 / (|h|^2 + N0))
            const float inv_den = __frcp_rn(__fadd_rn(h2, v.noise_var));
            const float ex = __fmul_rn(t.x, inv_den), ey = __fmul_rn(t.y, inv_den);
            const float inv_sig = __frcp_rn(fmaxf(__fdiv_rn(v.noise_var, h2), 1e-8f));
            float* o = out + (static_cast<long long>(d) * v.active_sc + sc) * bps;
            if (bps == 1) {
                const float dy = __fmul_rn(ey, ey);
                const float d0 = __fadd_rn(sq_dist(ex, 1.0f), dy), d1 = __fadd_rn(sq_dist(ex, -1.0f), dy);
                o[0] = __fmul_rn(__fsub_rn(d1, d0), inv_sig);
                continue;
            }
            // per-axis squared distances and minima
            float mi_all = FLT_MAX, mq_all = FLT_MAX;
            float mi0[3], mi1[3], mq0[3], mq1[3];
#pragma unroll
            for (int bb = 0; bb < 3; ++bb) { mi0[bb] = mi1[bb] = mq0[bb] = mq1[bb] = INFINITY; }
#pragma unroll
            for (int gq = 0; gq < 8; ++gq) {
                if (gq >= levels) break;
                const float lv = lvl[gq];
                const float di = sq_dist(ex, lv), dq = sq_dist(ey, lv);
                mi_all = fminf(mi_all, di);
                mq_all = fminf(mq_all, dq);
#pragma unroll
                for (int bb = 0; bb < 3; ++bb) {
                    if (bb < abits) {
                        const int bit = (gq >> (abits - 1 - bb)) & 1;
                        if (bit) { mi1[bb] = fminf(mi1[bb], di); mq1[bb] = fminf(mq1[bb], dq); }
                        else { mi0[bb] = fminf(mi0[bb], di); mq0[bb] = fminf(mq0[bb], dq); }
                    }
                }
            }
            float vals[6];
#pragma unroll
            for (int bb = 0; bb < 3; ++bb) {
                if (bb < abits) {
                    vals[bb] = __fmul_rn(__fsub_rn(__fadd_rn(mi1[bb], mq_all), __fadd_rn(mi0[bb], mq_all)), inv_sig);
                    vals[abits + bb] =
                        __fmul_rn(__fsub_rn(__fadd_rn(mi_all, mq1[bb]), __fadd_rn(mi_all, mq0[bb])), inv_sig);
                }
            }
            if (bps == 4) {
                *reinterpret_cast<float4*>(o) = make_float4(vals[0], vals[1], vals[2], vals[3]);
            } else if (bps == 2) {
                *reinterpret_cast<float2*>(o) = make_float2(vals[0], vals[1]);
            } else {
                for (int bb = 0; bb < bps; ++bb) o[bb] = vals[bb];
            }
        }
        __syncthreads();
    }
}

unsigned demod_wait_timeouts()
{
    unsigned v = 0;
    check_cuda(cudaMemcpyFromSymbol(&v, g_demod_wait_timeouts, sizeof v), "read the demodulator's wait counter");
    return v;
}

void launch_demod(const DemodView& v, const float2* samples, long long stride, const SyncOut* sync, int frames,
                  float* llr, long long llr_stride, cudaStream_t st, int symbols_per_cta, const long long* frame_off,
                  const long long* llr_off, const int* frames_ptr)
{
    if (frames <= 0 || v.num_data <= 0) return;
    if (v.nfft < 4 || (v.nfft & (v.nfft - 1))) throw InvalidArgument("nfft must be a power of two >= 4");
    if (v.bits_per_symbol != 1 && v.bits_per_symbol != 2 && v.bits_per_symbol != 4 && v.bits_per_symbol != 6)
        throw InvalidArgument("bits_per_symbol must be 1, 2, 4 or 6");
    if (v.kept_bits <= 0 || v.kept_bits > v.num_data * v.active_sc * v.bits_per_symbol || v.kept_bits % v.bits_per_symbol)
        throw InvalidArgument("kept LLRs must be a positive multiple of bits_per_symbol within the frame");
    // the owner of the view sized max_pilots_per_cta for exactly this grouping of data symbols
    const int spc = symbols_per_cta;
    if (spc <= 0 || spc > v.num_data) throw InvalidArgument("symbols_per_cta must be in 1..num_data");
    if (v.max_pilots_per_cta < 0 || v.max_pilots_per_cta > kDemodMaxPilots)
        throw InvalidArgument("a demodulator CTA can hold at most 4 pilot symbols");
    const size_t smem = (3 * static_cast<size_t>(v.nfft) + demod_twiddles(v.nfft) +
                         static_cast<size_t>(v.max_pilots_per_cta) * v.active_sc) *
                        sizeof(float2);
    if (smem > 227 * 1024) throw InvalidArgument("nfft and active_sc exceed the demodulator's shared memory");
    check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(demod_kernel), smem), "cudaFuncSetAttribute(demod)");
    const dim3 grid(frames, (v.num_data + spc - 1) / spc);
    demod_kernel<<<grid, kDemodThreads, smem, st>>>(v, samples, stride, sync, llr, llr_stride, spc, frame_off,
                                                    llr_off, frames_ptr);
    check_cuda(cudaGetLastError(), "demod_kernel launch");
}

// ---------------------------------------------------------------------------
// transmitter
// ---------------------------------------------------------------------------

namespace {

constexpr int kTxThreads = 256;
constexpr int kEncWarps = 8;

// Gray square QAM, bits MSB-first per axis (gpu_ofdm_pipeline.cu:84-109).
__device__ __forceinline__ float2 qam_from_bits(const uint8_t* bits, int bps)
{
    if (bps == 1) return make_float2(bits[0] ? -1.0f : 1.0f, 0.0f);
    if (bps == 2) {
        constexpr float s = 0.7071067811865475f;
        return make_float2(bits[0] ? -s : s, bits[1] ? -s : s);
    }
    const int ab = bps / 2, levels = 1 << ab;
    int gi = 0, gq = 0;
    for (int i = 0; i < ab; ++i) {
        gi = (gi << 1) | (bits[i] != 0);
        gq = (gq << 1) | (bits[ab + i] != 0);
    }
    int bi = 0, bq = 0;  // Gray -> binary
    for (; gi; gi >>= 1) bi ^= gi;
    for (; gq; gq >>= 1) bq ^= gq;
    const float scale = (bps == 4) ? 0.3162277660168379f : 0.1543033499620919f;
    return make_float2(__fmul_rn(static_cast<float>((levels - 1) - 2 * bi), scale),
                       __fmul_rn(static_cast<float>((levels - 1) - 2 * bq), scale));
}

// Counter-based normal deviates for the frequency-domain noise: a 32-bit
// integer hash (xor-shift / multiply, "lowbias32") of seed ^ (index * golden
// ratio) gives a uniform in (0, 1], and Box-Muller turns two of them into a
// normal deviate (gpu_ofdm_pipeline.cu:259-280).
__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ float uniform_open0(uint32_t seed, uint32_t idx)
{
    const uint32_t h = hash32(seed ^ (idx * 0x9e3779b9u));
    return __fmul_rn(__fadd_rn(__uint2float_rn(h), 1.0f), 2.3283064365386963e-10f);
}

__device__ __forceinline__ float normal_dev(uint32_t seed, uint32_t idx)
{
    const float u1 = fmaxf(uniform_open0(seed, idx * 2u), 1.0e-7f);
    const float u2 = uniform_open0(seed, idx * 2u + 1u);
    return __fmul_rn(sqrtf(__fmul_rn(-2.0f, logf(u1))), cosf(__fmul_rn(__fmul_rn(2.0f, 3.14159265358979323846f), u2)));
}

// four bits -> four bytes (0/1)
__device__ __forceinline__ uint32_t spread4(uint32_t x)
{
    return (x & 1u) | ((x & 2u) << 7) | ((x & 4u) << 14) | ((x & 8u) << 21);
}

}  // namespace

// c = u G over GF(2): one warp per codeword, 4 words of the codeword per lane
// per pass.  With the byte tables each 8 information bits select one
// precomputed XOR of their 8 generator rows; otherwise each set bit selects
// its bit-packed row.
__global__ void __launch_bounds__(kEncWarps * 32)
tx_encode_generator_kernel(TxView v, const uint8_t* __restrict__ info, uint8_t* __restrict__ coded, int count)
{
    const int lane = threadIdx.x & 31;
    const int n = v.code_n, k = v.code_k, gw = v.gen_stride;
    for (int cw = blockIdx.x * kEncWarps + (threadIdx.x >> 5); cw < count; cw += gridDim.x * kEncWarps) {
        const uint8_t* u = info + static_cast<size_t>(cw) * k;
        uint8_t* c = coded + static_cast<size_t>(cw) * n;
        for (int w0 = 0; w0 < (n + 31) / 32; w0 += 128) {
            uint32_t acc[4] = {0u, 0u, 0u, 0u};
            for (int i0 = 0; i0 < k; i0 += 32) {
                unsigned bits = __ballot_sync(0xffffffffu, i0 + lane < k && (u[i0 + lane] & 1u));
                if (v.gen_tab) {  // one table entry per byte of information bits: independent loads
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int g = (i0 >> 3) + q;
                        if (g * 8 >= k) break;
                        const uint32_t* e = v.gen_tab + (static_cast<size_t>(g) * 256 + ((bits >> (8 * q)) & 255u)) * gw;
#pragma unroll
                        for (int r = 0; r < 4; ++r) {
                            const int w = w0 + r * 32 + lane;
                            if (w < gw) acc[r] ^= __ldg(e + w);
                        }
                    }
                    continue;
                }
                while (bits) {
                    const int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    const uint32_t* row = v.gen_words + static_cast<size_t>(i0 + b) * gw;
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        const int w = w0 + r * 32 + lane;
                        if (w < gw) acc[r] ^= __ldg(row + w);
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int w = w0 + r * 32 + lane;
                if (w * 32 >= n) continue;
                if (w * 32 + 32 <= n && (n & 3) == 0) {  // 32 bytes as 8 words
                    uint32_t* dst = reinterpret_cast<uint32_t*>(c + w * 32);
#pragma unroll
                    for (int q = 0; q < 8; ++q) dst[q] = spread4((acc[r] >> (4 * q)) & 15u);
                } else {
                    for (int b = 0; b < 32 && w * 32 + b < n; ++b) c[w * 32 + b] = static_cast<uint8_t>((acc[r] >> b) & 1u);
                }
            }
        }
    }
}

// Systematic + accumulator encoder (gpu_ofdm_pipeline.cu:152-214): c[i] = u[i]
// for i < k, then parity r = sum of u over row r's information columns, XOR the
// previous parity: a prefix XOR over the rows, 32 rows per ballot.
__global__ void __launch_bounds__(kEncWarps * 32)
tx_encode_accumulator_kernel(TxView v, const uint8_t* __restrict__ info, uint8_t* __restrict__ coded, int count)
{
    const int lane = threadIdx.x & 31;
    const int n = v.code_n, k = v.code_k, m = n - k;
    for (int cw = blockIdx.x * kEncWarps + (threadIdx.x >> 5); cw < count; cw += gridDim.x * kEncWarps) {
        const uint8_t* u = info + static_cast<size_t>(cw) * k;
        uint8_t* c = coded + static_cast<size_t>(cw) * n;
        for (int i = lane; i < k; i += 32) c[i] = u[i] & 1u;
        unsigned carry = 0u;
        for (int r0 = 0; r0 < m; r0 += 32) {
            const int r = r0 + lane;
            unsigned s = 0u;
            if (r < m)
                for (int q = v.acc_offsets[r]; q < v.acc_offsets[r + 1]; ++q) s ^= u[v.acc_cols[q]] & 1u;
            unsigned y = __ballot_sync(0xffffffffu, s != 0u);
            y ^= y << 1;
            y ^= y << 2;
            y ^= y << 4;
            y ^= y << 8;
            y ^= y << 16;
            if (r < m) c[k + r] = static_cast<uint8_t>(((y >> lane) & 1u) ^ carry);
            carry ^= (y >> 31) & 1u;
        }
    }
}

// One CTA per (OFDM symbol, frame); blockIdx.x == num_symbols writes the preamble.
// The symbol's grid row is built in shared memory (gpu_ofdm_pipeline.cu:216-257,
// 282-314), inverse-transformed as conj(FFT(conj(X))) (unnormalised, as cuFFT's
// inverse) and written with its cyclic prefix, scaled by amplitude / nfft
// (gpu_ofdm_pipeline.cu:316-342).
__global__ void __launch_bounds__(kTxThreads)
tx_symbol_kernel(TxView v, const uint8_t* __restrict__ coded, float2* __restrict__ out, float noise_var,
                 unsigned long long noise_seed)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf0 = reinterpret_cast<float2*>(smem_raw);
    float2* buf1 = buf0 + v.nfft;
    const int sym = blockIdx.x, f = blockIdx.y;
    float2* frame = out + static_cast<size_t>(f) * v.frame_samples;
    if (sym == v.num_symbols) {
        for (int i = threadIdx.x; i < v.pre_len; i += blockDim.x) {
            const float2 p = v.preamble[i];
            frame[i] = make_float2(__fmul_rn(p.x, v.amplitude), __fmul_rn(p.y, v.amplitude));
        }
        return;
    }
    for (int i = threadIdx.x; i < v.nfft; i += blockDim.x) buf0[i] = make_float2(0.0f, 0.0f);
    __syncthreads();
    const int pidx = v.pilot_of_symbol[sym], didx = v.data_of_symbol[sym];
    const int coded_bits = v.blocks * v.code_n;
    const uint8_t* bits = coded + static_cast<size_t>(f) * coded_bits;
    const unsigned long long fs = noise_seed + static_cast<unsigned long long>(f);
    const uint32_t seed = static_cast<uint32_t>(fs ^ (fs >> 32));
    const float sigma = sqrtf(__fmul_rn(fmaxf(noise_var, 0.0f), 0.5f));
    uint8_t* sbits = reinterpret_cast<uint8_t*>(buf1);  // the symbol's coded bits (buf1 is free until the FFT)
    if (didx >= 0 && pidx < 0) {
        const int b0 = didx * v.active_sc * v.bits_per_symbol;
        for (int i = threadIdx.x; i < v.active_sc * v.bits_per_symbol; i += blockDim.x)
            sbits[i] = b0 + i < coded_bits ? bits[b0 + i] : 0;  // bits past the coded bits are filler zeros
        __syncthreads();
    }
    for (int sc = threadIdx.x; sc < v.active_sc; sc += blockDim.x) {
        const int re = sym * v.active_sc + sc;
        float2 value = make_float2(0.0f, 0.0f);
        if (pidx >= 0) {
            value = v.pilot_grid[static_cast<size_t>(pidx) * v.active_sc + sc];
        } else if (didx >= 0) {
            value = qam_from_bits(sbits + sc * v.bits_per_symbol, v.bits_per_symbol);
        }
        if (v.precomp_h) {
            const float2 h = v.precomp_h[re];
            const float s = __fdiv_rn(1.0f, fmaxf(cnorm(h), 1.0e-10f));
            value = cmul(value, make_float2(__fmul_rn(h.x, s), __fmul_rn(-h.y, s)));
        }
        if (v.actual_h) value = cmul(value, v.actual_h[re]);
        if (noise_var > 0.0f && didx >= 0)
            value = make_float2(__fadd_rn(value.x, __fmul_rn(sigma, normal_dev(seed, static_cast<uint32_t>(re)))),
                                __fadd_rn(value.y, __fmul_rn(sigma, normal_dev(seed ^ 0xa5a5a5a5u, static_cast<uint32_t>(re)))));
        buf0[v.used_bins[sc]] = make_float2(value.x, -value.y);  // conjugated for the inverse transform
    }
    __syncthreads();  // the grid row is complete and the staged bits are read
    const float2* Y = fft_stockham(buf0, buf1, v.nfft, v.twiddle);
    const float scale = v.amplitude / static_cast<float>(v.nfft);
    const int sym_len = v.nfft + v.cp;
    float2* dst = frame + v.pre_len + static_cast<size_t>(sym) * sym_len;
    for (int pos = threadIdx.x; pos < sym_len; pos += blockDim.x) {
        const float2 y = Y[pos < v.cp ? v.nfft - v.cp + pos : pos - v.cp];
        dst[pos] = make_float2(__fmul_rn(y.x, scale), __fmul_rn(-y.y, scale));
    }
}

void launch_tx(const TxView& v, const uint8_t* info_bits, int frames, float2* frames_out, float noise_var,
               unsigned long long noise_seed, cudaStream_t st)
{
    if (frames <= 0) return;
    const size_t smem = 2 * static_cast<size_t>(v.nfft) * sizeof(float2);
    if (smem > 200 * 1024) throw InvalidArgument("nfft too large for the TX kernel");
    const int codewords = frames * v.blocks;
    int device = 0;
    check_cuda(cudaGetDevice(&device), "cudaGetDevice");
    void* coded = nullptr;
    check_cuda(cudaMallocFromPoolAsync(&coded, static_cast<size_t>(codewords) * v.code_n, scratch_pool(device), st),
               "cudaMallocFromPoolAsync(tx)");
    uint8_t* cb = static_cast<uint8_t*>(coded);
    const int ctas = std::max(1, std::min((codewords + kEncWarps - 1) / kEncWarps, 8 * device_sm_count()));
    if (v.acc_offsets)
        tx_encode_accumulator_kernel<<<ctas, kEncWarps * 32, 0, st>>>(v, info_bits, cb, codewords);
    else
        tx_encode_generator_kernel<<<ctas, kEncWarps * 32, 0, st>>>(v, info_bits, cb, codewords);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess)
        err = grant_dynamic_smem(reinterpret_cast<const void*>(tx_symbol_kernel), smem);
    if (err == cudaSuccess) {
        tx_symbol_kernel<<<dim3(v.num_symbols + 1, frames), kTxThreads, smem, st>>>(v, cb, frames_out, noise_var,
                                                                                    noise_seed);
        err = cudaGetLastError();
    }
    const cudaError_t ferr = cudaFreeAsync(coded, st);
    check_cuda(err, "tx launch");
    check_cuda(ferr, "cudaFreeAsync(tx)");
}

void launch_ingest_extract(const float2* window, int n, const float2* preamble, const SyncParams& sp,
                           const IngestParams& ip, const int* slots, float2* pool, IngestRecord* rec,
                           IngestState* state, cudaStream_t st)
{
    const size_t smem = static_cast<size_t>((kSyncPass + sp.pre_len + 1) & ~1) * sizeof(float2) +
                        static_cast<size_t>(kSyncPass) * sizeof(float) + kSyncThreads * sizeof(float4) +
                        static_cast<size_t>(kSyncPass + 2 * kMaxRadius) * sizeof(float);
    if (smem > 200 * 1024) throw InvalidArgument("preamble too long for the sync kernel");
    if (sp.radius > kMaxRadius || sp.radius < 0) throw InvalidArgument("refinement radius must be 0..511");
    check_cuda(grant_dynamic_smem(reinterpret_cast<const void*>(ingest_extract_kernel), smem),
               "cudaFuncSetAttribute(ingest)");
    ingest_extract_kernel<<<1, kSyncThreads, smem, st>>>(window, n, preamble, sp, ip, slots, pool, rec, state);
    check_cuda(cudaGetLastError(), "ingest_extract_kernel launch");
}

}  // namespace sicc
