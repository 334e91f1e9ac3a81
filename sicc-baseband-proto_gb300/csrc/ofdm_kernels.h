// OFDM receive kernels: Schmidl-Cox timing/CFO sync and the fused demodulator.
#pragma once

#include "sicc_common.h"

namespace sicc {

// Result of one frame search; mirrors the reference's DeviceSyncResult
// (gpu_ofdm_pipeline.cu:398-404) plus the fields of the CPU SyncResult
// (uhd_ldpc_ofdm_link.cpp:350-357).
struct SyncOut {
    int found;       // 1 found, 2 incomplete frame, 0 not found
    int start;       // refined start sample (0-based)
    float coarse;    // Schmidl-Cox metric at the coarse candidate
    float fine;      // full-preamble correlation metric at the refined start
    float cfo_hz;
    int coarse_start;
};

struct SyncParams {
    int half_len;         // L
    int pre_len;          // 2L
    int radius;           // refinement radius (samples)
    float threshold;
    float sample_rate;
    int mode;             // 0: earliest crossing (find_frame_vector_earliest), 1: global maximum (find_frame)
    int max_search;       // > 0 limits the candidates to [0, max_search]
    int frame_len;        // > 0: report "incomplete" when the refined frame runs past the buffer
    float pre_energy;     // sum |preamble|^2
};

// One CTA per frame and pass of 4352 candidates, with stream-ordered scratch.  samples: frame f starts at samples + f*stride (or
// samples + frame_off[f], device offsets in complex samples) and holds counts[f] (or `count` when counts
// is null) samples, at most `stride`.
// With frames_ptr (device int) the grid is sized for `frames` and only the first
// *frames_ptr frames are searched.  With caller_scratch (at least
// sync_scratch_layout(...).bytes, its tickets zeroed in stream order before the
// launch) nothing is allocated; otherwise the scratch comes from a stream-ordered pool.
void launch_sync(const float2* samples, long long stride, const int* counts, int count, int frames,
                 const float2* preamble, const SyncParams& p, SyncOut* out, cudaStream_t st,
                 const long long* frame_off = nullptr, const int* frames_ptr = nullptr, void* caller_scratch = nullptr,
                 size_t caller_scratch_bytes = 0);

struct SyncScratchLayout {
    size_t bytes;          // the whole scratch
    size_t ticket_offset;  // the tickets (2 ints per frame), which start at zero
    size_t ticket_bytes;
};
SyncScratchLayout sync_scratch_layout(long long stride, const int* counts, int count, int frames, const SyncParams& p);

// Static demodulation tables resident on the device.
struct DemodView {
    int nfft, cp, num_symbols, active_sc, bits_per_symbol, pre_len;
    int num_pilots, num_data;
    float sample_rate;
    float noise_var;
    int use_pilot_est;
    int kept_bits;             // LLRs written per frame: the first kept_bits coded bits (whole codewords)
    const int* used_bins;      // [active_sc] natural FFT bin of each active subcarrier
    const int* pilot_symbols;  // [num_pilots]
    const int* data_symbols;   // [num_data]
    const int* interp_p0;      // [num_data]
    const int* interp_p1;      // [num_data]
    const float* interp_alpha; // [num_data]
    const float2* pilot_grid;  // [num_pilots][active_sc]
    const float2* twiddle;     // [nfft]: exp(-2 pi i j / nfft)
    const float* axis_levels;  // [2^(bps/2)] constellation amplitude by Gray axis index (bps >= 2)
    int max_pilots_per_cta;    // pilot symbols one CTA's data symbols refer to, at most kDemodMaxPilots
};

constexpr int kDemodMaxPilots = 4;

// Fused demodulator: CFO derotation + CP strip + FFT + LS pilot estimate +
// interpolation + MMSE equalisation + max-log LLR.  Frame f's samples start at
// samples + f*stride + sync[f].start (sync may be null: start 0, cfo 0 unless
// `cfo_override` is used); LLRs go to llr + f*llr_stride.  With frame_off / llr_off (device offsets in
// complex samples / floats) frame f is read from samples + frame_off[f] and written to llr + llr_off[f].
void launch_demod(const DemodView& v, const float2* samples, long long stride, const SyncOut* sync, int frames,
                  float* llr, long long llr_stride, cudaStream_t st, int symbols_per_cta,
                  const long long* frame_off = nullptr, const long long* llr_off = nullptr,
                  const int* frames_ptr = nullptr);
// Waits of the demodulator on its staged-sample copies that hit their iteration limit
// since the library loaded on the current device (each one is counted and the symbol is
// read from global memory instead; never expected).
unsigned demod_wait_timeouts();

// Device side of the real-time ingest: the frame-extraction loop of the receive
// path (GpuRxSyncExtractor::extract_device, uhd_ldpc_ofdm_link.cpp:6901-6979, as the
// RX loop drives it, :8549-8567) over one window of samples.
struct IngestState {
    int tracking;  // in: sync state (1 tracking, 0 acquisition); out: state after the loop
    int base;      // out: samples of the window used (start of the next search)
    int frames;    // out: frames extracted
    int pad;
    unsigned long long found, miss, tracking_miss, incomplete, skipped_samples, max_start, pool_exhausted;
};
struct IngestRecord {
    int slot;      // pool slot holding the frame
    int start;     // first sample of the frame in the window
    float peak;    // fine correlation metric
    float cfo_hz;
};
struct IngestParams {
    int frame_len;       // samples per frame
    int acq_window;      // acquisition search: max(frame_len, max_buffered_frames * frame_len)
    int track_window;    // tracking search: preamble + max(256, sync_tracking_window)
    int strict_window;   // late peaks beyond max(256, 4 cp) need the late threshold
    float late_threshold;// 0: off
    int max_frames;
    int free_slots;      // pool slots available (slot list)
};
// One CTA: extract frames one after another from window[0, n) into pool slots
// (pool + slots[i] * frame_len), records to `rec`, state in/out.
void launch_ingest_extract(const float2* window, int n, const float2* preamble, const SyncParams& sp,
                           const IngestParams& ip, const int* slots, float2* pool, IngestRecord* rec,
                           IngestState* state, cudaStream_t st);

// Transmit tables resident on the device (the TX chain of gpu_ofdm_pipeline.cu:129-343, 922-1075).
struct TxView {
    int nfft, cp, num_symbols, active_sc, bits_per_symbol, pre_len;
    int code_n, code_k, blocks;  // codewords per frame
    int frame_samples;
    float amplitude;
    const int* used_bins;        // [active_sc] natural FFT bin of each active subcarrier
    const int* pilot_of_symbol;  // [num_symbols] pilot index of the symbol, -1 for none
    const int* data_of_symbol;   // [num_symbols] data index of the symbol, -1 for none
    const float2* pilot_grid;    // [pilots][active_sc]
    const float2* preamble;      // [pre_len]
    const float2* precomp_h;     // [num_symbols][active_sc] or null
    const float2* actual_h;      // [num_symbols][active_sc] or null
    const float2* twiddle;       // [nfft] exp(-2 pi i j / nfft)
    const uint32_t* gen_words;   // [code_k][gen_stride] bit-packed generator rows (bit j of word w: column 32w + j)
    int gen_stride;
    const uint32_t* gen_tab;     // [ceil(code_k/8)][256][gen_stride]: XOR of the 8 rows 8g.. selected by a byte, or null
    const int* acc_offsets;      // accumulator encoder: [m + 1] row starts in acc_cols (null: generator encoder)
    const int* acc_cols;         // information columns of each parity row
};

// Encode and modulate `frames` frames of info bits (bytes, [frames][blocks * code_k]) into
// complex frames at frames_out + f * frame_samples: c = u G (or the accumulator encoder),
// resource grid, optional precompensation, channel and frequency-domain noise (noise_var > 0:
// frame f seeded with noise_seed + f), inverse FFT, cyclic prefix, preamble, amplitude.  The
// coded bits live in stream-ordered scratch.
void launch_tx(const TxView& v, const uint8_t* info_bits, int frames, float2* frames_out, float noise_var,
               unsigned long long noise_seed, cudaStream_t st);

}  // namespace sicc
