/*
 * sicc_pipe.h — C ABI of the GB300 OFDM receive pipeline (libsicc_gb300.so).
 *
 * A thin C layer under the C++ class usrp_gpu_pipeline_bridge::Pipeline
 * (include/gpu_ofdm_pipeline.hpp), which keeps the signatures of the
 * reference's bridge source/cpp_cuda/uhd_cpp/src/gpu_ofdm_pipeline.hpp:10-93
 * ("PH").  Each entry point cites the PH member it serves.  Status codes and
 * cuda_osd_get_last_error() follow include/sicc_fec.h.
 *
 * Complex samples are interleaved float32 (re, im), the layout of
 * std::complex<float> / cuFloatComplex.
 */
#ifndef SICC_PIPE_H
#define SICC_PIPE_H

#include "sicc_fec.h"

#ifdef __cplusplus
extern "C" {
#endif

/* PH:12-34 (Config), plus two trailing fields the reference fixes internally. */
typedef struct sicc_pipe_config_t {
    int nfft;
    int cp;
    int preamble_len;
    int pre_half_len;
    int num_symbols;
    int active_sc;
    int bits_per_symbol;
    int code_n;
    int code_k;
    int blocks_per_frame;
    int max_rx_search_samples;
    float sample_rate;
    float sync_threshold;
    float tx_amplitude;
    float demod_noise_var;
    int use_pilot_channel_est;
    /* extensions: 0 = defaults */
    int sync_radius;        /* fine-timing radius; 0 = min(16, cp) as the CPU receiver (L:5223) */
    int max_batch_frames;   /* frames per batched call (sicc_pipe_demod_batch); 0 = 256 */
} sicc_pipe_config_t;

/* PH:37-57 (StaticTables), receive-side members. */
typedef struct sicc_pipe_tables_t {
    const int* used_indices;   /* [active_sc] shifted-grid subcarrier indices */
    const int* pilot_symbols;  /* [pilot_count] */
    int pilot_count;
    const int* data_symbols;   /* [data_count] */
    int data_count;
    const int* interp_p0;      /* [data_count] */
    const int* interp_p1;      /* [data_count] */
    const float* interp_alpha; /* [data_count] */
    const float* pilot_grid;   /* [pilot_count][active_sc] complex */
    const float* preamble;     /* [preamble_len] complex */
} sicc_pipe_tables_t;

/* PH:59-63 */
typedef struct sicc_pipe_sync_t {
    int start;    /* -1 when no frame was found */
    float metric;
    float cfo_hz;
} sicc_pipe_sync_t;

SICC_API int sicc_pipe_create(const sicc_pipe_config_t* config, int slots, unsigned long long* out_handle); /* PH:67 */
SICC_API int sicc_pipe_destroy(unsigned long long handle);                                                   /* PH:68 */
SICC_API int sicc_pipe_upload_static_tables(unsigned long long handle, const sicc_pipe_tables_t* tables);   /* PH:73 */
/* PH:83-84: frame search on host / device samples; synchronous. */
SICC_API int sicc_pipe_find_frame(unsigned long long handle, int slot, const float* host_iq, int sample_count,
                                  sicc_pipe_sync_t* out_sync);
SICC_API int sicc_pipe_find_frame_device(unsigned long long handle, int slot, const float* device_iq,
                                         int sample_count, sicc_pipe_sync_t* out_sync);
/* PH:85: search a host frame of frame_samples() samples, demodulate it; the
 * returned device LLRs [coded_bits_per_frame] belong to the slot. */
SICC_API int sicc_pipe_demod_to_device(unsigned long long handle, int slot, const float* host_frame,
                                       sicc_pipe_sync_t* out_sync, const float** out_device_llr);
/* PH:86: demodulate a device frame that starts at sample 0 with the given CFO. */
SICC_API int sicc_pipe_demod_device_to_device(unsigned long long handle, int slot, const float* device_frame,
                                              const sicc_pipe_sync_t* sync, const float** out_device_llr);
/* PH:87 */
SICC_API int sicc_pipe_demod_to_host(unsigned long long handle, int slot, const float* host_frame, float* host_llr,
                                     sicc_pipe_sync_t* out_sync);

/* Per-frame search result of the batched extension (device memory layout). */
typedef struct sicc_pipe_sync_record_t {
    int found;         /* 1 found, 2 frame runs past the buffer, 0 not found */
    int start;         /* refined start sample */
    float coarse;      /* Schmidl-Cox metric at the coarse candidate */
    float fine;        /* full-preamble correlation metric at the start */
    float cfo_hz;
    int coarse_start;
} sicc_pipe_sync_record_t;

/* Extension (no counterpart in the reference): search and demodulate `frames`
 * device buffers at device_iq + f*stride (stride in complex samples, each
 * holding sample_count samples) in one pair of launches on `cuda_stream`.
 * LLRs go to device_llr + f*coded_bits_per_frame; per-frame search results to
 * device_sync (device memory, may be null).  frames <= max_batch_frames. */
SICC_API int sicc_pipe_demod_batch(unsigned long long handle, const float* device_iq, long long stride,
                                   int sample_count, int frames, float* device_llr,
                                   sicc_pipe_sync_record_t* device_sync, void* cuda_stream);
/* As sicc_pipe_demod_batch for frames scattered in device memory: frame f is
 * read from device_iq + 2*device_frame_offsets[f] (offsets in complex
 * samples, each frame holding sample_count samples) and its LLRs written to
 * device_llr + device_llr_offsets[f] (offsets in floats).  device_sync is
 * required.  Used to demodulate the frames of many requests in one launch. */
SICC_API int sicc_pipe_demod_gather(unsigned long long handle, const float* device_iq,
                                    const long long* device_frame_offsets, int sample_count, int frames,
                                    float* device_llr, const long long* device_llr_offsets,
                                    sicc_pipe_sync_record_t* device_sync, void* cuda_stream);
/* PH:37-57 (StaticTables), transmit-side members: the encoder and the channel
 * tables of the TX chain (gpu_ofdm_pipeline.cu:854-920).  The grid tables
 * (subcarriers, pilots, preamble) come from sicc_pipe_upload_static_tables. */
typedef struct sicc_pipe_tx_tables_t {
    const unsigned char* generator_kn; /* [code_k][code_n] 0/1, row-major; null with dvb_s2_accumulator */
    int dvb_s2_accumulator;            /* 1: systematic + accumulator encoder */
    const int* row_info_offsets;       /* [code_n - code_k + 1] starts of each parity row in row_info_cols */
    const int* row_info_cols;          /* information columns of each parity row */
    const float* precomp_h;            /* [num_symbols][active_sc] complex, or null */
    const float* actual_h;             /* [num_symbols][active_sc] complex, or null */
} sicc_pipe_tx_tables_t;

SICC_API int sicc_pipe_upload_tx_tables(unsigned long long handle, const sicc_pipe_tx_tables_t* tables); /* PH:73 */
/* PH:76-81 (submit_tx_frame_device_async): encode and modulate one frame of
 * host info bits [info_bits_per_frame] (bytes 0/1) on the slot's stream,
 * asynchronously; *out_device_frame ([frame_samples] complex) belongs to the
 * slot.  With add_frequency_noise and frequency_noise_var > 0, complex
 * Gaussian noise of that variance is added to the data resource elements. */
SICC_API int sicc_pipe_tx_frame_device(unsigned long long handle, int slot, const unsigned char* host_info_bits,
                                       float frequency_noise_var, unsigned long long noise_seed,
                                       int add_frequency_noise, const float** out_device_frame);
/* PH:75 (submit_tx_frame_async): as above without noise, then the frame is
 * copied to host_frame ([frame_samples] complex; pinned memory overlaps). */
SICC_API int sicc_pipe_tx_frame(unsigned long long handle, int slot, const unsigned char* host_info_bits,
                                float* host_frame);
/* PH:82 (synchronize_tx): wait for the slot's last TX frame. */
SICC_API int sicc_pipe_tx_synchronize(unsigned long long handle, int slot);
/* Extension: `frames` frames of device info bits ([frames][info_bits_per_frame])
 * into device frames ([frames][frame_samples] complex) on cuda_stream in two
 * launches; frame f's noise is seeded with noise_seed + f (no noise when
 * frequency_noise_var <= 0).  frames <= max_batch_frames. */
SICC_API int sicc_pipe_tx_batch(unsigned long long handle, const unsigned char* device_info_bits, int frames,
                                float* device_frames, float frequency_noise_var, unsigned long long noise_seed,
                                void* cuda_stream);

/* Kernel durations (ms) of the last sicc_pipe_demod_batch / _gather call: sync, demod. */
SICC_API int sicc_pipe_last_batch_ms(unsigned long long handle, float* out_sync_ms, float* out_demod_ms);
/* (No counterpart in the reference.)  The demodulator stages each symbol's samples in
 * shared memory with bulk asynchronous copies and waits on them with an iteration limit;
 * this reports how many waits on the current device hit that limit since the library
 * loaded (each one is counted and the symbol is read from global memory instead).
 * Expected to stay 0. */
SICC_API int sicc_pipe_wait_timeouts(unsigned int* out_count);
/* (No counterpart in the reference.)  Data symbols each demodulator CTA takes
 * (1..data symbols per frame; the default is about four).  Fewer per CTA gives more
 * CTAs; each CTA also transforms the pilot symbols its data symbols interpolate from
 * (at most four), so more per CTA repeats fewer pilot transforms.  Results do not
 * depend on it.  Call after upload_static_tables. */
SICC_API int sicc_pipe_set_demod_shape(unsigned long long handle, int symbols_per_cta);

#ifdef __cplusplus
}
#endif
#endif
