/*
 * sicc_tune.h — launch shapes and the autotuner of the GB300 decoders.
 *
 * No counterpart in the reference interface: the reference fixes these
 * shapes by hand (cuda_max_batch 4096 and osd_threads 256 at
 * source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp:153, 3215, 3242).
 * Here they are parameters of the library, chosen by measurement:
 *
 *   BP (stream and CSR decoders, layered schedules):
 *     lanes_per_codeword  lanes of a warp that update one codeword's rows of a
 *                         check-node layer together (a power of two <= 32;
 *                         each lane owns ceil(layer width / lanes) rows);
 *     slots_per_cta       codewords resident per CTA of the persistent kernel;
 *     ctas                persistent grid size;
 *   OSD (warp-per-codeword kernel):
 *     osd_share_rounds    candidates each warp tests between exchanges of its
 *                         best metric, in rounds of 32 (one per lane);
 *     osd_ctas            grid size;
 *   mixed-code engine (include/sicc_engine.h):
 *     warps per codeword of each registered code (1, 2 or 4: the check-node
 *     layer's rows spread over 32, 64 or 128 lanes) and warps per CTA.
 *
 * Every shape gives bit-identical results: rows of one layer share no
 * variable, and OSD pruning only drops candidates that cannot win.
 *
 * The autotuner times candidate shapes on the caller's own batch (CUDA events
 * on the decoder's stream, median of `reps` decodes after one warm-up),
 * applies the fastest to the handle and records it in a process-wide cache
 * keyed by the code (parity-check matrix and schedule), its decode settings
 * and the device (name and SM count).  Decoders and engine codes created
 * later with the same key start from the cached shape; sicc_tune_save /
 * sicc_tune_load carry the cache across processes as a text file.
 * Status codes and the last-error string are those of sicc_fec.h.
 */
#ifndef SICC_TUNE_H
#define SICC_TUNE_H

#include "sicc_fec.h"

#ifdef __cplusplus
extern "C" {
#endif

/* 0 in any field = the library's default for that field. */
typedef struct sicc_fec_shape_t {
    int lanes_per_codeword;
    int slots_per_cta;
    int ctas;
    int osd_share_rounds;
    int osd_ctas;
} sicc_fec_shape_t;

typedef struct sicc_tune_trial_t {
    sicc_fec_shape_t shape;
    float ms; /* median time of one decode of the tuning batch (BP + OSD where enabled) */
} sicc_tune_trial_t;

/* Current shape of a stream or CSR decoder (0 fields = defaults). */
SICC_API int sicc_fec_get_shape(unsigned long long handle, sicc_fec_shape_t* out_shape);
/* Sets a stream or CSR decoder's shape; a new lanes_per_codeword rebuilds the
 * layered tables (waits for the handle's work).  Rejects shapes a kernel
 * cannot run (lanes not a power of two <= 32, slots not a multiple of
 * 32 / lanes or more than 256 threads, negative sizes). */
SICC_API int sicc_fec_set_shape(unsigned long long handle, const sicc_fec_shape_t* shape);
/* Sweeps shapes on `codewords` device LLRs (<= max_batch_size), timing each
 * over `reps` decodes (1..50), applies the fastest and caches it.  Writes the
 * winner to out_best and up to max_trials trials (any may be null). */
SICC_API int sicc_fec_autotune(unsigned long long handle, const float* device_llrs, int codewords, int reps,
                               sicc_fec_shape_t* out_best, sicc_tune_trial_t* out_trials, int max_trials,
                               int* out_trial_count);

/* Warps per codeword (1, 2, 4) of an engine code: layers of width w spread
 * over 32 * warps lanes (w must be a multiple of 32 * warps for 2 and 4). */
SICC_API int sicc_engine_set_code_warps(unsigned long long engine, int code_id, int warps);
SICC_API int sicc_engine_get_code_warps(unsigned long long engine, int code_id, int* out_warps);
/* Coordinate search over every code's warps per codeword and the engine's
 * warps per CTA, timing the mixed BP kernel on the caller's batch (the
 * arguments of sicc_engine_decode_device; outputs are overwritten).  Applies
 * and caches the fastest; reports the default and the tuned BP time. */
SICC_API int sicc_engine_autotune(unsigned long long engine, int codewords, const unsigned char* device_code_ids,
                                  const float* device_llr, const long long* device_llr_offsets,
                                  unsigned char* device_info, const long long* device_info_offsets, int reps,
                                  float* out_default_ms, float* out_tuned_ms);

/* The process-wide shape cache: entries are "key value..." lines. */
SICC_API int sicc_tune_save(const char* path);
SICC_API int sicc_tune_load(const char* path);
SICC_API int sicc_tune_clear(void);
SICC_API int sicc_tune_entries(void);

#ifdef __cplusplus
}
#endif
#endif
