/*
 * sicc_engine.h — mixed-code batched decoding (libsicc_gb300.so).
 *
 * No counterpart in the reference interface: the reference decodes one code
 * per decoder handle and one frame's codewords per call (CudaBpOsdDecoder /
 * CudaBpDecoder, source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp:3162-3786).
 * An engine holds several codes and decodes a batch whose codewords belong to
 * different codes — different lengths and rates — in one persistent BP launch
 * (plus one OSD launch for the codewords whose syndrome fails), with a device
 * work queue ordered largest code first.  Per code: layered normalized
 * min-sum (the schedule of sicc_fec.h's flat-layered decoders, bit-exact with
 * it), its own iteration cap, and an optional OSD fallback.
 *
 * Codeword c of a batch: LLRs at llr + llr_offset[c] (n floats of its code),
 * information bits written at info + info_offset[c] (k bytes).  All batch
 * arrays are device memory; calls are asynchronous on the given stream.
 * max_llr_floats bounds the sum of n over a batch's codewords (the OSD
 * hand-off scratch); codewords whose code id is not a registered code are
 * skipped and their outputs left untouched.  Calls on one handle must not
 * overlap on the GPU.
 */
#ifndef SICC_ENGINE_H
#define SICC_ENGINE_H

#include "sicc_fec.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sicc_engine_config_t {
    int max_codewords;      /* per batch */
    long long max_llr_floats; /* largest sum of n over a batch (OSD hand-off scratch) */
    int max_codes;          /* <= 64 */
} sicc_engine_config_t;

typedef struct sicc_engine_code_t {
    int n;
    int m;
    const int* row_ptr;     /* host CSR of H, [m+1] */
    const int* col_ind;     /* host, [nnz] */
    int max_iterations;
    float normalization;
    float offset;
    int osd_order;          /* -1: no OSD; 0..3 (n <= 256, k <= 128: warp kernel; else m <= 1024, n <= 4096) */
    int osd_max_flip_positions;
    int osd_max_tests;
} sicc_engine_code_t;

SICC_API int sicc_engine_create(const sicc_engine_config_t* config, unsigned long long* out_handle);
SICC_API int sicc_engine_destroy(unsigned long long handle);
/* Registers a code; returns its id (0, 1, ...) used in the batch's code_ids. */
SICC_API int sicc_engine_add_code(unsigned long long handle, const sicc_engine_code_t* code, int* out_code_id);
/* Launch shape of the persistent BP kernel: warps per CTA (0 = default) and CTAs (0 = fill the GPU). */
SICC_API int sicc_engine_set_launch_shape(unsigned long long handle, int warps_per_cta, int ctas);
SICC_API int sicc_engine_decode_device(unsigned long long handle, int codewords, const unsigned char* device_code_ids,
                                       const float* device_llr, const long long* device_llr_offsets,
                                       unsigned char* device_info, const long long* device_info_offsets,
                                       unsigned char* device_success, unsigned char* device_used_osd,
                                       unsigned char* device_iterations, void* cuda_stream);
/* As sicc_engine_decode_device with a protection level per codeword
 * (device_protection[c] = 1: a failed syndrome falls back to OSD when the
 * code has OSD tables; 0: BP only). */
SICC_API int sicc_engine_decode_device_protected(unsigned long long handle, int codewords,
                                                 const unsigned char* device_code_ids,
                                                 const unsigned char* device_protection, const float* device_llr,
                                                 const long long* device_llr_offsets, unsigned char* device_info,
                                                 const long long* device_info_offsets, unsigned char* device_success,
                                                 unsigned char* device_used_osd, unsigned char* device_iterations,
                                                 void* cuda_stream);
/* OSD alone on given soft values: codeword c's n values at device_llr +
 * device_llr_offsets[c] go straight to its code's OSD (codes registered
 * without OSD are skipped).  Outputs: information bits, used flag (set to 1),
 * and the winning correlation discrepancy (device_metric, may be null). */
SICC_API int sicc_engine_osd_device(unsigned long long handle, int codewords, const unsigned char* device_code_ids,
                                    const float* device_llr, const long long* device_llr_offsets,
                                    unsigned char* device_info, const long long* device_info_offsets,
                                    unsigned char* device_used_osd, float* device_metric, void* cuda_stream);
/* Kernel durations (ms) of the last decode: prepare (sort), BP, OSD. */
SICC_API int sicc_engine_last_ms(unsigned long long handle, float* out_prepare_ms, float* out_bp_ms,
                                 float* out_osd_ms);

#ifdef __cplusplus
}
#endif
#endif
