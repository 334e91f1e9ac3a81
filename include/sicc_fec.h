/*
 * sicc_fec.h — C ABI of the GB300 LDPC decoder library (libsicc_gb300.so).
 *
 * Drop-in replacement for the reference's BP/OSD decoder library.  Every
 * declaration below keeps the name, argument order, argument meaning, status
 * codes and last-error convention of the reference interface it replaces;
 * citations are paths inside the reference project:
 *   API = source/cpp_cuda/portable/usrp_video_link_portable_20260513/third_party/
 *         cuda_osd/include/matlab_decoder_c_api.h
 *   L   = source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp (call sites of the
 *         two entry points and the config field that API does not declare)
 *
 * Conventions (API:67-71,134; L:3162-3786):
 *   - handles are opaque unsigned long long, 0 = invalid;
 *   - every int-returning call returns 0 (OK), 1 (INVALID_ARGUMENT) or
 *     2 (INTERNAL_ERROR) and leaves a message for cuda_osd_get_last_error();
 *   - LLRs are float32 [codewords][n], positive = bit 0;
 *   - bits are one per unsigned char; information bits are the first k
 *     codeword positions (systematic-front codes);
 *   - output arrays are caller-owned host memory unless a name says device.
 */
#ifndef SICC_FEC_H
#define SICC_FEC_H

#ifdef _WIN32
#define SICC_API __declspec(dllexport)
#else
#define SICC_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* API:17-32 */
typedef struct cuda_osd_stream_config_t {
    int n;
    int k;
    int m;
    int max_batch_size;
    int min_batch_size;
    unsigned long long max_latency_us;
    double arrival_ewma_alpha;
    unsigned long long default_interarrival_us;
    int bp_max_iterations;
    float bp_normalization;
    float bp_offset;
    float bp_damping;
    float bp_min_abs_llr_accept;
    int osd_threads;
} cuda_osd_stream_config_t;

/* API:34-39 */
typedef struct cuda_osd_osd_config_t {
    int n;
    int k;
    int max_batch_size;
    int osd_threads;
} cuda_osd_osd_config_t;

/* API:41-51 plus the `schedule` field the reference link driver sets
 * (L:3658; 0 flooding, 1 node-parallel, 2 coloured layered, 3 flat layered,
 * L:410). */
typedef struct cuda_osd_bp_csr_config_t {
    int n;
    int m;
    int max_batch_size;
    int max_iterations;
    float normalization;
    float offset;
    float damping;
    float min_abs_llr_accept;
    int nnz;
    int schedule;
} cuda_osd_bp_csr_config_t;

/* API:53-65 */
typedef struct cuda_osd_stream_stats_t {
    unsigned long long submitted_codewords;
    unsigned long long decoded_codewords;
    unsigned long long bp_success_codewords;
    unsigned long long osd_fallback_codewords;
    unsigned long long decoded_batches;
    unsigned long long current_pending_codewords;
    unsigned long long max_pending_codewords;
    unsigned long long last_submit_timestamp_us;
    double ewma_interarrival_us;
    double average_batch_size;
    double total_decode_ms;
} cuda_osd_stream_stats_t;

/* API:67-71 */
enum {
    CUDA_OSD_STATUS_OK = 0,
    CUDA_OSD_STATUS_INVALID_ARGUMENT = 1,
    CUDA_OSD_STATUS_INTERNAL_ERROR = 2
};

/* Stream BP->OSD decoder.  API:73-74.  Without matrices it decodes the
 * reference's default code, CCSDS (128,64) (API users: gpu_bp_osd_awgn_bench.cpp:181-201). */
SICC_API int cuda_osd_create_stream_decoder(const cuda_osd_stream_config_t* config,
                                            unsigned long long* out_handle);
/* L:3251-3256: dense H (m*n row-major 0/1) and the systematic parity table
 * [k][parity_words_per_row] (bit p of row i = parity bit p of encode(e_i)). */
SICC_API int cuda_osd_create_stream_decoder_with_matrices(const cuda_osd_stream_config_t* config,
                                                          const unsigned char* dense_h,
                                                          const unsigned long long* systematic_parity,
                                                          int parity_words_per_row,
                                                          unsigned long long* out_handle);
SICC_API int cuda_osd_destroy_stream_decoder(unsigned long long handle); /* API:75 */

/* OSD-only decoder.  API:76-78 */
SICC_API int cuda_osd_create_osd_decoder(const cuda_osd_osd_config_t* config, unsigned long long* out_handle);
SICC_API int cuda_osd_destroy_osd_decoder(unsigned long long handle);

/* Generic CSR BP decoder.  API:79-90 */
SICC_API int cuda_osd_create_bp_csr_decoder(const cuda_osd_bp_csr_config_t* config, const int* row_ptr,
                                            const int* col_ind, unsigned long long* out_handle);
SICC_API int cuda_osd_destroy_bp_csr_decoder(unsigned long long handle);
SICC_API int cuda_osd_decode_bp_csr_batch(unsigned long long handle, const float* llrs, int codewords,
                                          unsigned char* out_code_bits, unsigned char* out_success,
                                          double* out_total_decode_ms);
/* L:3753-3759: device-resident LLRs, host outputs. */
SICC_API int cuda_osd_decode_bp_csr_device_batch(unsigned long long handle, const float* device_llrs,
                                                 int codewords, unsigned char* out_code_bits,
                                                 unsigned char* out_success, double* out_total_decode_ms);

/* OSD batch on channel LLRs.  API:91-97 */
SICC_API int cuda_osd_decode_osd_batch(unsigned long long handle, const float* llrs, int codewords,
                                       unsigned char* out_info_bits, float* out_distances,
                                       double* out_total_decode_ms, double* out_throughput_mbps);

/* Streaming I/O.  API:98-120.  submit_device_codewords consumes the device
 * buffer before it returns (L:3366-3381).  poll_ready returns codewords in
 * completion order, possibly partial sets; after flush it blocks until at
 * least one pending codeword is ready (L:3497-3530). */
SICC_API int cuda_osd_submit_codewords(unsigned long long handle, const float* llrs, int codewords,
                                       const unsigned long long* timestamps_us,
                                       const unsigned long long* frame_ids, const unsigned int* block_indices);
SICC_API int cuda_osd_submit_device_codewords(unsigned long long handle, const float* device_llrs,
                                              int codewords, const unsigned long long* timestamps_us,
                                              const unsigned long long* frame_ids,
                                              const unsigned int* block_indices);
SICC_API int cuda_osd_poll_ready(unsigned long long handle, int max_codewords, unsigned char* out_info_bits,
                                 unsigned long long* out_timestamps_us, unsigned long long* out_frame_ids,
                                 unsigned int* out_block_indices, unsigned char* out_used_osd,
                                 int* out_codewords);
SICC_API int cuda_osd_flush(unsigned long long handle);
SICC_API int cuda_osd_get_stats(unsigned long long handle, cuda_osd_stream_stats_t* out_stats); /* API:122-123 */
SICC_API unsigned long long cuda_osd_get_decoded_codewords(unsigned long long handle);       /* API:124 */
SICC_API double cuda_osd_get_total_decode_ms(unsigned long long handle);                     /* API:125 */

/* Schmidl-Cox frame search on host double IQ (API:126-133): global-maximum
 * metric, full-preamble refinement, CFO; start index is 1-based. */
SICC_API int cuda_osd_find_frame(const double* signal_real, const double* signal_imag, int signal_length,
                                 const double* preamble_real, const double* preamble_imag, int preamble_length,
                                 int pre_half_len, double sync_peak_thresh, double fs,
                                 int* out_start_idx_1based, double* out_peak, double* out_cfo_hz);
SICC_API const char* cuda_osd_get_last_error(void); /* API:134 */

/* ---------------------------------------------------------------------------
 * Extensions.  They have no counterpart in the reference interface; they
 * expose the device-resident path and the settings the reference fixes
 * inside its library.
 * ------------------------------------------------------------------------- */

/* BP schedule of a stream decoder (default 3, flat layered). */
SICC_API int sicc_fec_set_schedule(unsigned long long handle, int schedule);
/* OSD order (0..3), flip-pool size and test cap of a stream or OSD decoder
 * (defaults: order 2, min(k, 64) positions, 4096 tests). */
SICC_API int sicc_fec_set_osd_params(unsigned long long handle, int order, int max_flip_positions, int max_tests);
/* Enables or disables the OSD fallback of a stream decoder (default on). */
SICC_API int sicc_fec_set_osd_enabled(unsigned long long handle, int enabled);

/* Device-resident BP->OSD decode with a stream decoder: device LLRs in,
 * device outputs, asynchronous on `cuda_stream` (a cudaStream_t; 0 = legacy
 * default stream).  codewords <= max_batch_size.  Output pointers other than
 * device_info_bits may be null.  Calls on one handle must not overlap. */
SICC_API int sicc_fec_decode_device(unsigned long long handle, const float* device_llrs, int codewords,
                                    unsigned char* device_info_bits, unsigned char* device_success,
                                    unsigned char* device_used_osd, unsigned char* device_iterations,
                                    void* cuda_stream);
/* Device-resident CSR BP: device LLRs in; code bits, success flags and the
 * final posterior LLRs [codewords][n] out (any output may be null). */
SICC_API int sicc_bp_csr_decode_device(unsigned long long handle, const float* device_llrs, int codewords,
                                       unsigned char* device_code_bits, unsigned char* device_success,
                                       float* device_posteriors, unsigned char* device_iterations,
                                       void* cuda_stream);
/* Device-resident OSD on device LLRs [codewords][n] (OSD or stream handle). */
SICC_API int sicc_osd_decode_device(unsigned long long handle, const float* device_llrs, int codewords,
                                    unsigned char* device_info_bits, unsigned char* device_code_bits,
                                    float* device_distances, void* cuda_stream);

/* Per-kernel timing of a handle's decode calls: when enabled, CUDA events
 * bracket the BP and the OSD kernel of every call on its launching stream.
 * get_kernel_ms waits for the calls made since the previous query (or since
 * timing was enabled) and reports how many there were, the summed BP and OSD
 * kernel times and how many codewords went to OSD. */
SICC_API int sicc_fec_set_timing(unsigned long long handle, int enabled);
SICC_API int sicc_fec_get_kernel_ms(unsigned long long handle, int* out_calls, float* out_bp_ms, float* out_osd_ms,
                                    long long* out_osd_codewords);

/* Device-resident BP->OSD decode that allocates nothing.  It has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory when they decode: a receiver whose device memory is fixed once
 * it starts (reserved up front, the rest owned by the application), or a
 * receive loop with a sample deadline, where a cudaMalloc may wait on work
 * already queued on the GPU.  The BP->OSD hand-off scratch lives in one
 * static device array of the library (about 8.4 MB on every GPU that loads
 * it, held until the process exits); batches hold at most
 * SICC_FEC_STATIC_MAX_CODEWORDS codewords of n <= 256, independent of the
 * decoder's max_batch_size, and larger batches are rejected with
 * INVALID_ARGUMENT.  The first call on a device resolves the array's address
 * there (set-up), so make that first call before any stream capture.  Every
 * call shares the one array: calls whose work overlaps on the GPU (other
 * streams, other handles, other threads) race and must be serialised by the
 * caller.  Outputs match sicc_fec_decode_device bit for bit.  These calls are
 * not counted by sicc_fec_set_timing / sicc_fec_get_kernel_ms (timing records
 * would need host allocations).  The array's address is cached per device for
 * the life of the process: a cudaDeviceReset while the library is loaded is
 * not supported. */
#define SICC_FEC_STATIC_MAX_CODEWORDS 8192
SICC_API int sicc_fec_decode_device_static(unsigned long long handle, const float* device_llrs, int codewords,
                                           unsigned char* device_info_bits, unsigned char* device_success,
                                           unsigned char* device_used_osd, unsigned char* device_iterations,
                                           void* cuda_stream);

/* Launch shape of the persistent BP kernel for a stream or CSR handle (0 = default). */
SICC_API int sicc_fec_set_launch_shape(unsigned long long handle, int slots_per_cta, int ctas);

#ifdef __cplusplus
}
#endif
#endif
