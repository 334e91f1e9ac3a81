/*
 * sicc_devloop.h — device-resident request loop of the GB300 decoder
 * (libsicc_gb300.so).
 *
 * No counterpart in the reference interface; the reference's nearest form is
 * the decode thread of its receive loop (source/cpp_cuda/uhd_cpp/src/
 * uhd_ldpc_ofdm_link.cpp:9922-10130), which batches on the host.
 *
 * The loop is one or more lanes, each a CUDA graph on its own stream whose
 * body is repeated on the device by a conditional (while) node, with no host
 * work between iterations.  The lanes share the request and completion rings
 * (each has its own engine and budgets), so one lane admits and decodes while
 * another finishes a batch.  Each lane iteration:
 *   1. admits requests in submission order from a request ring in pinned
 *      host memory, as many as fit the iteration's device state -- its
 *      codeword, LLR, frame and IQ-sample budgets (the HBM each lane holds
 *      for request state) -- when no other lane is admitting at that moment;
 *   2. copies the admitted requests' inputs (codeword LLRs, or OFDM IQ
 *      frames) from their pinned host buffers into that device state and lays
 *      out the batch;
 *   3. searches and demodulates the IQ frames of each registered OFDM profile
 *      (one batched sync + demod launch pair per profile), their LLRs landing
 *      in the batch beside the LLR requests';
 *   4. decodes the batch with the mixed-code engine: one persistent BP
 *      launch, then OSD for the codewords whose syndrome fails and whose
 *      request asked for it (protection level 1);
 *   5. copies every request's information bits to its host buffer and
 *      publishes one completion record per request in a completion ring in
 *      pinned host memory (lanes complete out of order; poll returns records
 *      as they appear): requests whose codewords are all final after BP
 *      (BP only, or no protected failure) as soon as BP ends, while OSD runs
 *      for the others, which complete after it;
 *   6. decides whether to go on: it stops when the host asks it to, after
 *      `idle_timeout_ms` without a request, or after 2^31 iterations.
 * An iteration that admits nothing skips steps 2-5 (a conditional node), so an
 * idle loop re-reads the ring about every 100 us.
 * The host only appends requests and reads completions; submit restarts the
 * lanes that have stopped.  Completions must be polled: a full completion
 * ring stops admission.  Results of a codeword do not depend on what it is
 * batched with (the engine's guarantee).  Requests arriving while an
 * iteration runs join the next one.
 *
 * Host buffers (`host_input`, `host_info` of sicc_request_t) must be
 * page-locked memory the GPU can address (cudaHostAlloc / cudaMallocHost /
 * cudaHostRegister) and stay valid until the request's completion is polled.
 * Requests are those of sicc_server.h: kind 0 (codeword LLRs of a registered
 * code) and kind 1 (OFDM IQ frames of a registered profile; frames the search
 * does not find decode from zero LLRs, as in the pipeline).  One thread at a time may
 * submit; one thread at a time may poll.  Status codes and the last-error
 * string are those of sicc_fec.h; SICC_SERVER_BUSY (sicc_server.h) means the
 * request ring is full.
 */
#ifndef SICC_DEVLOOP_H
#define SICC_DEVLOOP_H

#include "sicc_server.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sicc_devloop_config_t {
    int max_batch_codewords;         /* codewords one iteration decodes */
    long long max_batch_llr_floats;  /* LLR floats of one iteration: the request-state budget */
    int max_codes;                   /* codes the loop may register, <= 64 */
    int ring_requests;               /* request and completion ring capacity, a power of two */
    int idle_timeout_ms;             /* the loop ends after this long without a request (>= 1) */
    int max_batch_frames;            /* OFDM frames one iteration demodulates (0: no IQ requests) */
    long long max_batch_iq_samples;  /* complex IQ samples one iteration holds */
    int lanes;                       /* loop graphs sharing the rings, each with its own engine and
                                        budgets (0: one; at most 16) */
} sicc_devloop_config_t;

typedef struct sicc_devloop_stats_t {
    unsigned long long submitted, completed, iterations, busy_rejections, launches;
    unsigned long long codewords;    /* decoded by the loop */
    int running;                     /* lanes whose graph is on the device */
    unsigned long long busy_iterations;  /* iterations that admitted a request (the others skip to publication) */
    int lanes;
} sicc_devloop_stats_t;

SICC_API int sicc_devloop_create(const sicc_devloop_config_t* config, unsigned long long* out_handle);
SICC_API int sicc_devloop_destroy(unsigned long long handle);
/* Registers a code (before the first start).  OSD applies to n <= 256, k <= 128
 * (warp kernel) or m <= 1024, n <= 4096 (CTA kernel), as in the engine. */
SICC_API int sicc_devloop_add_code(unsigned long long handle, const sicc_engine_code_t* code, int* out_code_id);
/* Registers an OFDM profile (before the first start): the pipeline configuration
 * and tables of include/sicc_pipe.h, the per-frame stride of a request's IQ
 * buffer (complex samples) and the registered code of its codewords
 * (blocks_per_frame of them per frame). */
SICC_API int sicc_devloop_add_phy(unsigned long long handle, const sicc_pipe_config_t* config,
                                  const sicc_pipe_tables_t* tables, int frame_stride, int code_id, int* out_phy_id);
/* Records the loop graph (first call) and launches it on the loop's own stream. */
SICC_API int sicc_devloop_start(unsigned long long handle);
/* Appends a request; SICC_SERVER_BUSY when the ring is full. */
SICC_API int sicc_devloop_submit(unsigned long long handle, const sicc_request_t* request,
                                 unsigned long long* out_request_id);
/* Up to max completions; waits up to wait_us microseconds for the first one.
 * latency_us runs from submit to the host seeing the completion; queue_us
 * from submit to the iteration that admitted it starting its decode (device
 * clock mapped to the host's at start); batch_gpu_us is that iteration's
 * admission-to-publication time on the device. */
SICC_API int sicc_devloop_poll(unsigned long long handle, int max, sicc_completion_t* out, int* out_count,
                               int wait_us);
/* Asks the loop to end and waits for it (at most `wait_ms`). */
SICC_API int sicc_devloop_stop(unsigned long long handle, int wait_ms);
SICC_API int sicc_devloop_get_stats(unsigned long long handle, sicc_devloop_stats_t* out);
/* Offered-load driver, as sicc_server_replay. */
SICC_API int sicc_devloop_replay(unsigned long long handle, const sicc_request_t* requests, const double* arrival_us,
                                 int count, sicc_completion_t* out_completions, double* out_wall_us);

#ifdef __cplusplus
}
#endif
#endif
