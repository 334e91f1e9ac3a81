/*
 * sicc_server.h — device-resident continuous-batching decode service
 * (libsicc_gb300.so).
 *
 * No counterpart in the reference interface.  The reference's nearest form is
 * its real-time receive loop: a bounded device-frame queue feeding one decode
 * thread, fixed batching windows, drop counters and no latency accounting
 * (source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp:9922-10130).
 *
 * A server owns an HBM arena (the state budget).  A submitted request —
 * codeword LLRs of one registered code, or OFDM IQ frames of one registered
 * PHY profile that need demodulation first — is admitted first-in first-out
 * when its state fits in the arena: its input is copied to the device and
 * stays there until its results are back on the host.  A scheduler thread
 * launches whatever admitted requests are ready as one batch (demodulation of
 * the IQ requests, then one mixed-code BP launch with OSD on the codewords
 * whose request asked for it), while earlier batches are still running, so
 * requests that arrive while others are on the GPU join the next launch as
 * slots and memory free up.  Results of a codeword do not depend on what it is
 * batched with.
 *
 * Host buffers of a request (input and output) must stay valid until its
 * completion has been polled; pinned memory makes the copies asynchronous.
 */
#ifndef SICC_SERVER_H
#define SICC_SERVER_H

#include "sicc_engine.h"
#include "sicc_pipe.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { SICC_SERVER_BUSY = 3 }; /* submit: the pending queue is full, retry later */

typedef struct sicc_server_config_t {
    long long hbm_budget_bytes;  /* arena for request state */
    int max_batch_codewords;     /* codewords per launch */
    int max_inflight_batches;    /* batches overlapping on the device, 1..4 */
    int max_pending_requests;    /* submitted but not yet admitted */
    int max_codes;               /* codes the server may register, <= 64 */
    int max_n;                   /* largest code length to register */
} sicc_server_config_t;

typedef struct sicc_request_t {
    int kind;                    /* 0: codeword LLRs, 1: OFDM IQ frames */
    int code_id;                 /* kind 0: registered code of the codewords */
    int phy_id;                  /* kind 1: registered OFDM profile */
    int count;                   /* codewords (kind 0) or frames (kind 1) */
    int protection;              /* 0: BP only, 1: BP with OSD fallback */
    const float* host_input;     /* kind 0: [count][n] LLRs; kind 1: [count][frame_stride] complex IQ */
    unsigned char* host_info;    /* [codewords][k] decoded information bits */
    unsigned long long tag;      /* caller's value, returned in the completion */
} sicc_request_t;

typedef struct sicc_completion_t {
    unsigned long long request_id;
    unsigned long long tag;
    int status;                  /* 0 ok */
    int codewords;
    int failed_codewords;        /* syndrome not satisfied after BP (and OSD not used) */
    int osd_codewords;
    double latency_us;           /* submit -> results on the host */
    double queue_us;             /* submit -> admitted into the arena */
    double launch_us;            /* submit -> its batch launched */
    double batch_gpu_us;         /* device time of its batch (first copy to last copy back) */
} sicc_completion_t;

typedef struct sicc_server_stats_t {
    unsigned long long submitted, completed, batches, codewords;
    unsigned long long busy_rejections;
    long long arena_bytes_in_use, arena_bytes_peak;
    double mean_batch_codewords;
} sicc_server_stats_t;

SICC_API int sicc_server_create(const sicc_server_config_t* config, unsigned long long* out_handle);
SICC_API int sicc_server_destroy(unsigned long long handle);
SICC_API int sicc_server_add_code(unsigned long long handle, const sicc_engine_code_t* code, int* out_code_id);
/* A PHY profile: the pipeline configuration and tables of include/sicc_pipe.h,
 * the per-frame buffer stride (complex samples) and the registered code its
 * codewords use (blocks_per_frame of them per frame). */
SICC_API int sicc_server_add_phy(unsigned long long handle, const sicc_pipe_config_t* config,
                                 const sicc_pipe_tables_t* tables, int frame_stride, int code_id, int* out_phy_id);
SICC_API int sicc_server_start(unsigned long long handle);
SICC_API int sicc_server_submit(unsigned long long handle, const sicc_request_t* request,
                                unsigned long long* out_request_id);
/* Up to max completions; waits up to wait_us microseconds for the first one. */
SICC_API int sicc_server_poll(unsigned long long handle, int max, sicc_completion_t* out, int* out_count,
                              int wait_us);
SICC_API int sicc_server_get_stats(unsigned long long handle, sicc_server_stats_t* out);
/* Offered-load driver: submits requests[i] at arrival_us[i] microseconds after
 * the call starts (retrying while the pending queue is full), collects every
 * completion and returns them in request order, with latency_us measured from
 * the scheduled arrival.  out_wall_us: first arrival to last completion. */
SICC_API int sicc_server_replay(unsigned long long handle, const sicc_request_t* requests, const double* arrival_us,
                                int count, sicc_completion_t* out_completions, double* out_wall_us);

#ifdef __cplusplus
}
#endif
#endif
