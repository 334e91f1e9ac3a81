/*
 * sicc_ingest.h — real-time receive ingest on the device (libsicc_gb300.so).
 *
 * The reference keeps this in C++ classes of its link driver
 * (source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp, "L"), without a C ABI:
 *   GpuOnlineIqBuffer           L:7565-7847  device IQ ring fed from the radio thread
 *   DeviceFramePool             L:5666-5744  leased device frame buffers
 *   GpuRxSyncExtractor::extract_device  L:6901-6979  frame search + extraction
 * and the RX loop that drives them (L:8480-8567).  Here one object holds the
 * three: samples pushed from the host land in a device ring (with a mirrored
 * tail, so any search window is contiguous and is searched in place); one
 * call runs the loop's step -- take the window (the latest samples when the
 * ring is more than 3/4 full, else wait for buffered_min samples), extract
 * frames one after another in a single device launch (acquisition /
 * tracking, the late-peak and incomplete rules of extract_device), consume
 * the samples used -- and returns the frames found, each in a leased pool
 * slot, ready for sicc_pipe_demod_gather.  Status codes follow sicc_fec.h.
 */
#ifndef SICC_INGEST_H
#define SICC_INGEST_H

#include "sicc_pipe.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sicc_ingest_config_t {
    long long ring_samples;         /* ring capacity, complex samples (capacity_bytes / 8, >= 4096) */
    int pool_frames;                /* DeviceFramePool capacity (at least 4) */
    int max_buffered_frames;        /* acquisition window, in frames (PhyConfig::max_buffered_frames) */
    int sync_tracking_window;       /* tracking search beyond the preamble (at least 256 used) */
    float sync_late_peak_threshold; /* 0: off */
    int buffered_min;               /* samples the step waits for (RX loop: peek min) */
    int buffered_max;               /* samples of one window (RX loop: peek / latest max) */
} sicc_ingest_config_t;

typedef struct sicc_ingest_frame_t {
    int slot;           /* pool slot holding frame_samples complex samples */
    float peak;         /* fine correlation metric */
    float cfo_hz;
    int pad;
    long long position; /* stream index of the frame's first sample (samples pushed before it) */
} sicc_ingest_frame_t;

typedef struct sicc_ingest_stats_t {
    unsigned long long found, miss, tracking_miss, incomplete, skipped_samples, max_start;
    unsigned long long dropped_samples, pool_exhausted;
    long long buffered;   /* samples in the ring */
    int tracking;         /* 1 while tracking */
    int free_slots;
} sicc_ingest_stats_t;

/* Create on a pipeline (its PHY, tables and search parameters; tables uploaded). */
SICC_API int sicc_ingest_create(unsigned long long pipe_handle, const sicc_ingest_config_t* config,
                                unsigned long long* out_handle);
SICC_API int sicc_ingest_destroy(unsigned long long handle);
/* GpuOnlineIqBuffer::push (L:7593-7630): copy host samples into the ring
 * (asynchronously; pinned memory overlaps), dropping the oldest samples when
 * it is full.  Thread-safe against sicc_ingest_step; while a step searches
 * the oldest samples in place, a push that does not fit drops its own newest
 * samples instead (the reference searches a copy of the window). */
SICC_API int sicc_ingest_push(unsigned long long handle, const float* host_iq, long long count);
/* One step of the RX loop's device branch (L:8480-8567); frames found go to
 * out_frames[max_frames] (*out_count of them), each holding a pool slot until
 * sicc_ingest_release.  Waits up to timeout_ms for buffered_min samples. */
SICC_API int sicc_ingest_step(unsigned long long handle, int max_frames, int timeout_ms,
                              sicc_ingest_frame_t* out_frames, int* out_count);
/* Device address of a pool slot ([frame_samples] complex) and of the pool
 * (slot s at pool + 2 * s * frame_samples floats, for sicc_pipe_demod_gather). */
SICC_API int sicc_ingest_frame_ptr(unsigned long long handle, int slot, const float** out_device_frame);
SICC_API int sicc_ingest_pool(unsigned long long handle, const float** out_device_pool, int* out_frame_samples);
/* DeviceFramePool::Lease release (L:5679-5686). */
SICC_API int sicc_ingest_release(unsigned long long handle, int slot);
SICC_API int sicc_ingest_stats(unsigned long long handle, sicc_ingest_stats_t* out);
/* GpuOnlineIqBuffer::close (L:7768-7773): wakes a waiting step. */
SICC_API int sicc_ingest_close(unsigned long long handle);

#ifdef __cplusplus
}
#endif
#endif
