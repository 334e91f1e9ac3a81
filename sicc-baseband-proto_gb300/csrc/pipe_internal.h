// Pipeline entries used inside the library (the device-resident request loop).
#pragma once

#include "sicc_common.h"

namespace sicc {

struct PipeDims {
    int frame_samples;  // complex samples of one frame
    int coded_bits;     // LLRs kept per frame (whole codewords)
    int code_n, code_k, blocks;
    int preamble_len;
    int max_frames;     // max_batch_frames of the pipeline
};

int pipe_dims(unsigned long long handle, PipeDims* out);

// Scratch of the batched frame search for `frames` frames of up to `sample_count`
// samples: its size, and where its tickets (which must be zero before each search) lie.
int pipe_gather_scratch(unsigned long long handle, int sample_count, int frames, size_t* out_bytes,
                        size_t* out_ticket_offset, size_t* out_ticket_bytes);

// sicc_pipe_demod_gather for the first *frames_ptr of up to max_frames frames (device count),
// on caller scratch (tickets zeroed by the caller in stream order): allocates and
// synchronises nothing, so it can be recorded into a graph and replayed.
int pipe_gather_counted(unsigned long long handle, const float* device_iq, const long long* device_frame_offsets,
                        int sample_count, int max_frames, const int* frames_ptr, float* device_llr,
                        const long long* device_llr_offsets, void* device_sync, void* scratch, size_t scratch_bytes,
                        cudaStream_t stream);

}  // namespace sicc
