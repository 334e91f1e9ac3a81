// Engine entry used inside the library (the serving loop).
#pragma once

#include "sicc_common.h"

namespace sicc {

// sicc_engine_decode_device_protected, plus `bp_done` (may be null) recorded on
// `stream` after the BP kernel, before the OSD launches: results of codewords
// that cannot go to OSD are final once it completes.
// With `device_count` (device int) the batch holds *device_count codewords, at most
// `codewords`: the launches are sized for `codewords` and every kernel reads the count on
// the device, so one recorded sequence serves batches of any size up to it.
int engine_decode(unsigned long long handle, int codewords, const unsigned char* device_code_ids,
                  const unsigned char* device_protection, const float* device_llr, const long long* device_llr_offsets,
                  unsigned char* device_info, const long long* device_info_offsets, unsigned char* device_success,
                  unsigned char* device_used_osd, unsigned char* device_iterations, cudaStream_t stream,
                  cudaEvent_t bp_done, const int* device_count = nullptr);

// Before recording engine_decode into a CUDA graph: uploads the code tables and sizes the
// mixed kernel's scratch for batches of up to `max_codewords`, so the recorded launches
// allocate and copy nothing.
int engine_prepare_capture(unsigned long long handle, int max_codewords);

// The device the engine's tables live on, its largest n and k (for buffer sizing).
int engine_bounds(unsigned long long handle, int* out_n_max, int* out_k_max);

// Per registered code (in id order, at most `max_codes`): 1 when a protected codeword of it that
// BP fails goes on to OSD, else 0 (its BP result is final).
int engine_code_routes(unsigned long long handle, unsigned char* out_routes, int max_codes, int* out_count);

}  // namespace sicc
