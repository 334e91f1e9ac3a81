// Engine entry used inside the library (the serving loop).
#pragma once

#include "sicc_common.h"

namespace sicc {

// sicc_engine_decode_device_protected, plus `bp_done` (may be null) recorded on
// `stream` after the BP kernel, before the OSD launches: results of codewords
// that cannot go to OSD are final once it completes.
int engine_decode(unsigned long long handle, int codewords, const unsigned char* device_code_ids,
                  const unsigned char* device_protection, const float* device_llr, const long long* device_llr_offsets,
                  unsigned char* device_info, const long long* device_info_offsets, unsigned char* device_success,
                  unsigned char* device_used_osd, unsigned char* device_iterations, cudaStream_t stream,
                  cudaEvent_t bp_done);

}  // namespace sicc
