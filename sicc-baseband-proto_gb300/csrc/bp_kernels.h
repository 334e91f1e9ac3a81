// Launch interface of the belief-propagation and OSD kernels.
#pragma once

#include "sicc_common.h"

namespace sicc {

constexpr int kBpThreads = 256;

// Launch shape of the persistent layered kernel; zero fields take defaults.
struct BpLaunch {
    int slots_per_cta = 0;  // codewords resident per CTA (multiple of 32/group)
    int ctas = 0;           // grid size (persistent CTAs)
};

// All launchers are asynchronous on `st`; io.work_counter must point at one
// device int (reset by the launcher).
void launch_bp_layered(const LayeredView& cv, const BpParams& p, const BpIO& io, const BpLaunch& shape,
                       cudaStream_t st);
void launch_bp_flooding(const FloodView& cv, const BpParams& p, const BpIO& io, cudaStream_t st);
size_t layered_smem_bytes(const LayeredView& cv, int slots, bool track_best, int* slot_floats_out);
int layered_default_slots(const LayeredView& cv, bool track_best);

// OSD over a device work list; `warps_per_cta`/`ctas` <= 0 take defaults.
void launch_osd(const OsdView& ov, const OsdIO& io, int max_items, cudaStream_t st, int warps_per_cta = 0,
                int ctas = 0);

// OSD of long codes, one CTA per codeword (io.hviews for mixed batches, else
// `hv`); nmax/mmax/poolmax/nnzmax (edges of H) bound the codes of the launch.
void launch_osd_h(const OsdHView& hv, int nmax, int mmax, int poolmax, int nnzmax, const OsdIO& io, int max_items,
                  cudaStream_t st);
size_t osd_h_smem_bytes(int nmax, int mmax, int poolmax);

}  // namespace sicc
