// Launch interface of the belief-propagation and OSD kernels.
#pragma once

#include "sicc_common.h"

namespace sicc {

constexpr int kBpThreads = 256;

// Launch shape of the persistent layered kernel; zero fields take defaults.
// Slot stride (floats) of codewords that share a warp, G lanes each: groups sit
// max(G, 4) banks apart, so their simultaneous gathers of the same table column
// do not collide, and every slot stays 16-byte aligned for the float4 copies of
// the posteriors (`floats` is a multiple of 4 on entry).
inline int pad_slot_stride(int floats, int group)
{
    if (group >= 32) return floats;
    const int bank = group < 4 ? 4 : group;
    return floats + ((bank - floats % 32) + 32) % 32;
}

struct BpLaunch {
    int slots_per_cta = 0;    // codewords resident per CTA (multiple of 32/group)
    int ctas = 0;             // grid size (persistent CTAs)
    int osd_share_rounds = 0; // warp OSD: candidate rounds between best-metric exchanges (0 = 2)
    int osd_ctas = 0;         // warp OSD grid size (0 = occupancy x SMs)
};

// All launchers are asynchronous on `st`; io.work_counter must point at one
// device int (reset by the launcher).
void launch_bp_layered(const LayeredView& cv, const BpParams& p, const BpIO& io, const BpLaunch& shape,
                       cudaStream_t st);
void launch_bp_flooding(const FloodView& cv, const BpParams& p, const BpIO& io, cudaStream_t st);
size_t layered_smem_bytes(const LayeredView& cv, int slots, bool track_best, int* slot_floats_out);
int layered_default_slots(const LayeredView& cv, bool track_best);
size_t flooding_smem_bytes(const FloodView& cv, int warps, int* slot_floats_out);

// Long codes whose state does not fit one CTA's shared memory (bp_wide.cu): one CTA per
// codeword, state in an L2-sized global scratch block.  launch_bp_layered /
// launch_bp_flooding hand such codes to these.
bool layered_needs_wide(const LayeredView& cv, bool track_best);
bool flooding_needs_wide(const FloodView& cv);
void launch_bp_layered_wide(const LayeredView& cv, const BpParams& p, const BpIO& io, cudaStream_t st);
void launch_bp_flooding_wide(const FloodView& cv, const BpParams& p, const BpIO& io, cudaStream_t st);

// OSD over a device work list; `warps_per_cta`/`ctas` <= 0 take defaults.
void launch_osd(const OsdView& ov, const OsdIO& io, int max_items, cudaStream_t st, int warps_per_cta = 0,
                int ctas = 0);

// OSD of long codes, one CTA per codeword (io.hviews for mixed batches, else
// `hv`); nmax/mmax/poolmax/nnzmax (edges of H) bound the codes of the launch.
// Launch bounds of the large-code OSD over a set of codes.
struct OsdHBounds {
    int nmax = 0, mmax = 0, poolmax = 0, nnzmax = 0;
    void add(int n, int m, int pool, int nnz);
    bool empty() const { return nmax == 0; }
};
// The large-code OSD runs in classes by m: m <= 512 and m <= 640 on 256-thread CTAs (two per SM:
// their serial pivot selections overlap; the second without staged column lists), m <= 1024 on
// 512-thread CTAs (one per SM: T fills it).
constexpr int kOsdHClasses = 3;
constexpr int kOsdHClassMaxM[kOsdHClasses] = {512, 640, 1024};
inline int osd_h_class(int m) { return m <= 512 ? 0 : m <= 640 ? 1 : 2; }
// Large-code OSD over the items of io, one launch per class present in cls[kOsdHClasses]; with more
// than one class and side streams given (kOsdHClasses - 1 of them, and as many join events), the
// classes run side by side, forked from `st` and joined back to it.
void launch_osd_h(const OsdHBounds* cls, const OsdIO& io, int max_items, cudaStream_t st,
                  const cudaStream_t* side = nullptr, cudaEvent_t fork = nullptr, const cudaEvent_t* join = nullptr);
size_t osd_h_smem_bytes(int nmax, int mmax, int poolmax);

}  // namespace sicc
