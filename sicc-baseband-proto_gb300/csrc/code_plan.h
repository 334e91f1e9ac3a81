// Host-side compilation of a parity-check matrix into the device tables the
// decoding kernels read (layered schedule, flooding schedule, OSD tables).
#pragma once

#include "sicc_common.h"

#include <memory>
#include <vector>

namespace sicc {

// BP schedules, numbered as the reference's CSR BP configuration field
// `schedule` (uhd_ldpc_ofdm_link.cpp:410, 3658): 0 flooding, 1 node-parallel
// flooding, 2 coloured layered, 3 flat (row-order) layered.
enum Schedule : int { kFlooding = 0, kNodeParallel = 1, kColoredLayered = 2, kFlatLayered = 3 };

struct OsdSettings {
    int order = 2;
    int max_flip_positions = 64;
    int max_tests = 4096;
};

// Owns a code's device tables.  Immutable after construction; safe to share
// between decoders on the same device.
class DeviceCode {
public:
    // layered_group: lanes that update one codeword's rows of a layer together (a power of
    // two <= 32; each lane then owns ceil(widest layer / group) rows of every layer).  0 = the
    // smallest power of two covering the widest layer.  Rows of one layer share no variable,
    // so every group size gives the same arithmetic.
    DeviceCode(int n, int m, const int* row_ptr, const int* col_ind, int schedule,
               const uint64_t* parity, int parity_words, bool need_osd, const OsdSettings& osd,
               int layered_group = 0);
    ~DeviceCode();
    DeviceCode(const DeviceCode&) = delete;
    DeviceCode& operator=(const DeviceCode&) = delete;

    int n() const { return n_; }
    int m() const { return m_; }
    int k() const { return k_; }
    int edges() const { return edges_; }
    int schedule() const { return schedule_; }
    bool layered() const { return schedule_ == kColoredLayered || schedule_ == kFlatLayered; }
    bool has_osd() const { return osd_.pcols != nullptr; }
    bool has_osd_h() const { return osd_h_.n != 0; }

    const LayeredView& layered_view() const { return lv_; }
    const FloodView& flood_view() const { return fv_; }
    const OsdView& osd_view() const { return osd_; }
    const OsdHView& osd_h_view() const { return osd_h_; }
    const std::vector<int>& row_order() const { return row_order_; }
    const std::vector<uint64_t>& parity_table() const { return parity_; }
    int parity_words() const { return parity_words_; }
    int layered_group_request() const { return layered_group_; }

    void set_osd(const OsdSettings& s);
    // Tables of the large-code OSD kernel (elimination on H): any full-rank
    // code with m <= 1024, n <= 4096, flip pool <= 128.
    void set_osd_h(const OsdSettings& s);

private:
    void build_layered();
    void build_flood();

    int n_ = 0, m_ = 0, k_ = 0, edges_ = 0, schedule_ = kFlatLayered;
    int layered_group_ = 0;
    std::vector<int> row_ptr_, col_ind_;
    std::vector<int> row_order_;
    std::vector<uint64_t> parity_;
    int parity_words_ = 0;
    LayeredView lv_{};
    FloodView fv_{};
    OsdView osd_{};
    OsdHView osd_h_{};
    std::vector<void*> owned_;
    void* combos_buf_ = nullptr;
    void* combos_h_buf_ = nullptr;
};

// Front-systematic parity table [k][words] (bit p of row i = parity bit p of
// the encoding of unit vector e_i), by the reduced-row-echelon construction of
// uhd_ldpc_ofdm_link.cpp:2811-2945 / 3133-3160.  Returns false when the code
// is rank deficient or its information bits are not the first k positions.
bool systematic_parity(int n, int m, const int* row_ptr, const int* col_ind, std::vector<uint64_t>& out,
                       int& words, int& k);

// Greedy row colouring (rows ascending, smallest colour without a shared
// variable); returns the rows ordered by (colour, row) and the layer sizes.
void greedy_coloring(int n, int m, const int* row_ptr, const int* col_ind, std::vector<int>& order,
                     std::vector<int>& layer_sizes);

// Flat layering: maximal runs of consecutive rows with pairwise disjoint variables.
void consecutive_layers(int n, int m, const int* row_ptr, const int* col_ind, std::vector<int>& layer_sizes);

// OSD flip combinations in the enumeration order of cpu_bp_osd_decode.m:211-229
// (order 1..order, lexicographic over the flip pool), truncated so the total
// number of tests including the base is at most max_tests.
std::vector<uint32_t> osd_combos(int pool, int order, int max_tests);

template <class T>
T* device_upload(const std::vector<T>& v, std::vector<void*>& owned)
{
    if (v.empty()) return nullptr;
    void* p = nullptr;
    check_cuda(cudaMalloc(&p, v.size() * sizeof(T)), "cudaMalloc(code table)");
    check_cuda(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload code table");
    owned.push_back(p);
    return static_cast<T*>(p);
}

}  // namespace sicc
