// Shared host/device definitions of the SICC GB300 receive-path library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

namespace sicc {

// Thrown by host code; the C ABI converts it to a status code plus a
// thread-local last-error string (the convention of the reference's
// matlab_decoder_c_api.h:67-71,134).
struct InvalidArgument : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void check_cuda(cudaError_t st, const char* what)
{
    if (st != cudaSuccess) {
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(st));
    }
}

void set_last_error(const std::string& msg);
const char* last_error();

// Number of streaming multiprocessors on the current device (cached per device).
int device_sm_count();

// Stream-ordered pool of kernel scratch on `device` (cudaMallocFromPoolAsync /
// cudaFreeAsync around a launch); blocks are kept for later launches.
cudaMemPool_t scratch_pool(int device);

// Raises a kernel's dynamic shared-memory limit on the current device to at
// least `bytes`; never lowers it, so launches of the same kernel with other
// sizes that are still queued on other streams keep their grant.
cudaError_t grant_dynamic_smem(const void* kernel, size_t bytes);

// ---------------------------------------------------------------------------
// Device views shared by the kernels and their launchers.
// ---------------------------------------------------------------------------

// Layered schedule of one code: `num_layers` layers of `width` row slots, each
// row slot holding up to `maxdeg` variable indices (-1 = no edge).  Rows of a
// layer touch disjoint variables, so processing a layer's rows in parallel is
// the same computation as processing them one after another.  Table layout is
// [layer][slot j][row] so the lanes of a group read consecutive words.
struct LayeredView {
    int n;
    int num_layers;
    int width;          // padded rows per layer (multiple of group)
    int maxdeg;         // max row degree (<= 27)
    int group;          // lanes per codeword: power of two, <= 32
    int rows_per_lane;  // width / group
    const int* vars;    // [num_layers][maxdeg][width]
    int m;              // rows of the code
    const int* layer_start;  // [num_layers + 1] first row of each layer in layer order (rows packed)
};

// Flooding schedule: rows in CSR order plus the column view used for the
// variable-node sums (edges of each column in increasing row order).
struct FloodView {
    int n, m, edges, maxdeg;
    const int* row_ptr;   // [m+1]
    const int* col_ind;   // [E]
    const int* col_ptr;   // [n+1]
    const int* col_edge;  // [E] edge id
    const int* edge_row;  // [E] row of the edge
};

struct BpParams {
    float alpha;           // normalization
    float beta;            // offset (0 = plain normalized min-sum)
    float damping;         // flooding only: variable-message damping
    float min_abs_accept;  // a zero-syndrome result with min |posterior| below this goes to OSD
    int max_iter;
    int route_failures_to_osd;  // 1: failures are appended to the OSD work list
};

// Outputs of a BP launch; every pointer except llr/success may be null.
struct BpIO {
    const float* llr;      // [count][n]
    int count;
    uint8_t* out_bits;     // [count][out_stride]: first out_len hard-decision bits
    int out_len;
    int out_stride;
    uint8_t* success;      // [count] 1 = zero syndrome (and accepted)
    uint8_t* iterations;   // [count]
    float* app_out;        // [count][n] final posterior LLRs
    // OSD hand-off (scratch, device memory): the best-syndrome posterior of each
    // routed codeword, its index, and the running count.
    float* osd_llr;        // [cap][n]
    int* osd_index;        // [cap]
    int* osd_count;        // [1]
    uint8_t* used_osd;     // [count]
    int* work_counter;     // [1] dynamic-scheduling counter (zeroed by the launcher)
};

// Ordered-statistics decoding of one code.
struct OsdView {
    int n, k;
    int nw;                // 64-bit words per length-n row
    int kw;                // 64-bit words per length-k column
    const uint64_t* pcols; // [n-k][kw]: column c of the parity part P as a k-bit vector
    int pool;              // flip-pool size K = min(k, max_flip_positions)
    int num_tests;         // total tests including the base (<= max_tests)
    const uint32_t* combos;// [num_tests-1]: flip-pool indices packed 3 x 10 bits (1023 = none)
};

// OSD tables of a code the warp kernel does not cover (n > 256 or k > 128):
// elimination runs on H (m x n) instead of G, see osd_large.cu.
struct OsdHView {
    int n, m, k;           // n == 0: not handled by the large-code kernel
    int mw;                // 32-bit words per row-operation row: ceil(m / 32)
    const int* col_ptr;    // [n+1] columns of H
    const int* col_rows;   // [nnz]
    const int* row_ptr;    // [m+1] rows of H
    const int* col_ind;    // [nnz]
    int pool;              // flip-pool size min(k, max_flip_positions)
    int num_tests;         // tests including the base
    const uint32_t* combos;// [num_tests-1] packed flip-pool indices, as OsdView::combos
};

struct OsdIO {
    const float* llr;        // posterior rows, indexed by work item
    const int* index;        // [items] codeword index of each item (null: item i -> codeword i)
    const int* count_ptr;    // device count of items (null: use count)
    int count;
    uint8_t* out_info;       // [codewords][info_stride] first k decoded bits
    int info_stride;
    uint8_t* out_code;       // [codewords][n] decoded codeword (optional)
    float* out_metric;       // [codewords] winning metric (optional)
    uint8_t* used_osd;       // [codewords] set to 1 (optional)
    // mixed-code batches (all null for one code): per item its code's tables,
    // its posterior row at llr + row_off[item] (or llr + llr_off[codeword]),
    // its info bits at out_info + info_off[codeword]
    const OsdView* views;
    const OsdHView* hviews;  // large-code tables by code id (the large-code kernel)
    const uint8_t* code_of;  // [codewords] code id
    const long long* llr_off;
    const long long* info_off;
    const long long* row_off;
    // warp OSD: rounds of 32 candidates (one per lane) between exchanges of the
    // warp's best metric, which tightens every lane's pruning bound (0 = 2);
    // the winner does not depend on it
    int share_rounds;
    // Work counters (device ints the launcher zeroes on the stream): each warp (warp kernel) or
    // CTA (large-code kernel, one counter per class) takes its next item from them, so a few
    // expensive codewords do not hold up one warp's share.  Null: items by static striding.
    int* work;      // warp kernel
    int* work_h;    // [kOsdHClasses] large-code kernel
};

}  // namespace sicc
