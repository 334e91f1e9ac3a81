// Host-side code compilation: CSR parity-check matrix -> device tables.
#include "code_plan.h"
#include "bp_kernels.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

namespace sicc {

namespace {
thread_local std::string g_last_error;
}

void set_last_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

int device_sm_count()
{
    static std::mutex mu;
    static int cache[64] = {0};
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 0 && dev < 64 && cache[dev] > 0) return cache[dev];
    int sms = 0;
    check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    if (dev >= 0 && dev < 64) cache[dev] = sms;
    return sms;
}

cudaMemPool_t scratch_pool(int device)
{
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= 64) throw InvalidArgument("device ordinal out of range");
    if (!pools[device]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t pool = nullptr;
        check_cuda(cudaMemPoolCreate(&pool, &props), "cudaMemPoolCreate(scratch)");
        uint64_t keep = UINT64_MAX;  // freed blocks stay in the pool for the next launch
        check_cuda(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep), "cudaMemPoolSetAttribute");
        pools[device] = pool;
    }
    return pools[device];
}

cudaError_t grant_dynamic_smem(const void* kernel, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> granted;
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    std::lock_guard<std::mutex> lock(mu);
    size_t& g = granted[{kernel, dev}];
    if (bytes <= g) return cudaSuccess;
    err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    if (err == cudaSuccess) g = bytes;
    return err;
}

bool systematic_parity(int n, int m, const int* row_ptr, const int* col_ind, std::vector<uint64_t>& out,
                       int& words, int& k)
{
    // GF(2) elimination with the parity columns (the last m) tried first, as in
    // the systematic-front construction; pivots on those columns only succeed
    // when the parity part of H is invertible.
    const int rw = (n + 63) / 64;
    std::vector<uint64_t> rows(static_cast<size_t>(m) * rw, 0);
    for (int r = 0; r < m; ++r)
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e)
            rows[static_cast<size_t>(r) * rw + (col_ind[e] >> 6)] ^= 1ull << (col_ind[e] & 63);
    if (n <= m) return false;
    k = n - m;
    std::vector<int> pivot_col(m, -1);
    int rank = 0;
    auto bit = [&](int r, int c) { return (rows[static_cast<size_t>(r) * rw + (c >> 6)] >> (c & 63)) & 1ull; };
    for (int col = k; col < n && rank < m; ++col) {
        int piv = -1;
        for (int r = rank; r < m; ++r)
            if (bit(r, col)) { piv = r; break; }
        if (piv < 0) return false;  // parity part singular: information bits are not the first k
        if (piv != rank)
            for (int w = 0; w < rw; ++w)
                std::swap(rows[static_cast<size_t>(piv) * rw + w], rows[static_cast<size_t>(rank) * rw + w]);
        for (int r = 0; r < m; ++r)
            if (r != rank && bit(r, col))
                for (int w = 0; w < rw; ++w)
                    rows[static_cast<size_t>(r) * rw + w] ^= rows[static_cast<size_t>(rank) * rw + w];
        pivot_col[rank] = col;
        ++rank;
    }
    if (rank != m) return false;
    // Row r now reads: x_{pivot_col[r]} = sum over information columns of row r.
    words = (n - k + 63) / 64;
    out.assign(static_cast<size_t>(k) * words, 0);
    for (int r = 0; r < m; ++r) {
        const int p = pivot_col[r] - k;
        for (int i = 0; i < k; ++i)
            if (bit(r, i)) out[static_cast<size_t>(i) * words + (p >> 6)] |= 1ull << (p & 63);
    }
    return true;
}

void greedy_coloring(int n, int m, const int* row_ptr, const int* col_ind, std::vector<int>& order,
                     std::vector<int>& layer_sizes)
{
    std::vector<int> color(m, 0);
    std::vector<std::vector<uint8_t>> used;
    for (int r = 0; r < m; ++r) {
        int chosen = -1;
        for (size_t c = 0; c < used.size() && chosen < 0; ++c) {
            bool clash = false;
            for (int e = row_ptr[r]; e < row_ptr[r + 1] && !clash; ++e) clash = used[c][col_ind[e]] != 0;
            if (!clash) chosen = static_cast<int>(c);
        }
        if (chosen < 0) {
            used.emplace_back(static_cast<size_t>(n), 0);
            chosen = static_cast<int>(used.size()) - 1;
        }
        color[r] = chosen;
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e) used[chosen][col_ind[e]] = 1;
    }
    order.clear();
    layer_sizes.assign(used.size(), 0);
    for (size_t c = 0; c < used.size(); ++c)
        for (int r = 0; r < m; ++r)
            if (color[r] == static_cast<int>(c)) {
                order.push_back(r);
                ++layer_sizes[c];
            }
}

void consecutive_layers(int n, int m, const int* row_ptr, const int* col_ind, std::vector<int>& layer_sizes)
{
    layer_sizes.clear();
    std::vector<int> stamp(n, -1);
    int layer = -1, size = 0;
    for (int r = 0; r < m; ++r) {
        bool clash = (layer < 0);
        for (int e = row_ptr[r]; e < row_ptr[r + 1] && !clash; ++e) clash = stamp[col_ind[e]] == layer;
        if (clash) {
            if (layer >= 0) layer_sizes.push_back(size);
            ++layer;
            size = 0;
        }
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e) stamp[col_ind[e]] = layer;
        ++size;
    }
    if (size > 0) layer_sizes.push_back(size);
}

std::vector<uint32_t> osd_combos(int pool, int order, int max_tests)
{
    std::vector<uint32_t> out;
    int tests = 1;
    for (int o = 1; o <= order && o <= 3; ++o) {
        if (pool < o || tests >= max_tests) break;
        int c[3] = {0, 1, 2};
        while (true) {
            uint32_t packed = 0x3FFFFFFFu;  // three 10-bit fields, 1023 = unused
            for (int i = 0; i < o; ++i) packed = (packed & ~(0x3FFu << (10 * i))) | (static_cast<uint32_t>(c[i]) << (10 * i));
            out.push_back(packed);
            ++tests;
            if (tests >= max_tests) break;
            int i = o - 1;
            while (i >= 0 && c[i] == pool - o + i) --i;
            if (i < 0) break;
            ++c[i];
            for (int j = i + 1; j < o; ++j) c[j] = c[j - 1] + 1;
        }
    }
    return out;
}

DeviceCode::DeviceCode(int n, int m, const int* row_ptr, const int* col_ind, int schedule,
                       const uint64_t* parity, int parity_words, bool need_osd, const OsdSettings& osd,
                       int layered_group)
    : n_(n), m_(m), schedule_(schedule), layered_group_(layered_group)
{
    if (n <= 0 || m <= 0 || m >= n) throw InvalidArgument("code dimensions must satisfy 0 < m < n");
    if (schedule < 0 || schedule > 3) throw InvalidArgument("schedule must be 0..3");
    if (layered_group < 0 || layered_group > 32 || (layered_group & (layered_group - 1)) != 0)
        throw InvalidArgument("lanes per codeword must be 0 (default) or a power of two <= 32");
    edges_ = row_ptr[m];
    if (edges_ <= 0) throw InvalidArgument("parity-check matrix has no edges");
    row_ptr_.assign(row_ptr, row_ptr + m + 1);
    col_ind_.assign(col_ind, col_ind + edges_);
    for (int r = 0; r < m; ++r) {
        if (row_ptr[r + 1] < row_ptr[r]) throw InvalidArgument("row_ptr must be non-decreasing");
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e)
            if (col_ind[e] < 0 || col_ind[e] >= n) throw InvalidArgument("col_ind out of range");
    }
    k_ = n - m;
    if (parity != nullptr) {
        if (parity_words != (n - k_ + 63) / 64) throw InvalidArgument("parity_words_per_row must be ceil((n-k)/64)");
        parity_.assign(parity, parity + static_cast<size_t>(k_) * parity_words);
        parity_words_ = parity_words;
    } else if (need_osd) {
        int kk = 0;
        if (!systematic_parity(n, m, row_ptr, col_ind, parity_, parity_words_, kk))
            throw InvalidArgument("OSD needs a full-rank code with the information bits first (systematic-front)");
    }
    if (layered()) build_layered(); else build_flood();
    if (need_osd) set_osd(osd);
}

DeviceCode::~DeviceCode()
{
    for (void* p : owned_) cudaFree(p);
    if (combos_buf_) cudaFree(combos_buf_);
    if (combos_h_buf_) cudaFree(combos_h_buf_);
}

void DeviceCode::build_layered()
{
    std::vector<int> sizes;
    if (schedule_ == kColoredLayered) {
        greedy_coloring(n_, m_, row_ptr_.data(), col_ind_.data(), row_order_, sizes);
    } else {
        consecutive_layers(n_, m_, row_ptr_.data(), col_ind_.data(), sizes);
        row_order_.resize(m_);
        for (int r = 0; r < m_; ++r) row_order_[r] = r;
    }
    int maxdeg = 0, maxw = 0;
    for (int r = 0; r < m_; ++r) maxdeg = std::max(maxdeg, row_ptr_[r + 1] - row_ptr_[r]);
    for (int s : sizes) maxw = std::max(maxw, s);
    if (maxdeg > 27) throw InvalidArgument("layered schedule supports row degree <= 27");
    int group = 1;
    while (group < maxw && group < 32) group <<= 1;
    if (layered_group_ > 0) group = std::min(layered_group_, group);  // never wider than the default
    const int rows_per_lane = (maxw + group - 1) / group;
    const int width = rows_per_lane * group;
    const int L = static_cast<int>(sizes.size());
    std::vector<int> vars(static_cast<size_t>(L) * maxdeg * width, -1);
    int pos = 0;
    for (int l = 0; l < L; ++l) {
        for (int t = 0; t < sizes[l]; ++t, ++pos) {
            const int r = row_order_[pos];
            for (int e = row_ptr_[r], j = 0; e < row_ptr_[r + 1]; ++e, ++j)
                vars[(static_cast<size_t>(l) * maxdeg + j) * width + t] = col_ind_[e];
        }
    }
    lv_.n = n_;
    lv_.num_layers = L;
    lv_.width = width;
    lv_.maxdeg = maxdeg;
    lv_.group = group;
    lv_.rows_per_lane = rows_per_lane;
    lv_.vars = device_upload(vars, owned_);
    std::vector<int> starts(static_cast<size_t>(L) + 1, 0);
    for (int l = 0; l < L; ++l) starts[l + 1] = starts[l] + sizes[l];
    lv_.m = m_;
    lv_.layer_start = device_upload(starts, owned_);
}

void DeviceCode::build_flood()
{
    std::vector<int> col_ptr(n_ + 1, 0), col_edge(edges_), edge_row(edges_);
    int maxdeg = 0;
    for (int r = 0; r < m_; ++r) {
        maxdeg = std::max(maxdeg, row_ptr_[r + 1] - row_ptr_[r]);
        for (int e = row_ptr_[r]; e < row_ptr_[r + 1]; ++e) {
            ++col_ptr[col_ind_[e] + 1];
            edge_row[e] = r;
        }
    }
    if (maxdeg > 27) throw InvalidArgument("flooding schedule supports row degree <= 27");
    for (int v = 0; v < n_; ++v) col_ptr[v + 1] += col_ptr[v];
    std::vector<int> fill(col_ptr.begin(), col_ptr.end() - 1);
    for (int e = 0; e < edges_; ++e) col_edge[fill[col_ind_[e]]++] = e;
    fv_.n = n_;
    fv_.m = m_;
    fv_.edges = edges_;
    fv_.maxdeg = maxdeg;
    fv_.row_ptr = device_upload(row_ptr_, owned_);
    fv_.col_ind = device_upload(col_ind_, owned_);
    fv_.col_ptr = device_upload(col_ptr, owned_);
    fv_.col_edge = device_upload(col_edge, owned_);
    fv_.edge_row = device_upload(edge_row, owned_);
    row_order_.resize(m_);
    for (int r = 0; r < m_; ++r) row_order_[r] = r;
}

void DeviceCode::set_osd(const OsdSettings& s)
{
    if (parity_.empty()) throw InvalidArgument("OSD tables need the systematic parity table");
    if (s.order < 0 || s.order > 3) throw InvalidArgument("OSD order must be 0..3");
    if (s.max_tests < 1) throw InvalidArgument("OSD max_tests must be >= 1");
    if (n_ > 256 || k_ > 128) throw InvalidArgument("OSD supports n <= 256 and k <= 128");
    const int kw = (k_ + 63) / 64;
    const int nk = n_ - k_;
    if (osd_.pcols == nullptr) {
        std::vector<uint64_t> pc(static_cast<size_t>(nk) * kw, 0);
        for (int c = 0; c < nk; ++c)
            for (int i = 0; i < k_; ++i)
                if ((parity_[static_cast<size_t>(i) * parity_words_ + (c >> 6)] >> (c & 63)) & 1ull)
                    pc[static_cast<size_t>(c) * kw + (i >> 6)] |= 1ull << (i & 63);
        osd_.pcols = device_upload(pc, owned_);
    }
    const int pool = std::min(k_, std::max(s.max_flip_positions, 0));
    if (pool > 1023) throw InvalidArgument("OSD flip pool must be <= 1023");
    const auto combos = osd_combos(pool, s.order, s.max_tests);
    if (combos_buf_) {
        cudaFree(combos_buf_);
        combos_buf_ = nullptr;
    }
    if (!combos.empty()) {
        check_cuda(cudaMalloc(&combos_buf_, combos.size() * sizeof(uint32_t)), "cudaMalloc(osd combos)");
        check_cuda(cudaMemcpy(combos_buf_, combos.data(), combos.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
                   "upload osd combos");
    }
    osd_.n = n_;
    osd_.k = k_;
    osd_.nw = (n_ + 63) / 64;
    osd_.kw = kw;
    osd_.pool = pool;
    osd_.num_tests = 1 + static_cast<int>(combos.size());
    osd_.combos = static_cast<const uint32_t*>(combos_buf_);
}

void DeviceCode::set_osd_h(const OsdSettings& s)
{
    if (s.order < 0 || s.order > 3) throw InvalidArgument("OSD order must be 0..3");
    if (s.max_tests < 1) throw InvalidArgument("OSD max_tests must be >= 1");
    if (m_ > 1024 || n_ > 4096) throw InvalidArgument("large-code OSD supports m <= 1024 and n <= 4096");
    const int pool = std::min(k_, std::max(s.max_flip_positions, 0));
    if (pool > 128) throw InvalidArgument("large-code OSD flip pool must be <= 128");
    if (osd_h_smem_bytes(n_, m_, pool) > 227 * 1024) throw InvalidArgument("large-code OSD tables exceed shared memory");
    if (osd_h_.n == 0) {
        std::vector<int> col_ptr(n_ + 1, 0), col_rows(edges_);
        for (int e = 0; e < edges_; ++e) ++col_ptr[col_ind_[e] + 1];
        for (int v = 0; v < n_; ++v) col_ptr[v + 1] += col_ptr[v];
        std::vector<int> fill(col_ptr.begin(), col_ptr.end() - 1);
        for (int r = 0; r < m_; ++r)
            for (int e = row_ptr_[r]; e < row_ptr_[r + 1]; ++e) col_rows[fill[col_ind_[e]]++] = r;
        osd_h_.col_ptr = device_upload(col_ptr, owned_);
        osd_h_.col_rows = device_upload(col_rows, owned_);
        osd_h_.row_ptr = device_upload(row_ptr_, owned_);
        osd_h_.col_ind = device_upload(col_ind_, owned_);
    }
    const auto combos = osd_combos(pool, s.order, s.max_tests);
    if (combos_h_buf_) {
        cudaFree(combos_h_buf_);
        combos_h_buf_ = nullptr;
    }
    if (!combos.empty()) {
        check_cuda(cudaMalloc(&combos_h_buf_, combos.size() * sizeof(uint32_t)), "cudaMalloc(osd combos)");
        check_cuda(cudaMemcpy(combos_h_buf_, combos.data(), combos.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
                   "upload osd combos");
    }
    osd_h_.n = n_;
    osd_h_.m = m_;
    osd_h_.k = k_;
    osd_h_.mw = (m_ + 31) / 32;
    osd_h_.pool = pool;
    osd_h_.num_tests = 1 + static_cast<int>(combos.size());
    osd_h_.combos = static_cast<const uint32_t*>(combos_h_buf_);
}

}  // namespace sicc
