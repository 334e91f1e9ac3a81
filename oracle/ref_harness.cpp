// Reference harness: the reference's own CPU receive path, compiled from its
// unmodified sources where they lie, with plain extern "C" entry points so the
// oracle tests can drive it on seeded inputs.
//
// TEST INFRASTRUCTURE ONLY.  It is built by oracle/Makefile into oracle/_ref/,
// never shipped, never linked into the product library, and used only to pin
// the C restatement in oracle/sicc_oracle.c (and as the CPU baseline).
//
// The translation unit below is the reference link driver
// source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp, included verbatim with its
// `main` renamed so its file-static functions become callable from here:
//   build_ldpc              uhd_ldpc_ofdm_link.cpp:2811-2945
//   ldpc_encode             uhd_ldpc_ofdm_link.cpp:2947-2997
//   check_syndrome          uhd_ldpc_ofdm_link.cpp:2999-3011
//   ldpc_decode_min_sum     uhd_ldpc_ofdm_link.cpp:3013-3094
//   build_systematic_parity_for_cuda_osd  uhd_ldpc_ofdm_link.cpp:3133-3160
//   fft_to_shifted_grid     uhd_ldpc_ofdm_link.cpp:3845-3859
//   symbol_to_llr_maxlog    uhd_ldpc_ofdm_link.cpp:2552-2568
//   find_frame_vector_earliest / refine  uhd_ldpc_ofdm_link.cpp:5214-5329
//   find_frame (global max) uhd_ldpc_ofdm_link.cpp:5123-5212
//   decode_frame            uhd_ldpc_ofdm_link.cpp:5331-5603
//   build_tx_frame_from_info uhd_ldpc_ofdm_link.cpp:4589-4630
#define main sicc_reference_link_main
#include "uhd_ldpc_ofdm_link.cpp"
#undef main

namespace {

struct RefPhy {
    PhyConfig phy;
};

Alist alist_from_csr(int n, int m, const int* row_ptr, const int* col_ind)
{
    Alist a;
    a.n = n;
    a.m = m;
    a.row_cols.assign(static_cast<size_t>(m), {});
    a.col_rows.assign(static_cast<size_t>(n), {});
    for (int r = 0; r < m; ++r) {
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e) {
            a.row_cols[static_cast<size_t>(r)].push_back(col_ind[e]);
            a.col_rows[static_cast<size_t>(col_ind[e])].push_back(r);
        }
    }
    return a;
}

thread_local std::string g_last_error;

} // namespace

extern "C" {

const char* ref_last_error(void) { return g_last_error.c_str(); }

void* ref_code_create(int n, int m, const int* row_ptr, const int* col_ind, int systematic_front)
{
    try {
        auto* code = new LdpcCode(build_ldpc(alist_from_csr(n, m, row_ptr, col_ind), systematic_front != 0));
        return code;
    } catch (const std::exception& ex) {
        g_last_error = ex.what();
        return nullptr;
    }
}

void ref_code_destroy(void* h) { delete static_cast<LdpcCode*>(h); }

int ref_code_k(void* h) { return static_cast<LdpcCode*>(h)->k; }

int ref_code_is_accumulator(void* h)
{
    return static_cast<LdpcCode*>(h)->encoder_kind == LdpcCode::EncoderKind::DvbS2Accumulator ? 1 : 0;
}

void ref_code_info_cols(void* h, int* out_info, int* out_pivot)
{
    const auto* c = static_cast<LdpcCode*>(h);
    for (size_t i = 0; i < c->info_cols.size(); ++i) out_info[i] = c->info_cols[i];
    for (size_t i = 0; i < c->pivot_cols.size(); ++i) out_pivot[i] = c->pivot_cols[i];
}

void ref_encode(void* h, const uint8_t* info, uint8_t* out_cw)
{
    const auto* c = static_cast<LdpcCode*>(h);
    const auto cw = ldpc_encode(*c, info);
    std::copy(cw.begin(), cw.end(), out_cw);
}

int ref_check_syndrome(void* h, const uint8_t* bits)
{
    const auto* c = static_cast<LdpcCode*>(h);
    std::vector<uint8_t> b(bits, bits + c->n);
    return check_syndrome(*c, b) ? 1 : 0;
}

int ref_systematic_parity(void* h, unsigned long long* out_table, int* out_words)
{
    try {
        int words = 0;
        const auto t = build_systematic_parity_for_cuda_osd(*static_cast<LdpcCode*>(h), words);
        if (out_table != nullptr) std::copy(t.begin(), t.end(), out_table);
        *out_words = words;
        return 0;
    } catch (const std::exception& ex) {
        g_last_error = ex.what();
        return 1;
    }
}

// Decodes `count` codewords with the reference's flooding normalized min-sum.
void ref_decode_min_sum(void* h, const float* llr, int count, int max_iter, double normalization,
                        uint8_t* out_code_bits, uint8_t* out_parity_ok, int* out_iterations)
{
    const auto* c = static_cast<LdpcCode*>(h);
    for (int b = 0; b < count; ++b) {
        const auto r = ldpc_decode_min_sum(*c, llr + static_cast<size_t>(b) * c->n, max_iter, normalization);
        std::copy(r.code_bits.begin(), r.code_bits.end(), out_code_bits + static_cast<size_t>(b) * c->n);
        if (out_parity_ok) out_parity_ok[b] = r.parity_ok ? 1 : 0;
        if (out_iterations) out_iterations[b] = r.iterations;
    }
}

void ref_fft_shifted(const float* time_iq, int nfft, float* out_shifted_iq)
{
    const auto* t = reinterpret_cast<const cf32*>(time_iq);
    const auto s = fft_to_shifted_grid(t, nfft);
    std::copy(s.begin(), s.end(), reinterpret_cast<cf32*>(out_shifted_iq));
}

// PHY configuration built by the reference's build_phy_config, with the
// preamble and pilot grid replaced by caller tables (the synthetic generator
// draws its own tables; the reference's are mt19937-seeded).
void* ref_phy_create(int nfft, int cp, int num_symbols, int active_sc, int pre_half_len,
                     const char* modulation, int pilot_period, double rate, double sync_threshold,
                     const float* preamble_iq, const float* pilot_grid_iq)
{
    try {
        Options opt;
        opt.nfft = nfft;
        opt.cp = cp;
        opt.num_symbols = num_symbols;
        opt.active_sc = active_sc;
        opt.pre_half_len = pre_half_len;
        opt.modulation = modulation;
        opt.pilot_period = pilot_period;
        opt.rate = rate;
        opt.sync_threshold = sync_threshold;
        auto* p = new RefPhy{build_phy_config(opt)};
        if (preamble_iq != nullptr) {
            const auto* pre = reinterpret_cast<const cf32*>(preamble_iq);
            p->phy.preamble.assign(pre, pre + 2 * pre_half_len);
        }
        if (pilot_grid_iq != nullptr) {
            const auto* pg = reinterpret_cast<const cf32*>(pilot_grid_iq);
            for (size_t q = 0; q < p->phy.pilot_grid.size(); ++q) {
                for (int sc = 0; sc < active_sc; ++sc) {
                    p->phy.pilot_grid[q][static_cast<size_t>(sc)] = pg[q * static_cast<size_t>(active_sc) + sc];
                }
            }
        }
        return p;
    } catch (const std::exception& ex) {
        g_last_error = ex.what();
        return nullptr;
    }
}

void ref_phy_destroy(void* h) { delete static_cast<RefPhy*>(h); }

int ref_phy_frame_len(void* h) { return static_cast<RefPhy*>(h)->phy.frame_len(); }
int ref_phy_coded_bits(void* h) { return static_cast<RefPhy*>(h)->phy.coded_bits_per_frame(); }
int ref_phy_num_pilots(void* h) { return static_cast<int>(static_cast<RefPhy*>(h)->phy.pilot_symbols.size()); }

void ref_phy_tables(void* h, int* used_indices, int* pilot_symbols, int* data_symbols, float* constellation_iq)
{
    const auto& phy = static_cast<RefPhy*>(h)->phy;
    std::copy(phy.used_indices.begin(), phy.used_indices.end(), used_indices);
    std::copy(phy.pilot_symbols.begin(), phy.pilot_symbols.end(), pilot_symbols);
    std::copy(phy.data_symbols.begin(), phy.data_symbols.end(), data_symbols);
    std::copy(phy.constellation.begin(), phy.constellation.end(), reinterpret_cast<cf32*>(constellation_iq));
}

void ref_llr_maxlog(void* h, const float* x_iq, int count, const double* sigma2, float* out)
{
    const auto& phy = static_cast<RefPhy*>(h)->phy;
    const auto* x = reinterpret_cast<const cf32*>(x_iq);
    for (int i = 0; i < count; ++i) {
        symbol_to_llr_maxlog(phy, x[i], sigma2[i], out + static_cast<size_t>(i) * phy.bits_per_symbol);
    }
}

int ref_find_frame_earliest(void* h, const float* buf_iq, int count, int max_search,
                            long long* out_start, double* out_coarse, double* out_fine, double* out_cfo_hz)
{
    const auto& phy = static_cast<RefPhy*>(h)->phy;
    const auto* x = reinterpret_cast<const cf32*>(buf_iq);
    std::vector<cf32> buf(x, x + count);
    SyncResult r;
    const bool found = find_frame_vector_earliest(buf, 0, phy, static_cast<size_t>(std::max(max_search, 0)), r);
    *out_start = static_cast<long long>(r.start);
    *out_coarse = r.coarse_metric;
    *out_fine = r.fine_peak;
    *out_cfo_hz = r.cfo_hz;
    return found ? 1 : (r.incomplete ? 2 : 0);
}

int ref_find_frame_max(void* h, const float* buf_iq, int count, long long* out_start, double* out_peak,
                       double* out_cfo_hz)
{
    const auto& phy = static_cast<RefPhy*>(h)->phy;
    const auto* x = reinterpret_cast<const cf32*>(buf_iq);
    std::deque<cf32> buf(x, x + count);
    size_t start = 0;
    double peak = 0.0;
    double cfo = 0.0;
    const bool found = find_frame(buf, phy, start, peak, cfo);
    *out_start = static_cast<long long>(start);
    *out_peak = peak;
    *out_cfo_hz = cfo;
    return found ? 1 : 0;
}

// Runs the reference decode_frame (CPU demod + CPU flooding min-sum) on one
// frame that starts at sample 0, with a known noise variance.
int ref_decode_frame(void* hp, void* hc, const float* frame_iq, double cfo_hz, int max_iter,
                     double normalization, double known_noise_var, uint8_t* out_info_bits,
                     int* out_parity_ok)
{
    try {
        const auto& phy = static_cast<RefPhy*>(hp)->phy;
        const auto* code = static_cast<LdpcCode*>(hc);
        const auto* x = reinterpret_cast<const cf32*>(frame_iq);
        std::vector<cf32> frame(x, x + phy.frame_len());
        const auto r = decode_frame(frame, phy, *code, nullptr, nullptr, cfo_hz, 1.0, max_iter, normalization,
                                    -120.0, false, nullptr, std::nullopt,
                                    known_noise_var > 0.0 ? std::optional<double>(known_noise_var) : std::nullopt);
        std::copy(r.info_bits.begin(), r.info_bits.end(), out_info_bits);
        *out_parity_ok = r.parity_ok ? 1 : 0;
        return static_cast<int>(r.info_bits.size());
    } catch (const std::exception& ex) {
        g_last_error = ex.what();
        return -1;
    }
}

// The reference transmitter for one frame: encode, map, pilot insert, IFFT, CP,
// preamble, peak normalisation to `amplitude`.
int ref_build_tx_frame(void* hp, void* hc, const uint8_t* info_bits, int info_count, float* out_iq)
{
    try {
        const auto& phy = static_cast<RefPhy*>(hp)->phy;
        const auto* code = static_cast<LdpcCode*>(hc);
        std::vector<uint8_t> info(info_bits, info_bits + info_count);
        const auto f = build_tx_frame_from_info(phy, *code, info);
        std::copy(f.begin(), f.end(), reinterpret_cast<cf32*>(out_iq));
        return static_cast<int>(f.size());
    } catch (const std::exception& ex) {
        g_last_error = ex.what();
        return -1;
    }
}

} // extern "C"
