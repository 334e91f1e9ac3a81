// Per-frame benchmark of the usrp_gpu_pipeline_bridge::Pipeline class.
//
// Written against the class interface only (gpu_ofdm_pipeline.hpp), so the
// same source builds against either implementation of that interface: the
// GB300 library (include/ + libsicc_gb300.so) or the reference's own CUDA
// pipeline (source/cpp_cuda/uhd_cpp/src/gpu_ofdm_pipeline.cu + .hpp).  It
// times what a link driver does per frame with that class, in the reference's
// offline pipeline benchmark configuration
// (source/cpp_cuda/uhd_cpp/tests/gpu_ofdm_pipeline_bench.cpp:21-38): FFT 1024,
// CP 72, 96 symbols with a full-band QPSK pilot every 4th, 768 active
// subcarriers, a 512-sample half-repeated preamble, a rate-1/2 repetition code
// (n = 128, k = 64), 12.5 MS/s, amplitude 0.2, known noise variance 1e-5.
//
//   tx:        submit_tx_frame_async + synchronize_tx   (host info -> host frame)
//   rx:        demod_frame_to_host_llr                  (host frame -> sync,
//              demod -> host LLRs)
//   roundtrip: both, on each frame's own bits
//
// Hard decisions of a few transmitted frames are checked against the coded
// bits (noiseless loop-back: every bit must be right).  Prints one JSON line.
#include "gpu_ofdm_pipeline.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

using usrp_gpu_pipeline_bridge::Complex32;
using usrp_gpu_pipeline_bridge::Config;
using usrp_gpu_pipeline_bridge::Pipeline;
using usrp_gpu_pipeline_bridge::StaticTables;

namespace {

struct Args {
    int frames = 4000;
    int warmup = 64;
    int slots = 3;
    int check = 8;
};

Complex32 qpsk_point(unsigned two_bits)
{
    const float a = 0.70710678118654752f;
    return Complex32((two_bits & 2u) ? -a : a, (two_bits & 1u) ? -a : a);
}

// Tables with the structure of the benchmark configuration; contents drawn from
// one seeded generator (QPSK preamble halves and pilots).
StaticTables make_tables(const Config& c, int pilot_period, std::vector<int>& data_syms)
{
    StaticTables t;
    std::mt19937 rng(20260513u);
    t.generator_kn.assign(static_cast<size_t>(c.code_k) * c.code_n, 0);
    for (int r = 0; r < c.code_k; ++r) {
        t.generator_kn[static_cast<size_t>(r) * c.code_n + r] = 1;
        t.generator_kn[static_cast<size_t>(r) * c.code_n + r + c.code_k] = 1;
    }
    const int n2 = c.nfft / 2, a2 = c.active_sc / 2;
    for (int i = n2 - a2; i < n2; ++i) t.used_indices.push_back(i);
    for (int i = n2 + 1; i <= n2 + a2; ++i) t.used_indices.push_back(i);
    t.pilot_symbol_index.assign(c.num_symbols, -1);
    t.data_symbol_index.assign(c.num_symbols, -1);
    for (int s = 0; s < c.num_symbols; ++s) {
        if (s % pilot_period == 0) {
            t.pilot_symbol_index[s] = static_cast<int>(t.pilot_symbols.size());
            t.pilot_symbols.push_back(s);
        } else {
            t.data_symbol_index[s] = static_cast<int>(t.data_symbols.size());
            t.data_symbols.push_back(s);
        }
    }
    const int P = static_cast<int>(t.pilot_symbols.size());
    for (int s : t.data_symbols) {
        // surrounding pilots; symbols after the last pilot take the last one
        int lo = (s / pilot_period);
        int hi = lo + 1;
        if (hi >= P) hi = lo = P - 1;
        t.interp_p0.push_back(lo);
        t.interp_p1.push_back(hi);
        t.interp_alpha.push_back(lo == hi ? 0.0f
                                          : static_cast<float>(s - t.pilot_symbols[lo]) /
                                                static_cast<float>(t.pilot_symbols[hi] - t.pilot_symbols[lo]));
    }
    std::vector<Complex32> half(static_cast<size_t>(c.pre_half_len));
    for (auto& x : half) x = qpsk_point(rng() & 3u);
    t.preamble = half;
    t.preamble.insert(t.preamble.end(), half.begin(), half.end());
    t.pilot_grid.resize(static_cast<size_t>(P) * c.active_sc);
    for (auto& x : t.pilot_grid) x = qpsk_point(rng() & 3u);
    data_syms = t.data_symbols;
    return t;
}

void fill_info(std::vector<uint8_t>& info, uint32_t frame)
{
    std::mt19937 rng(0x9e3779b9u ^ frame);
    for (auto& b : info) b = static_cast<uint8_t>(rng() & 1u);
}

double seconds(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b)
{
    return std::chrono::duration<double>(b - a).count();
}

}  // namespace

int main(int argc, char** argv)
{
    Args a;
    for (int i = 1; i + 1 < argc; i += 2) {
        const std::string k = argv[i];
        const int v = std::atoi(argv[i + 1]);
        if (k == "--frames") a.frames = v;
        else if (k == "--warmup") a.warmup = v;
        else if (k == "--slots") a.slots = v;
        else if (k == "--check-frames") a.check = v;
    }
    try {
        Config c;
        c.nfft = 1024;
        c.cp = 72;
        c.num_symbols = 96;
        c.active_sc = 768;
        c.pre_half_len = 256;
        c.preamble_len = 512;
        c.bits_per_symbol = 2;
        c.code_n = 128;
        c.code_k = 64;
        c.sample_rate = 12.5e6f;
        c.tx_amplitude = 0.20f;
        c.demod_noise_var = 1.0e-5f;
        const int pilot_period = 4;
        std::vector<int> data_syms;
        StaticTables t = make_tables(c, pilot_period, data_syms);
        c.blocks_per_frame = static_cast<int>(data_syms.size()) * c.active_sc * c.bits_per_symbol / c.code_n;
        c.max_rx_search_samples = c.frame_samples();

        Pipeline pipe(c, a.slots);
        pipe.upload_static_tables(t);
        std::vector<std::vector<uint8_t>> info(a.slots, std::vector<uint8_t>(c.info_bits_per_frame()));
        std::vector<std::vector<Complex32>> frame(a.slots, std::vector<Complex32>(c.frame_samples()));
        std::vector<std::vector<float>> llr(a.slots, std::vector<float>(c.coded_bits_per_frame()));

        auto tx = [&](int i) {
            const int s = i % a.slots;
            fill_info(info[s], static_cast<uint32_t>(i));
            pipe.submit_tx_frame_async(s, info[s].data(), frame[s].data());
            pipe.synchronize_tx(s);
        };
        auto rx = [&](int i, int src) {
            const int s = i % a.slots;
            pipe.demod_frame_to_host_llr(s, frame[src].data(), llr[s].data());
        };
        for (int i = 0; i < a.warmup; ++i) {
            tx(i);
            rx(i, i % a.slots);
        }
        auto t0 = std::chrono::steady_clock::now();
        for (int i = 0; i < a.frames; ++i) tx(i);
        const double tx_s = seconds(t0, std::chrono::steady_clock::now());
        t0 = std::chrono::steady_clock::now();
        for (int i = 0; i < a.frames; ++i) rx(i, 0);
        const double rx_s = seconds(t0, std::chrono::steady_clock::now());

        long long errors = 0, bits = 0;
        for (int i = 0; i < a.check && i < a.frames; ++i) {
            tx(i);
            rx(i, i % a.slots);
            const int s = i % a.slots;
            for (int b = 0; b < c.coded_bits_per_frame(); ++b) {
                const int blk = b / c.code_n, col = b % c.code_n;
                const uint8_t want = info[s][static_cast<size_t>(blk) * c.code_k + col % c.code_k];
                errors += ((llr[s][b] < 0.0f ? 1 : 0) != want);
                ++bits;
            }
        }
        t0 = std::chrono::steady_clock::now();
        for (int i = 0; i < a.frames; ++i) {
            tx(i);
            rx(i, i % a.slots);
        }
        const double rt_s = seconds(t0, std::chrono::steady_clock::now());
        std::printf("{\"frames\": %d, \"frame_samples\": %d, \"coded_bits_per_frame\": %d, "
                    "\"info_bits_per_frame\": %d, \"tx_fps\": %.3f, \"rx_fps\": %.3f, \"roundtrip_fps\": %.3f, "
                    "\"hard_errors\": %lld, \"checked_bits\": %lld}\n",
                    a.frames, c.frame_samples(), c.coded_bits_per_frame(), c.info_bits_per_frame(),
                    a.frames / tx_s, a.frames / rx_s, a.frames / rt_s, errors, bits);
        return errors == 0 ? 0 : 3;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
