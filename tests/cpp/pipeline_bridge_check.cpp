// Drives usrp_gpu_pipeline_bridge::Pipeline (include/gpu_ofdm_pipeline.hpp) the
// way the reference link driver does (GpuRxSyncExtractor / GpuRxDemodChain,
// uhd_ldpc_ofdm_link.cpp:6831-7182): construct, upload tables, find a frame in
// a host buffer, demodulate it to host LLRs, and demodulate the same frame
// from device memory; then transmit a frame (host and device paths).  Inputs and outputs are raw files in one directory,
// written and checked by tests/test_gpu_ofdm.py.
//
// usage: pipeline_bridge_check <dir>
#include "gpu_ofdm_pipeline.hpp"

#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

using namespace usrp_gpu_pipeline_bridge;

template <class T>
static std::vector<T> read_bin(const std::string& path)
{
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) throw std::runtime_error("cannot open " + path);
    const auto bytes = static_cast<size_t>(f.tellg());
    f.seekg(0);
    std::vector<T> v(bytes / sizeof(T));
    f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(bytes));
    return v;
}

template <class T>
static void write_bin(const std::string& path, const T* p, size_t n)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), static_cast<std::streamsize>(n * sizeof(T)));
}

int main(int argc, char** argv)
{
    if (argc != 2) {
        std::cerr << "usage: " << argv[0] << " <dir>\n";
        return 2;
    }
    const std::string dir = argv[1];
    try {
        const auto ic = read_bin<int>(dir + "/cfg_int.bin");     // nfft cp pre_half num_symbols active_sc bps n k blocks
        const auto fc = read_bin<float>(dir + "/cfg_float.bin");  // sample_rate threshold noise_var
        Config cfg;
        cfg.nfft = ic[0];
        cfg.cp = ic[1];
        cfg.pre_half_len = ic[2];
        cfg.preamble_len = 2 * ic[2];
        cfg.num_symbols = ic[3];
        cfg.active_sc = ic[4];
        cfg.bits_per_symbol = ic[5];
        cfg.code_n = ic[6];
        cfg.code_k = ic[7];
        cfg.blocks_per_frame = ic[8];
        cfg.sample_rate = fc[0];
        cfg.sync_threshold = fc[1];
        cfg.demod_noise_var = fc[2];
        StaticTables t;
        t.used_indices = read_bin<int>(dir + "/used.bin");
        t.pilot_symbols = read_bin<int>(dir + "/pilots.bin");
        t.data_symbols = read_bin<int>(dir + "/data.bin");
        t.interp_p0 = read_bin<int>(dir + "/p0.bin");
        t.interp_p1 = read_bin<int>(dir + "/p1.bin");
        t.interp_alpha = read_bin<float>(dir + "/alpha.bin");
        t.pilot_grid = read_bin<Complex32>(dir + "/grid.bin");
        t.preamble = read_bin<Complex32>(dir + "/pre.bin");
        const auto frame = read_bin<Complex32>(dir + "/frame.bin");
        cfg.max_rx_search_samples = static_cast<int>(frame.size());

        Pipeline pipe(cfg, 3);
        pipe.upload_static_tables(t);
        const SyncResult s = pipe.find_frame(0, frame.data(), static_cast<int>(frame.size()));
        std::vector<float> llr(static_cast<size_t>(cfg.coded_bits_per_frame()));
        const SyncResult s2 = pipe.demod_frame_to_host_llr(1, frame.data() + (s.start > 0 ? s.start : 0), llr.data());
        write_bin(dir + "/llr_host.bin", llr.data(), llr.size());

        Complex32* d_frame = nullptr;
        if (cudaMalloc(&d_frame, frame.size() * sizeof(Complex32)) != cudaSuccess) throw std::runtime_error("cudaMalloc");
        cudaMemcpy(d_frame, frame.data() + (s.start > 0 ? s.start : 0),
                   (frame.size() - static_cast<size_t>(s.start > 0 ? s.start : 0)) * sizeof(Complex32),
                   cudaMemcpyHostToDevice);
        const float* d_llr = pipe.demod_frame_device_to_device_llr(2, d_frame, s);
        std::vector<float> llr_dev(llr.size());
        cudaMemcpy(llr_dev.data(), d_llr, llr_dev.size() * sizeof(float), cudaMemcpyDeviceToHost);
        cudaFree(d_frame);
        write_bin(dir + "/llr_device.bin", llr_dev.data(), llr_dev.size());

        // transmit: refused before a generator is uploaded (gpu_ofdm_pipeline.cu:930-932), then one
        // frame through submit_tx_frame_async and one with frequency-domain noise through the device path
        bool tx_threw = false;
        const auto info = read_bin<uint8_t>(dir + "/tx_info.bin");
        std::vector<Complex32> txf(static_cast<size_t>(cfg.frame_samples()));
        try {
            pipe.submit_tx_frame_async(0, info.data(), txf.data());
        } catch (const std::runtime_error&) {
            tx_threw = true;
        }
        t.generator_kn = read_bin<uint8_t>(dir + "/gen.bin");
        pipe.upload_static_tables(t);
        pipe.submit_tx_frame_async(0, info.data(), txf.data());
        pipe.synchronize_tx(0);
        write_bin(dir + "/tx_frame.bin", txf.data(), txf.size());
        const Complex32* d_tx = pipe.submit_tx_frame_device_async(1, info.data(), 0.05f, 99, true);
        pipe.synchronize_tx(1);
        std::vector<Complex32> txn(txf.size());
        cudaMemcpy(txn.data(), d_tx, txn.size() * sizeof(Complex32), cudaMemcpyDeviceToHost);
        write_bin(dir + "/tx_frame_noise.bin", txn.data(), txn.size());
        bool bad_slot_threw = false;
        try {
            pipe.find_frame(7, frame.data(), static_cast<int>(frame.size()));
        } catch (const std::runtime_error&) {
            bad_slot_threw = true;
        }
        std::FILE* out = std::fopen((dir + "/sync.txt").c_str(), "w");
        std::fprintf(out, "%d %.9g %.9g %d %.9g %.9g %d %d\n", s.start, s.metric, s.cfo_hz, s2.start, s2.metric,
                     s2.cfo_hz, tx_threw ? 1 : 0, bad_slot_threw ? 1 : 0);
        std::fclose(out);
        return 0;
    } catch (const std::exception& ex) {
        std::cerr << "error: " << ex.what() << "\n";
        return 1;
    }
}
