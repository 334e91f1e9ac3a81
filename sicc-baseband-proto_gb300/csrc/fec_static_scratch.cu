// BP -> OSD decoding without any device allocation.
//
// Some callers cannot allocate device memory when they decode: a receiver
// whose device memory is fixed once it starts (its budget reserved up front,
// the rest owned by other parts of the application), or a receive loop with a
// sample deadline, where a cudaMalloc may wait on work already queued on the
// GPU and has no bound on its time.  For them this entry point
// keeps the BP -> OSD hand-off scratch (failed-codeword posteriors, their
// index list, two counters) in one file-scope device array of fixed size,
// so a call allocates nothing and its batch size is not bound by the
// decoder's max_batch_size.  The array exists once per GPU that loads the
// library and stays resident until the process exits.
#include "../../include/sicc_fec.h"
#include "sicc_common.h"

#include <mutex>

namespace sicc {

int decode_with_caller_scratch(unsigned long long handle, const float* d_llr, int count, uint8_t* d_info,
                               uint8_t* d_success, uint8_t* d_used_osd, uint8_t* d_iter,
                               unsigned char* (*scratch_on_current_device)(), int cap, cudaStream_t st);

namespace {

constexpr int kStaticMaxCodewords = SICC_FEC_STATIC_MAX_CODEWORDS;
constexpr int kStaticMaxN = 256;
constexpr size_t kStaticScratchBytes =
    256 + ((static_cast<size_t>(kStaticMaxCodewords) * 4 + 255) & ~size_t(255)) +
    static_cast<size_t>(kStaticMaxCodewords) * kStaticMaxN * sizeof(float);

// The scratch itself.  Host code must not take its address directly (the
// host-side name is only a stand-in for the device symbol); the device
// address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_fec_static_scratch[kStaticScratchBytes];

std::mutex g_addr_mu;
unsigned char* g_addr[64] = {nullptr};

// Set-up: resolves the array's device address on the current device the
// first time that device is used, and caches it for the life of the process
// (a cudaDeviceReset while the library is loaded is not supported: the cached
// address would outlive the context it belongs to).
unsigned char* static_scratch_address()
{
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64) throw std::runtime_error("device ordinal out of range for the static scratch");
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (g_addr[dev] == nullptr) {
        void* p = nullptr;
        check_cuda(cudaGetSymbolAddress(&p, g_fec_static_scratch), "cudaGetSymbolAddress(static scratch)");
        g_addr[dev] = static_cast<unsigned char*>(p);
    }
    return g_addr[dev];
}

}  // namespace
}  // namespace sicc

extern "C" int sicc_fec_decode_device_static(unsigned long long handle, const float* device_llrs, int codewords,
                                             unsigned char* device_info_bits, unsigned char* device_success,
                                             unsigned char* device_used_osd, unsigned char* device_iterations,
                                             void* cuda_stream)
{
    try {
        if (device_llrs == nullptr || device_info_bits == nullptr)
            throw sicc::InvalidArgument("null device pointer");
        if (codewords <= 0 || codewords > sicc::kStaticMaxCodewords)
            throw sicc::InvalidArgument("codewords must be in 1.." + std::to_string(sicc::kStaticMaxCodewords) +
                                        " (the fixed capacity of the static scratch)");
        // The helper makes the decoder's device current, then resolves the
        // array's address on it (set-up on that device's first call).
        return sicc::decode_with_caller_scratch(handle, device_llrs, codewords, device_info_bits, device_success,
                                                device_used_osd, device_iterations, &sicc::static_scratch_address,
                                                sicc::kStaticMaxCodewords, static_cast<cudaStream_t>(cuda_stream));
    } catch (const sicc::InvalidArgument& e) {
        sicc::set_last_error(e.what());
        return CUDA_OSD_STATUS_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        sicc::set_last_error(e.what());
        return CUDA_OSD_STATUS_INTERNAL_ERROR;
    }
}
