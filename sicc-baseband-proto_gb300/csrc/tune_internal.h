// Shape cache shared by the decoders and the engine (include/sicc_tune.h).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace sicc {

// FNV-1a over a sequence of integers (the code's tables and settings).
struct Fingerprint {
    uint64_t h = 1469598103934665603ull;
    void add(long long v)
    {
        for (int b = 0; b < 8; ++b) {
            h ^= static_cast<uint64_t>((v >> (8 * b)) & 0xff);
            h *= 1099511628211ull;
        }
    }
    void add(const int* p, size_t n)
    {
        add(static_cast<long long>(n));
        for (size_t i = 0; i < n; ++i) add(p[i]);
    }
    void add_float(float f)
    {
        uint32_t u = 0;
        static_assert(sizeof u == sizeof f, "float is 32 bits");
        __builtin_memcpy(&u, &f, sizeof u);
        add(static_cast<long long>(u));
    }
};

// "<kind>:<fingerprint hex>@<device name>/<SMs>" for the current device.
std::string tune_key(const char* kind, uint64_t fingerprint);
bool tune_cache_get(const std::string& key, std::vector<int>& values);
void tune_cache_put(const std::string& key, const std::vector<int>& values);
// Median of a small sample.
float median_of(std::vector<float> v);

}  // namespace sicc
