// Process-wide cache of tuned launch shapes (include/sicc_tune.h).
//
// Keys name the code (a fingerprint of its parity-check matrix, schedule and
// decode settings) and the device (name and SM count); values are the shape
// fields of the owner (a stream / CSR decoder, or an engine code).  The cache
// is a plain text file on disk: one "key v1 v2 ..." line per entry.
#include "../../include/sicc_tune.h"
#include "sicc_common.h"
#include "tune_internal.h"

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>

namespace sicc {
namespace {

std::mutex g_tune_mu;
std::map<std::string, std::vector<int>> g_tune;

}  // namespace

std::string tune_key(const char* kind, uint64_t fingerprint)
{
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    cudaDeviceProp prop{};
    check_cuda(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    std::string name(prop.name);
    std::replace(name.begin(), name.end(), ' ', '_');
    char buf[64];
    std::snprintf(buf, sizeof buf, "%016llx", static_cast<unsigned long long>(fingerprint));
    return std::string(kind) + ":" + buf + "@" + name + "/" + std::to_string(prop.multiProcessorCount);
}

bool tune_cache_get(const std::string& key, std::vector<int>& values)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(key);
    if (it == g_tune.end()) return false;
    values = it->second;
    return true;
}

void tune_cache_put(const std::string& key, const std::vector<int>& values)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[key] = values;
}

float median_of(std::vector<float> v)
{
    if (v.empty()) return 0.0f;
    std::sort(v.begin(), v.end());
    return v[v.size() / 2];
}

}  // namespace sicc

using namespace sicc;

extern "C" {

int sicc_tune_save(const char* path)
{
    try {
        if (!path) throw InvalidArgument("null path");
        std::ofstream f(path);
        if (!f) throw InvalidArgument(std::string("cannot write ") + path);
        std::lock_guard<std::mutex> lock(g_tune_mu);
        for (const auto& kv : g_tune) {
            f << kv.first;
            for (int v : kv.second) f << ' ' << v;
            f << '\n';
        }
        if (!f) throw std::runtime_error(std::string("write failed: ") + path);
        return CUDA_OSD_STATUS_OK;
    } catch (const InvalidArgument& e) {
        set_last_error(e.what());
        return CUDA_OSD_STATUS_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return CUDA_OSD_STATUS_INTERNAL_ERROR;
    }
}

int sicc_tune_load(const char* path)
{
    try {
        if (!path) throw InvalidArgument("null path");
        std::ifstream f(path);
        if (!f) throw InvalidArgument(std::string("cannot read ") + path);
        std::map<std::string, std::vector<int>> fresh;
        std::string line;
        int lineno = 0;
        while (std::getline(f, line)) {
            ++lineno;
            if (line.empty() || line[0] == '#') continue;
            std::istringstream in(line);
            std::string key;
            in >> key;
            std::vector<int> vals;
            long long v = 0;
            while (in >> v) {
                if (v < -1 || v > (1 << 24)) throw InvalidArgument("value out of range on line " + std::to_string(lineno));
                vals.push_back(static_cast<int>(v));
            }
            if (!in.eof() || key.find(':') == std::string::npos || vals.empty())
                throw InvalidArgument("malformed shape cache line " + std::to_string(lineno));
            fresh[key] = vals;
        }
        std::lock_guard<std::mutex> lock(g_tune_mu);
        for (auto& kv : fresh) g_tune[kv.first] = kv.second;
        return CUDA_OSD_STATUS_OK;
    } catch (const InvalidArgument& e) {
        set_last_error(e.what());
        return CUDA_OSD_STATUS_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return CUDA_OSD_STATUS_INTERNAL_ERROR;
    }
}

int sicc_tune_clear(void)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.clear();
    return CUDA_OSD_STATUS_OK;
}

int sicc_tune_entries(void)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    return static_cast<int>(g_tune.size());
}

}  // extern "C"
