// tunecache.h - host helpers of the autotuner's JSON cache (tuning.cu: tile
// shapes, batch.cu: batch schedules): the device's name, a 64-bit FNV-1a hash
// for the batch's signature, whole-file reads, and the device check.
#pragma once

#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <string>

namespace mhd {

// the current device's name ("" without a device)
inline std::string tune_device_name()
{
    int dev = 0;
    cudaDeviceProp p;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
        cudaGetLastError();
        return std::string();
    }
    std::string s(p.name);
    for (char &c : s)
        if (c == '"' || c == '\\') c = '_';
    return s;
}

struct Fnv64 {
    unsigned long long h = 1469598103934665603ull;
    void add(long long v)
    {
        for (int i = 0; i < 8; ++i) {
            h ^= (unsigned long long)((v >> (8 * i)) & 0xff);
            h *= 1099511628211ull;
        }
    }
};

// the file's contents, or false
inline bool read_text(const char *path, std::string &out)
{
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    char buf[4096];
    size_t n;
    out.clear();
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
    fclose(f);
    return true;
}

// the value of "key": "..." in a JSON text written by the cache writers
inline bool json_string(const std::string &text, const char *key, std::string &out)
{
    const std::string k = std::string("\"") + key + "\"";
    size_t p = text.find(k);
    if (p == std::string::npos) return false;
    p = text.find(':', p + k.size());
    if (p == std::string::npos) return false;
    p = text.find('"', p);
    if (p == std::string::npos) return false;
    const size_t e = text.find('"', p + 1);
    if (e == std::string::npos) return false;
    out = text.substr(p + 1, e - p - 1);
    return true;
}

// a cache entry applies when it was recorded on a device of the same name
// (or either name is unknown)
inline bool same_device(const std::string &file_dev, const std::string &dev)
{
    return file_dev.empty() || dev.empty() || file_dev == dev;
}

}  // namespace mhd
