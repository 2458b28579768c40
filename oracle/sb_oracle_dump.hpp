// Named-array container behind the sbo_* dump interface (sb_oracle.h). Test infrastructure only.
#pragma once
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace sbo {
struct Dump {
    std::map<std::string, std::vector<int64_t>> i64;
    std::map<std::string, std::vector<double>> f64;
};
} // namespace sbo

#define SBO_DUMP_ACCESSORS                                                                          \
    extern "C" long sbo_len(void *h, const char *name)                                              \
    {                                                                                               \
        auto *d = static_cast<sbo::Dump *>(h);                                                      \
        auto a = d->i64.find(name);                                                                 \
        if (a != d->i64.end())                                                                      \
            return (long)a->second.size();                                                          \
        auto b = d->f64.find(name);                                                                 \
        if (b != d->f64.end())                                                                      \
            return (long)b->second.size();                                                          \
        return -1;                                                                                  \
    }                                                                                               \
    extern "C" int sbo_get_i64(void *h, const char *name, int64_t *out)                             \
    {                                                                                               \
        auto *d = static_cast<sbo::Dump *>(h);                                                      \
        auto a = d->i64.find(name);                                                                 \
        if (a == d->i64.end())                                                                      \
            return -1;                                                                              \
        if (!a->second.empty())                                                                     \
            std::memcpy(out, a->second.data(), a->second.size() * sizeof(int64_t));                 \
        return 0;                                                                                   \
    }                                                                                               \
    extern "C" int sbo_get_f64(void *h, const char *name, double *out)                              \
    {                                                                                               \
        auto *d = static_cast<sbo::Dump *>(h);                                                      \
        auto a = d->f64.find(name);                                                                 \
        if (a == d->f64.end())                                                                      \
            return -1;                                                                              \
        if (!a->second.empty())                                                                     \
            std::memcpy(out, a->second.data(), a->second.size() * sizeof(double));                  \
        return 0;                                                                                   \
    }                                                                                               \
    extern "C" void sbo_free(void *h) { delete static_cast<sbo::Dump *>(h); }
