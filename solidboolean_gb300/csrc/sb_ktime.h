// Optional per-kernel device timing. When enabled (sb_kernel_timing), a KTime scope records a CUDA event
// pair on the launching stream around one kernel launch; sb_kernel_timing_read sums them per kernel name.
#pragma once
#include <cuda_runtime.h>

namespace sbg {
bool ktime_enabled();
int ktime_begin(const char *name, cudaStream_t s); // returns a record id or -1
void ktime_end(int id, cudaStream_t s);

struct KTime {
    int id;
    cudaStream_t s;
    KTime(const char *name, cudaStream_t st) : id(ktime_enabled() ? ktime_begin(name, st) : -1), s(st) {}
    ~KTime()
    {
        if (id >= 0)
            ktime_end(id, s);
    }
};
} // namespace sbg
