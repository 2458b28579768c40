// Device hash tables keyed by 64-bit values: open addressing, linear probing, power-of-two capacity. A slot
// is claimed by CAS on its key; the value keeps the minimum inserted (the "first owner" of the key when the
// values are indices in the order the reference inserts them).
#pragma once
#include "sb_common.cuh"

namespace sbg {

constexpr uint64_t kEmpty64 = ~0ull;

// directed edge (a -> b) of a triangle, as a table key
SB_HD uint64_t he_key(uint32_t a, uint32_t b) { return ((uint64_t)a << 32) | b; }

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t slot_of(uint64_t h, uint32_t mask) { return (uint32_t)(mix64(h) & mask); }

// map key -> min(value)
__device__ __forceinline__ void u64map_insert_min(uint64_t *keys, int *vals, uint32_t mask, uint64_t key, int val)
{
    uint32_t s = slot_of(key, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const uint64_t prev = atomicCAS((unsigned long long *)(keys + s), (unsigned long long)kEmpty64,
                                        (unsigned long long)key);
        if (prev == kEmpty64 || prev == key) {
            atomicMin(vals + s, val);
            return;
        }
        s = (s + 1) & mask;
    }
}

// map key -> min(value), returning the key's slot (-1 when the table is full)
__device__ __forceinline__ int u64map_insert_min_slot(uint64_t *keys, int *vals, uint32_t mask, uint64_t key,
                                                      int val)
{
    uint32_t s = slot_of(key, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const uint64_t prev = atomicCAS((unsigned long long *)(keys + s), (unsigned long long)kEmpty64,
                                        (unsigned long long)key);
        if (prev == kEmpty64 || prev == key) {
            atomicMin(vals + s, val);
            return (int)s;
        }
        s = (s + 1) & mask;
    }
    return -1;
}

// value of key, or -1
__device__ __forceinline__ int u64map_find(const uint64_t *keys, const int *vals, uint32_t mask, uint64_t key)
{
    uint32_t s = slot_of(key, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const uint64_t k = keys[s];
        if (k == key)
            return vals[s];
        if (k == kEmpty64)
            return -1;
        s = (s + 1) & mask;
    }
    return -1;
}
#endif

} // namespace sbg
