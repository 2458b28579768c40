// Shared device/host definitions for the GB300 mesh-boolean kernels.
//
// Every floating-point expression that decides topology or produces an output coordinate is written with
// the same operations, in the same order, as the reference's FP64 CPU code, and every .cu file is built
// with -fmad=false, so that no multiply-add is contracted and results are bit-identical to the
// reference compiled without FMA.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

#define SB_HD __host__ __device__ __forceinline__
#define SB_HDF __host__ __device__

namespace sbg {

constexpr double kDblEps = DBL_EPSILON;
constexpr double kDblMax = DBL_MAX;

struct d3 {
    double x, y, z;
};
SB_HD d3 mk(double x, double y, double z) { return d3{x, y, z}; }
SB_HD d3 operator+(d3 a, d3 b) { return d3{a.x + b.x, a.y + b.y, a.z + b.z}; }
SB_HD d3 operator-(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
SB_HD d3 neg(d3 a) { return d3{-a.x, -a.y, -a.z}; }
SB_HD d3 scale(double s, d3 a) { return d3{s * a.x, s * a.y, s * a.z}; }
SB_HD d3 divs(d3 a, double d) { return d3{a.x / d, a.y / d, a.z / d}; }
// (a.x*b.x + a.y*b.y) + a.z*b.z, left to right (vector3.h:150-153)
SB_HD double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// vector3.h:143-148
SB_HD d3 cross(d3 a, d3 b) { return d3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
SB_HD double comp(d3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// unit normal of triangle (a, b, c); zero vector when |cross| <= DBL_EPSILON (vector3.h:155-176)
SB_HD d3 unit_normal(d3 a, d3 b, d3 c)
{
    double bax = b.x - a.x, bay = b.y - a.y, baz = b.z - a.z;
    double cax = c.x - a.x, cay = c.y - a.y, caz = c.z - a.z;
    double nx = bay * caz - baz * cay;
    double ny = baz * cax - bax * caz;
    double nz = bax * cay - bay * cax;
    double len = sqrt(nx * nx + ny * ny + nz * nz);
    if (fabs(len) <= kDblEps)
        return d3{0.0, 0.0, 0.0};
    return d3{nx / len, ny / len, nz / len};
}
// vector3.h:119-128
SB_HD d3 normalized(d3 v)
{
    double len = sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    if (fabs(len) <= kDblEps)
        return d3{0.0, 0.0, 0.0};
    return d3{v.x / len, v.y / len, v.z / len};
}

struct d2 {
    double x, y;
};

// Quantised weld key: (long)(c * factor) per coordinate, truncation toward zero (positionkey.cpp:32-37).
struct Key {
    long long x, y, z;
};
SB_HD Key make_key(d3 p, double factor)
{
    return Key{(long long)(p.x * factor), (long long)(p.y * factor), (long long)(p.z * factor)};
}
SB_HD bool key_eq(const Key &a, const Key &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
SB_HD bool key_lt(const Key &a, const Key &b)
{
    if (a.x != b.x)
        return a.x < b.x;
    if (a.y != b.y)
        return a.y < b.y;
    return a.z < b.z;
}
SB_HD uint64_t key_hash(const Key &k)
{
    uint64_t h = (uint64_t)k.x * 0x9E3779B97F4A7C15ull;
    h ^= (uint64_t)k.y + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
    h ^= (uint64_t)k.z + 0x94D049BB133111EBull + (h << 6) + (h >> 2);
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    return h;
}

SB_HD uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------------------------------------------
// Iteration order of libstdc++'s std::unordered_{set,map}<size_t, ...> (identity hash, unique keys,
// max load factor 1, default-constructed, single-element inserts). The reference walks such containers
// to pick polyline starts, inner-loop starts and neighbour preference, so the order is reproduced:
//   * nodes form one singly linked list; each bucket remembers the node *before* its first node;
//   * a key whose bucket is non-empty is linked right after that "before" node;
//   * a key whose bucket is empty is linked at the list head (the old head's bucket then points at it);
//   * when the element count would exceed the bucket count the table is rebuilt by walking the old list
//     and applying the same two rules with the new bucket count.
// Bucket counts after the first insert follow the library's prime schedule below (measured, not derived).
// ---------------------------------------------------------------------------------------------------
__host__ __device__ inline uint32_t hash_bucket_count(uint32_t elements)
{
    // bucket count held while the table has `elements` elements (elements >= 1)
    const uint32_t sched[] = {13u,     29u,     59u,      127u,     257u,     541u,      1109u,
                              2357u,   5087u,   10273u,   20753u,   42043u,   85229u,    172933u,
                              351061u, 712697u, 1447153u, 2938679u, 5967347u, 12117689u, 24607243u,
                              49969847u};
    for (int i = 0; i < (int)(sizeof(sched) / sizeof(sched[0])); ++i)
        if (elements <= sched[i])
            return sched[i];
    return 0xFFFFFFFFu;
}

// Orders `n` distinct keys inserted in sequence `keys[0..n)` the way the library iterates them.
// next[] and bucket[] are caller scratch: next has n entries, bucket has hash_bucket_count(n) entries.
// Writes the iteration order (as positions into keys[]) to order[0..n).
__host__ __device__ inline void hash_iteration_order(const uint64_t *keys, int n, int *next, int *bucket,
                                                     int *order)
{
    const int HEAD = -2, EMPTY = -1;
    int head = -1;
    uint32_t bc = 0;
    for (int i = 0; i < n; ++i) {
        uint32_t want = hash_bucket_count((uint32_t)(i + 1));
        if (want != bc) {
            // rebuild with the new bucket count, walking the old list
            for (uint32_t b = 0; b < want; ++b)
                bucket[b] = EMPTY;
            int p = head;
            head = -1;
            uint32_t beginBkt = 0;
            while (p >= 0) {
                int nx = next[p];
                uint32_t b = (uint32_t)(keys[p] % want);
                if (bucket[b] == EMPTY) {
                    next[p] = head;
                    head = p;
                    bucket[b] = HEAD;
                    if (next[p] >= 0)
                        bucket[beginBkt] = p;
                    beginBkt = b;
                } else {
                    int bf = bucket[b];
                    if (bf == HEAD) {
                        next[p] = head;
                        head = p;
                    } else {
                        next[p] = next[bf];
                        next[bf] = p;
                    }
                }
                p = nx;
            }
            bc = want;
        }
        uint32_t b = (uint32_t)(keys[i] % bc);
        int bf = bucket[b];
        if (bf != EMPTY) {
            if (bf == HEAD) {
                next[i] = head;
                head = i;
            } else {
                next[i] = next[bf];
                next[bf] = i;
            }
        } else {
            next[i] = head;
            if (head >= 0)
                bucket[(uint32_t)(keys[head] % bc)] = i;
            head = i;
            bucket[b] = HEAD;
        }
    }
    int k = 0;
    for (int p = head; p >= 0; p = next[p])
        order[k++] = p;
}

SB_HD uint64_t dbl_bits(double x)
{
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
}
SB_HD double bits_dbl(uint64_t u)
{
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
}

// x / 3 rounded to nearest (ties to even), in integer arithmetic. With x = m 2^e (m the 53-bit significand),
// N = m 2^11 lies in [2^63, 2^64); q = N / 3 and r = N mod 3 give the exact quotient q + r/3, which has 62
// or 63 bits; keeping 53 of them and rounding on the dropped bits plus the sticky remainder is the IEEE
// result. Inputs whose quotient would leave the normal range, infinities and NaNs use the hardware divide.
SB_HD double div3_rn(double x)
{
    const uint64_t u = dbl_bits(x);
    const int E = (int)((u >> 52) & 0x7FF);
    if (E < 3 || E == 0x7FF) {
        if ((u << 1) == 0)
            return x; // +-0
        return x / 3.0;
    }
    const uint64_t N = ((u & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 11;
    const uint64_t q = N / 3, r = N - 3 * q;
    const int sh = (q >> 62) ? 10 : 9;
    uint64_t mant = q >> sh;
    const uint64_t rem = q & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (r != 0 || (mant & 1))))
        ++mant;
    int Er = E - 11 + sh;
    if (mant >> 53) {
        mant >>= 1;
        ++Er;
    }
    return bits_dbl((u & 0x8000000000000000ull) | ((uint64_t)Er << 52) | (mant & 0xFFFFFFFFFFFFFull));
}

#ifdef __CUDACC__
// order-preserving map from double to uint64 (for integer min/max of doubles)
__device__ __forceinline__ uint64_t dbl_to_ord(double d)
{
    uint64_t u = (uint64_t)__double_as_longlong(d);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_to_dbl(uint64_t u)
{
    u = (u & 0x8000000000000000ull) ? (u & 0x7FFFFFFFFFFFFFFFull) : ~u;
    return __longlong_as_double((long long)u);
}
#endif

} // namespace sbg

namespace sbg {
// every kernel launch of this library goes through SB_COUNT so the number of launches can be reported
void count_launch();
} // namespace sbg
#define SB_COUNT(kernel) (::sbg::count_launch(), &kernel)

#define SB_CUDA_CHECK(expr)                                                                               \
    do {                                                                                                     \
        cudaError_t _e = (expr);                                                                             \
        if (_e != cudaSuccess)                                                                               \
            return sbg::cuda_fail(_e, #expr, __FILE__, __LINE__);                                            \
    } while (0)
