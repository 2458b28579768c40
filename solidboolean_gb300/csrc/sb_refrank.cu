// Leaf order of the reference's AABB tree, built on the GPU.
//
// The reference's candidate pairs reach each cut face in the order of its tree traversal, and that order
// numbers the face's cut points (src/solidboolean.cpp:315-341), which in turn decides where closed inner
// loops start and so how they are ear-clipped, which point of a weld class survives, and whether a face
// fails. For a fixed first-mesh triangle the dual traversal (src/axisalignedboundingboxtree.h:54-88)
// visits second-mesh leaves in that tree's left-to-right order (a split of the first tree never reorders
// the second), and inside a leaf pair in the leaf's stored order. So the per-face order is the position of
// the other triangle in the other mesh's leaf order, which is what this file computes.
//
// The tree (src/axisalignedboundingboxtree.cpp:27-45, 71-141; root box and member list from
// src/solidmesh.cpp:57-76): a node with more than 20 boxes splits on the longest axis of its box (spans
// compared as float, first maximum wins) at the mean of its box centres (sequential sum in member order
// divided by (float)count); boxes with centre < mean go left in reverse order of appearance, the others right
// in order; an empty side takes half of the other.
//
// Two facts shape the GPU build:
//  * A child's member list is a subsequence of its parent's, kept in order or reversed. The root lists the
//    triangles by index, so every node lists its members by ascending or by descending triangle index: one
//    direction bit per node describes the order, and the large-node phase moves no data at all.
//  * The mean is needed exactly only through the comparisons centre < mean. Each node's centre sum is kept
//    exactly in 64-bit fixed point (every centre truncated to a common power-of-two grid); with the
//    recursive-summation bound this gives an interval that contains the reference's sequential mean. A
//    member outside the interval is classified with one integer comparison of order-preserving keys; a node
//    with a member inside it recomputes the sequential sum in member order. No per-member FP64 arithmetic
//    remains, which matters on a part whose FP64 rate is a small fraction of its integer rate.
//
// Phases: nodes with more than kSub members split level by level over all triangles (classify, rare exact
// resolution, children), visiting the triangles in the LBVH's Morton order so that a node's members form
// long runs for the reductions; one radix sort then lists each remaining node's members in order, and one
// block per such node finishes its subtree in shared memory and writes the final positions.
#include <algorithm>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <vector>

#include <cub/cub.cuh>

#include "sb_common.cuh"
#include "sb_internal.h"
#include "sb_ktime.h"

namespace sbg {

constexpr int kLeaf = 20;        // reference leaf size (src/axisalignedboundingboxtree.cpp:25)
constexpr int kSub = 1024;       // nodes with at most this many members finish in one block
constexpr int kSubThreads = 256;
constexpr int kSubNodes = 272;   // node records per subtree block (shared memory)

// counters[] slots
enum {
    kCtNodes = 0,   // node records allocated
    kCtTerms = 1,   // terminal nodes listed
    kCtOverflow = 2,
    kCtFirst = 4,   // current level: first node
    kCtLast = 5,    //                one past the last node
    kCtSubErr = 6,  // subtree blocks that ran out of node records
    kCtTNodes = 7,  // node-table records allocated (subtree nodes are numbered from maxNodes up)
    kCtCount = 8
};

// One triangle in integer form, stored by Morton position: order-preserving keys of its box centre and box
// (centres compare with one integer comparison, boxes reduce with integer min/max; ord_to_dbl recovers the
// exact doubles) and the fixed-point centre that node sums add up. 96 bytes, three sectors.
struct RRec {
    unsigned long long c[3];
    unsigned long long lo[3], hi[3];
    long long fx[3];
};

// box (order-preserving keys) and fixed-point centre sum of a set of members
struct RStat {
    unsigned long long lo[3], hi[3];
    long long sum[3];
    int count, pad;
};

struct RNode {
    int begin, count;  // begin: position of the node's first member in the final leaf order
    int dir;           // member order: 0 ascending triangle index, 1 descending
    int flags;         // bit 0: a member fell inside the interval
    int mode, pad[3];  // 0 regular split, 1 left side was empty, 2 right side was empty
    RStat st;          // the node's own members
    RStat acc[2];      // left / right members, accumulated while classifying
};

// what the per-member passes read of a node, in one 32-byte sector
struct NParam {
    int child;         // left child id (right = child + 1), -1 while unsplit or terminal
    int count, axis, pad;
    unsigned long long clo, chi; // order-preserving keys of an interval holding the reference's split value
};

// per-member state word: node id << 2 | tag, tag 0 settled in that node, 1 / 2 pending move to its left /
// right child, 3 inside the node's interval (rewritten by the exact resolution)
__device__ __forceinline__ int st_node(int v) { return v >> 2; }
__device__ __forceinline__ int st_tag(int v) { return v & 3; }

// order-preserving key of a double with -0 folded onto +0 (they compare equal)
__device__ __forceinline__ unsigned long long ordc(double d)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(d);
    if (u == 0x8000000000000000ull)
        u = 0;
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

// x truncated toward zero onto the grid 2^-sc, as an integer (|x| 2^sc stays below 2^62 by the choice of sc)
__device__ __forceinline__ long long to_fixed(double x, int sc)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    int E = (int)((u >> 52) & 0x7FF);
    unsigned long long m = (u & 0xFFFFFFFFFFFFFull) | (E ? (1ull << 52) : 0ull);
    int shift = (E ? E : 1) - 1075 + sc;
    unsigned long long v;
    if (shift >= 0)
        v = m << (shift < 10 ? shift : 10);
    else
        v = (-shift >= 64) ? 0ull : (m >> (-shift));
    return (u >> 63) ? -(long long)v : (long long)v;
}

// 2^-sc for sc in [-1000, 1000]
__device__ __forceinline__ double pow2_neg(int sc)
{
    return __longlong_as_double((long long)(1023 - sc) << 52);
}

// grid exponent of one axis: |c| 2^sc < 2^(62 - bits(nt)), so that any sum of members fits in 62 bits
__device__ __forceinline__ int fixed_scale(double M, int nt)
{
    int B = 62 - (32 - __clz(nt));
    unsigned long long u = (unsigned long long)__double_as_longlong(M);
    int E = (int)((u >> 52) & 0x7FF);
    int e = E ? E - 1023 : -1023;
    int sc = B - 1 - e;
    return sc < -1000 ? -1000 : (sc > 1000 ? 1000 : sc);
}

// gamma_n = n u / (1 - n u), rounded up
__device__ __forceinline__ double rr_gamma(int n)
{
    const double u = 1.1102230246251565e-16;
    double nu = __dmul_ru((double)n, u);
    return __ddiv_ru(nu, __dsub_rd(1.0, nu));
}

__device__ __forceinline__ void rstat_clear(RStat &s)
{
    for (int k = 0; k < 3; ++k) {
        s.lo[k] = ~0ull;
        s.hi[k] = 0ull;
        s.sum[k] = 0;
    }
    s.count = 0;
    s.pad = 0;
}

// Split axis and interval of a node from its box and exact fixed-point sum. The reference's sequential sum s
// satisfies |s - sum c| <= gamma_n sum|c| <= gamma_n n M (M bounds |c| through the box, with a margin for
// the centre's own rounding); the fixed-point sum is within n 2^-sc of sum c; division by (float)count is
// monotone, so rounding the ends outward gives an interval that holds the reference's split value.
__device__ void node_params(const unsigned long long *lo, const unsigned long long *hi, const long long *sum,
                            int count, const int *sc, int &axis, unsigned long long &clo, unsigned long long &chi)
{
    float span[3];
    for (int k = 0; k < 3; ++k)
        span[k] = __double2float_rn(ord_to_dbl(hi[k]) - ord_to_dbl(lo[k]));
    axis = 0;
    for (int k = 1; k < 3; ++k)
        if (span[axis] < span[k])
            axis = k;
    const double M = fmax(fabs(ord_to_dbl(lo[axis])), fabs(ord_to_dbl(hi[axis])));
    const double p2 = pow2_neg(sc[axis]);
    const double n = (double)count;
    double delta = __dmul_ru(__dmul_ru(rr_gamma(count), n), __dmul_ru(M, 1.000001));
    delta = __dadd_ru(delta, __dmul_ru(n, p2));
    const double slo = __dmul_rd(__ll2double_rd(sum[axis]), p2);
    const double shi = __dmul_ru(__ll2double_ru(sum[axis]), p2);
    const double cnt = (double)(float)count;
    clo = ordc(__ddiv_rd(__dsub_rd(slo, delta), cnt));
    chi = ordc(__ddiv_ru(__dadd_ru(shi, delta), cnt));
}

// per-member statistics in integer form
struct EStat {
    unsigned long long lo[3], hi[3];
    long long s[3];
};

__device__ __forceinline__ EStat estat_of(bool valid, const RRec &r)
{
    EStat e;
    for (int k = 0; k < 3; ++k) {
        e.lo[k] = valid ? r.lo[k] : ~0ull;
        e.hi[k] = valid ? r.hi[k] : 0ull;
        e.s[k] = valid ? r.fx[k] : 0;
    }
    return e;
}

__device__ __forceinline__ void estat_merge(EStat &a, const EStat &b)
{
    for (int k = 0; k < 3; ++k) {
        a.lo[k] = min(a.lo[k], b.lo[k]);
        a.hi[k] = max(a.hi[k], b.hi[k]);
        a.s[k] += b.s[k];
    }
}

// Segmented inclusive reduction over runs of equal `key` among the 32 lanes; `len` is an int payload summed
// alongside (1 per member on entry). Returns true on the last lane of each run, which then holds the run's
// total. All 32 lanes must call it.
__device__ __forceinline__ bool warp_segment_reduce(int key, EStat &r, int &len)
{
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const int prevKey = __shfl_up_sync(full, key, 1);
    int head = (lane == 0 || prevKey != key) ? lane : 0;
    for (int o = 1; o < 32; o <<= 1) {
        int h = __shfl_up_sync(full, head, o);
        if (lane >= o)
            head = max(head, h);
    }
    for (int o = 1; o < 32; o <<= 1) {
        EStat t;
        for (int k = 0; k < 3; ++k) {
            t.lo[k] = __shfl_up_sync(full, r.lo[k], o);
            t.hi[k] = __shfl_up_sync(full, r.hi[k], o);
            t.s[k] = __shfl_up_sync(full, r.s[k], o);
        }
        const int tl = __shfl_up_sync(full, len, o);
        if (lane - o >= head) {
            estat_merge(r, t);
            len += tl;
        }
    }
    const int nextKey = __shfl_down_sync(full, key, 1);
    return lane == 31 || nextKey != key;
}

// Reduction of a whole warp whose 32 lanes share one key, with the warp reduction instructions on 32-bit
// words: a 64-bit minimum is the minimum high word, then the minimum low word among the lanes holding it (the
// maximum likewise); a fixed-point sum is summed as its signed high word and two 16-bit pieces of its low word
// (each member's |sum| is below 2^(62 - bits(nt)) with nt > 1024, so every partial sum fits its 32 bits). All
// lanes receive the totals. All 32 lanes must call it.
__device__ __forceinline__ void warp_uniform_reduce(EStat &e, int &len)
{
    const unsigned full = 0xFFFFFFFFu;
    for (int k = 0; k < 3; ++k) {
        const unsigned lh = (unsigned)(e.lo[k] >> 32), hh = (unsigned)(e.hi[k] >> 32);
        const unsigned mlh = __reduce_min_sync(full, lh), mhh = __reduce_max_sync(full, hh);
        const unsigned mll = __reduce_min_sync(full, lh == mlh ? (unsigned)e.lo[k] : 0xFFFFFFFFu);
        const unsigned mhl = __reduce_max_sync(full, hh == mhh ? (unsigned)e.hi[k] : 0u);
        e.lo[k] = ((unsigned long long)mlh << 32) | mll;
        e.hi[k] = ((unsigned long long)mhh << 32) | mhl;
        const unsigned long long u = (unsigned long long)e.s[k];
        const int sh = __reduce_add_sync(full, (int)(unsigned)(u >> 32));
        const unsigned s1 = __reduce_add_sync(full, (unsigned)(u >> 16) & 0xFFFFu);
        const unsigned s0 = __reduce_add_sync(full, (unsigned)u & 0xFFFFu);
        e.s[k] = (long long)(((unsigned long long)(long long)sh << 32) + ((unsigned long long)s1 << 16) +
                             (unsigned long long)s0);
    }
    len = (int)__reduce_add_sync(full, (unsigned)len);
}

// Segmented inclusive scan over the 32 lanes: a lane with `start` set begins a new segment (lane 0 must).
__device__ __forceinline__ void warp_segmented_scan(bool start, EStat &r)
{
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    int head = start ? lane : 0;
    for (int o = 1; o < 32; o <<= 1) {
        const int h = __shfl_up_sync(full, head, o);
        if (lane >= o)
            head = max(head, h);
    }
    for (int o = 1; o < 32; o <<= 1) {
        EStat t;
        for (int k = 0; k < 3; ++k) {
            t.lo[k] = __shfl_up_sync(full, r.lo[k], o);
            t.hi[k] = __shfl_up_sync(full, r.hi[k], o);
            t.s[k] = __shfl_up_sync(full, r.s[k], o);
        }
        if (lane - o >= head)
            estat_merge(r, t);
    }
}

// Merges a run's box and sum into an accumulator (global or shared); sums add as two's complement. The
// results are unused, so on global memory these are fire-and-forget reductions.
__device__ __forceinline__ void stat_atomic(RStat &dst, const EStat &e, int len)
{
    for (int k = 0; k < 3; ++k) {
        atomicMin(&dst.lo[k], e.lo[k]);
        atomicMax(&dst.hi[k], e.hi[k]);
        atomicAdd(reinterpret_cast<unsigned long long *>(&dst.sum[k]), (unsigned long long)e.s[k]);
    }
    atomicAdd(&dst.count, len);
}

// Groups the warp's lanes by key (bitonic sort of (key, lane) over the 32 lanes, then every lane fetches the
// statistics of the lane it now stands for) and reduces each group: afterwards the last lane of each group
// holds the group's total, its key in `key` and its member count in `len`, and the function returns true
// there. Keys may arrive in any order. All 32 lanes must call it.
__device__ __forceinline__ bool warp_group_reduce(int &key, EStat &e, int &len)
{
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    int k = key, src = lane;
    for (int size = 2; size <= 32; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const int ok = __shfl_xor_sync(full, k, stride);
            const int os = __shfl_xor_sync(full, src, stride);
            const bool ascending = (lane & size) == 0 || size == 32;
            const bool lower = (lane & stride) == 0;
            const bool mineFirst = k < ok || (k == ok && src < os);
            if (mineFirst != (lower == ascending)) {
                k = ok;
                src = os;
            }
        }
    EStat g;
    for (int q = 0; q < 3; ++q) {
        g.lo[q] = __shfl_sync(full, e.lo[q], src);
        g.hi[q] = __shfl_sync(full, e.hi[q], src);
        g.s[q] = __shfl_sync(full, e.s[q], src);
    }
    int l = __shfl_sync(full, len, src);
    const bool tail = warp_segment_reduce(k, g, l);
    key = k;
    e = g;
    len = l;
    return tail;
}

// Warp reduction by key: when the keys already arrive in a few runs (the usual case in Morton order) a
// segmented reduction suffices; a warp with many key changes groups its lanes first. Returns true on the
// lane holding a group's total (its key in `key`, its member count in `len`).
__device__ __forceinline__ bool warp_reduce_by_key(int &key, EStat &e, int &len)
{
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(0xFFFFFFFFu, key, 1);
    const unsigned changes = __ballot_sync(0xFFFFFFFFu, lane > 0 && prev != key);
    if (__popc(changes) > 3)
        return warp_group_reduce(key, e, len);
    return warp_segment_reduce(key, e, len);
}

// Block-level reduce-by-key. Every warp's group totals are compacted, in lane order, into shared memory;
// warp 0 merges neighbouring entries of equal key and issues one accumulator update per merged run.
// Entries past the shared capacity update their accumulator directly. All threads of the block must call
// it; `target(key)` names the accumulator of a key. There is no barrier at the end: the next call's first
// barrier orders the reuse of `runs`, and a caller that reads a shared target must synchronise first.
constexpr int kRunCap = 64;
struct RunRec {
    int key, len;
    EStat e;
};

__device__ __forceinline__ void estat_neutral(EStat &e)
{
    for (int q = 0; q < 3; ++q) {
        e.lo[q] = ~0ull;
        e.hi[q] = 0ull;
        e.s[q] = 0;
    }
}

template <class Target>
__device__ __forceinline__ void block_reduce_keys(int key, EStat e, int len, RunRec *runs, int *warpRuns,
                                                  Target target)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const bool mine = warp_reduce_by_key(key, e, len) && key >= 0;
    const unsigned bal = __ballot_sync(0xFFFFFFFFu, mine);
    if (lane == 0)
        warpRuns[w] = __popc(bal);
    __syncthreads();
    int off = 0, total = 0;
    for (int i = 0; i < nw; ++i) {
        const int c = warpRuns[i];
        off += i < w ? c : 0;
        total += c;
    }
    const int idx = off + __popc(bal & ((1u << lane) - 1u));
    if (mine) {
        if (idx < kRunCap) {
            runs[idx].key = key;
            runs[idx].len = len;
            runs[idx].e = e;
        } else {
            stat_atomic(target(key), e, len);
        }
    }
    __syncthreads();
    if (w == 0) {
        const int nr = total < kRunCap ? total : kRunCap;
        for (int b = 0; b < nr; b += 32) {
            const int j = b + lane;
            const bool v = j < nr;
            int k2 = v ? runs[j].key : -1;
            int l2 = v ? runs[j].len : 0;
            EStat e2;
            if (v)
                e2 = runs[j].e;
            else
                estat_neutral(e2);
            if (warp_segment_reduce(k2, e2, l2) && k2 >= 0)
                stat_atomic(target(k2), e2, l2);
        }
    }
}

// block-wide exclusive scan of one int per thread (blockDim.x a multiple of 32, at most 1024)
__device__ __forceinline__ int block_exclusive_scan(int v, int &total, int *warpSums)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o)
            incl += t;
    }
    if (lane == 31)
        warpSums[w] = incl;
    __syncthreads();
    int off = 0, tot = 0;
    for (int i = 0; i < nw; ++i) {
        int s = warpSums[i];
        off += i < w ? s : 0;
        tot += s;
    }
    __syncthreads();
    total = tot;
    return off + incl - v;
}

// ---------------------------------------------------------------------------------------------------
// Root: records, box, grid exponents, fixed-point sum, split parameters
// ---------------------------------------------------------------------------------------------------
constexpr int kElemThreads = 256; // block size of the per-member passes

__device__ __forceinline__ void node_clear(RNode &r, int begin, int count, int dir)
{
    r.begin = begin;
    r.count = count;
    r.dir = dir;
    r.flags = 0;
    r.mode = 0;
    r.pad[0] = r.pad[1] = r.pad[2] = 0;
    rstat_clear(r.st);
    rstat_clear(r.acc[0]);
    rstat_clear(r.acc[1]);
    r.st.count = count;
}

__global__ void k_rr_init(RNode *nodes, NParam *np, int nt, int *counters, unsigned *bar)
{
    bar[0] = bar[1] = bar[2] = bar[3] = 0;
    node_clear(nodes[0], 0, nt, 0);
    np[0] = NParam{-1, nt, 0, 0, 0ull, 0ull};
    for (int i = 0; i < kCtCount; ++i)
        counters[i] = 0;
    counters[kCtNodes] = 1;
}

// Split parameters of the root (or the root listed as a terminal node when it is small), from its box and
// fixed-point sum.
__device__ void root_params(RNode *nodes, NParam *np, int nt, const int *sc, int *counters, int *terms)
{
    if (nt > kSub) {
        unsigned long long lo[3], hi[3];
        long long sum[3];
        for (int k = 0; k < 3; ++k) { // other blocks' atomics: read through L2
            lo[k] = __ldcg(&nodes[0].st.lo[k]);
            hi[k] = __ldcg(&nodes[0].st.hi[k]);
            sum[k] = __ldcg(&nodes[0].st.sum[k]);
        }
        NParam q{-1, nt, 0, 0, 0ull, 0ull};
        node_params(lo, hi, sum, nt, sc, q.axis, q.clo, q.chi);
        np[0] = q;
        counters[kCtFirst] = 0;
        counters[kCtLast] = 1;
    } else {
        terms[0] = 0;
        counters[kCtTerms] = 1;
        counters[kCtFirst] = 1;
        counters[kCtLast] = 1;
    }
}

// Box centre of each triangle as AxisAlignedBoudingBox::updateCenter computes it, (((0 + v0) + v1) + v2) /
// (float)3 (src/axisalignedboundingbox.h:31-53), its box, its fixed-point centre, and the root's box and
// fixed-point sum (src/solidmesh.cpp:68-72); the last block to finish computes the root's split parameters.
// Records are stored in Morton order (position p holds triangle leafTri[p]): member order is carried by the
// direction bits, so the processing order is free, and in Morton order a node's members form long runs.
// The fixed-point grid of each axis comes from an upper bound of the coordinates' magnitude (absMax: the
// triangle boxes' largest |coordinate|, rounded up to FP32, from the preparation's box pass) rather than
// from the root box, so that no second pass over the members waits for the root box. Any grid that keeps
// the sums in range gives the same leaf order: the fixed-point sums only bound the reference's mean, and
// members inside the bound are resolved exactly.
__global__ void __launch_bounds__(kElemThreads) k_rr_elems(int nt, const double *__restrict__ v,
                                                           const uint32_t *__restrict__ t,
                                                           const double *__restrict__ box64,
                                                           const int *__restrict__ leafTri, RRec *rec,
                                                           unsigned long long *soa, int *posOf, int *state,
                                                           RNode *nodes, NParam *np, int *counters, int *terms,
                                                           int *scg, const unsigned int *__restrict__ absMax,
                                                           unsigned int *ticket)
{
    __shared__ unsigned long long sLo[3], sHi[3];
    __shared__ long long sSum[3];
    __shared__ int sc[3];
    __shared__ bool lastBlock;
    if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        sLo[a] = ~0ull;
        sHi[a] = 0ull;
        sSum[a] = 0;
        sc[a] = fixed_scale((double)__uint_as_float(absMax[a]), nt);
        if (blockIdx.x == 0)
            scg[a] = sc[a];
    }
    __syncthreads();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    long long fs[3] = {0, 0, 0};
    if (p < nt) {
        const int i = leafTri[p];
        RRec r;
        for (int a = 0; a < 3; ++a) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                s = s + v[3 * (size_t)t[3 * (size_t)i + k] + a];
            const double c = div3_rn(s);
            r.c[a] = ordc(c);
            lo[a] = r.lo[a] = ordc(box64[6 * (size_t)i + a]);
            hi[a] = r.hi[a] = ordc(box64[6 * (size_t)i + 3 + a]);
            fs[a] = r.fx[a] = to_fixed(c, sc[a]);
            soa[(size_t)a * nt + p] = r.c[a];
            soa[(size_t)(3 + a) * nt + p] = r.lo[a];
            soa[(size_t)(6 + a) * nt + p] = r.hi[a];
            soa[(size_t)(9 + a) * nt + p] = (unsigned long long)r.fx[a];
        }
        rec[p] = r;
        posOf[i] = p;
        state[p] = 0;
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int a = 0; a < 3; ++a) {
            lo[a] = min(lo[a], __shfl_xor_sync(0xFFFFFFFFu, lo[a], o));
            hi[a] = max(hi[a], __shfl_xor_sync(0xFFFFFFFFu, hi[a], o));
            fs[a] += __shfl_xor_sync(0xFFFFFFFFu, fs[a], o);
        }
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; ++a) {
            atomicMin(&sLo[a], lo[a]);
            atomicMax(&sHi[a], hi[a]);
            atomicAdd(reinterpret_cast<unsigned long long *>(&sSum[a]), (unsigned long long)fs[a]);
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        atomicMin(&nodes[0].st.lo[a], sLo[a]);
        atomicMax(&nodes[0].st.hi[a], sHi[a]);
        atomicAdd(reinterpret_cast<unsigned long long *>(&nodes[0].st.sum[a]), (unsigned long long)sSum[a]);
        __threadfence(); // the root's statistics are in L2 before this block counts as done
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        lastBlock = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (lastBlock && threadIdx.x == 0) {
        __threadfence();
        root_params(nodes, np, nt, sc, counters, terms);
    }
}

// ---------------------------------------------------------------------------------------------------
// Large-node phase: one persistent cooperative kernel runs every level (classify the members, grid barrier,
// resolve and split the nodes, grid barrier). Data that other blocks write inside the kernel (member states,
// node parameters, accumulators, counters) is read through L2 (ld.global.cg), never from a stale L1 line.
// ---------------------------------------------------------------------------------------------------
struct GridBar {
    unsigned count, gen;
    int err;
    unsigned ticket; // element blocks done (the last one computes the root's split)
};

// bounded wait: a barrier gives up and flags an error after this long (the levels take microseconds)
constexpr unsigned long long kBarrierNs = 200ull * 1000ull * 1000ull;
constexpr int kMaxLevels = 4096;

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for a cooperative launch (every block resident). Returns false once any block gave up
// waiting; the kernel then returns and the host reports the error.
__device__ bool grid_sync(GridBar *gb)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &gb->gen;
        const unsigned g = *vgen;
        __threadfence();
        int good = 1;
        if (atomicAdd(&gb->count, 1u) == gridDim.x - 1) {
            atomicExch(&gb->count, 0u);
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (*vgen == g) {
                if (global_ns() - t0 > kBarrierNs) {
                    atomicExch(&gb->err, 1);
                    good = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok = good && *reinterpret_cast<volatile int *>(&gb->err) == 0;
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ NParam ld_nparam(const NParam *q)
{
    NParam r;
    r.child = __ldcg(&q->child);
    r.count = __ldcg(&q->count);
    r.axis = __ldcg(&q->axis);
    r.pad = 0;
    r.clo = __ldcg(&q->clo);
    r.chi = __ldcg(&q->chi);
    return r;
}

__device__ __forceinline__ RStat ld_rstat(const RStat *a)
{
    RStat r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = __ldcg(&a->lo[k]);
        r.hi[k] = __ldcg(&a->hi[k]);
        r.sum[k] = __ldcg(&a->sum[k]);
    }
    r.count = __ldcg(&a->count);
    r.pad = 0;
    return r;
}

// Node tables of one level in shared memory: the child ids of the previous level's nodes (to move pending
// members) and the split parameters of this level's nodes. Levels with more nodes than fit read them from
// global memory instead.
constexpr int kTabNodes = 1024;
struct LevelTab {
    int child[kTabNodes];
    NParam par[kTabNodes];
};

__device__ __forceinline__ void load_level_tab(LevelTab &tab, const NParam *np, int prevFirst, int first, int last)
{
    if (first - prevFirst <= kTabNodes)
        for (int k = threadIdx.x; k < first - prevFirst; k += blockDim.x)
            tab.child[k] = __ldcg(&np[prevFirst + k].child);
    if (last - first <= kTabNodes)
        for (int k = threadIdx.x; k < last - first; k += blockDim.x)
            tab.par[k] = ld_nparam(&np[first + k]);
    __syncthreads();
}

// One warp walks the contiguous Morton range [wb, we) in chunks of 32 (lane = position, so every field loads
// coalesced from the structure-of-arrays copy): moves members decided at the previous level into their child,
// classifies the members of large nodes against their intervals, and reduces their statistics by key
// (child, side). Keys come in long runs; a run still open at the end of a chunk is carried in lane 0 into the
// next chunk, runs completed inside the range update their accumulators directly, and the run open at the
// end of the range joins one block reduction. All threads of the block must call it.
__device__ __forceinline__ void classify_range(int wb, int we, int prevFirst, int first, int last,
                                               const unsigned long long *__restrict__ soa, int nt, int *state,
                                               const NParam *np, RNode *nodes, RunRec *runs, int *warpRuns,
                                               const LevelTab &tab)
{
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const bool childTab = first - prevFirst <= kTabNodes, parTab = last - first <= kTabNodes;
    auto target = [&](int k) -> RStat & { return nodes[first + (k >> 1)].acc[k & 1]; };
    int openKey = -1, openLen = 0; // lane 0's carried run
    EStat open;
    estat_neutral(open);
    // the state words of the next chunk are loaded while this one is processed
    int vNext = wb + lane < we ? __ldcg(&state[wb + lane]) : 0;
    for (int base = wb; base < we; base += 32) {
        const int p = base + lane;
        int key = -1;
        EStat e;
        estat_neutral(e);
        const int v = vNext;
        vNext = base + 32 + lane < we ? __ldcg(&state[base + 32 + lane]) : 0;
        if (p < we) {
            int node = st_node(v), tag = st_tag(v);
            if (tag == 1 || tag == 2) {
                const int c = childTab && node >= prevFirst ? tab.child[node - prevFirst] : __ldcg(&np[node].child);
                if (c >= 0)
                    node = c + tag - 1;
                tag = 0;
            }
            if (node >= first && node < last) {
                const NParam q = parTab ? tab.par[node - first] : ld_nparam(&np[node]);
                if (q.count > kSub) {
                    // the split-axis key and the box and sum fields in one round trip (the fields go unused
                    // for the rare member inside the interval)
                    const unsigned long long o = soa[(size_t)q.axis * nt + p];
                    for (int k = 0; k < 3; ++k) {
                        e.lo[k] = soa[(size_t)(3 + k) * nt + p];
                        e.hi[k] = soa[(size_t)(6 + k) * nt + p];
                        e.s[k] = (long long)soa[(size_t)(9 + k) * nt + p];
                    }
                    const int sd = o < q.clo ? 0 : (o >= q.chi ? 1 : 2);
                    tag = sd + 1;
                    if (sd == 2) {
                        atomicOr(&nodes[node].flags, 1);
                        estat_neutral(e);
                    } else {
                        key = (node - first) * 2 + sd;
                    }
                }
            }
            const int nv = (node << 2) | tag;
            if (nv != v)
                state[p] = nv;
        }
        int len = key >= 0 ? 1 : 0;
        // the usual case in Morton order: the whole chunk holds one key (or none). The carried run is kept as
        // one partial per lane while chunks continue it, each lane adding its own member (no warp reduction);
        // it is summed across the warp only when it ends. A chunk without keys leaves the carried run open
        // (runs of one key merge in any grouping).
        const int key0 = __shfl_sync(full, key, 0);
        if (__all_sync(full, key == key0)) {
            if (key0 < 0)
                continue;
            if (openKey == key0) {
                estat_merge(open, e);
                openLen += len;
            } else {
                if (openKey >= 0) {
                    warp_uniform_reduce(open, openLen);
                    if (lane == 0)
                        stat_atomic(target(openKey), open, openLen);
                }
                openKey = key0;
                openLen = len;
                open = e;
            }
            continue;
        }
        // a chunk of several keys: the carried run's partials are summed into lane 0 first
        if (openKey >= 0) {
            warp_uniform_reduce(open, openLen);
            if (lane != 0) {
                estat_neutral(open);
                openLen = 0;
            }
        }
        // the carried run continues into lane 0 or is complete
        if (lane == 0) {
            if (openKey >= 0 && openKey == key) {
                estat_merge(e, open);
                len += openLen;
            } else if (openKey >= 0) {
                stat_atomic(target(openKey), open, openLen);
            }
        }
        const int prev = __shfl_up_sync(full, key, 1);
        const unsigned changes = __ballot_sync(full, lane > 0 && prev != key);
        if (__popc(changes) > 3) {
            // many short runs: group by key, flush every group, carry nothing
            int k2 = key, l2 = len;
            EStat e2 = e;
            if (warp_group_reduce(k2, e2, l2) && k2 >= 0)
                stat_atomic(target(k2), e2, l2);
            openKey = -1;
            openLen = 0;
            continue;
        }
        const bool tail = warp_segment_reduce(key, e, len);
        if (tail && lane != 31 && key >= 0)
            stat_atomic(target(key), e, len); // completed inside this chunk
        // the run through lane 31 stays open
        const int k31 = __shfl_sync(full, key, 31);
        const int l31 = __shfl_sync(full, len, 31);
        EStat e31;
        for (int k = 0; k < 3; ++k) {
            e31.lo[k] = __shfl_sync(full, e.lo[k], 31);
            e31.hi[k] = __shfl_sync(full, e.hi[k], 31);
            e31.s[k] = __shfl_sync(full, e.s[k], 31);
        }
        // the run through lane 31 stays open, held by lane 0 (the other lanes' partials start empty)
        openKey = k31;
        openLen = lane == 0 ? l31 : 0;
        if (lane == 0)
            open = e31;
        else
            estat_neutral(open);
    }
    // the open run's partials summed into lane 0; it joins the block reduction
    if (openKey >= 0)
        warp_uniform_reduce(open, openLen);
    const int fk = lane == 0 ? openKey : -1;
    block_reduce_keys(fk, open, lane == 0 ? openLen : 0, runs, warpRuns, target);
}

// Exact sides of one node whose member order matters: a member inside the interval (the reference's
// sequential sum in member order decides), or an empty side (the split takes halves of the member order).
// Run by the whole block; lists the members by triangle index, rewrites their state words and the children's
// statistics. `stage` is 2 x kStage doubles of shared memory. Symmetric inputs (an unjittered sphere: centres
// exactly on the mean by symmetry) send most large nodes here.
constexpr int kStage = 2048;
static_assert(sizeof(NParam) * kTabNodes >= 2 * kStage * sizeof(double), "staging aliases the level table");
__device__ void resolve_node(int id, int nt, const RRec *__restrict__ rec, int *state, const NParam &q, RNode &nd,
                             int *list, const int *__restrict__ posOf, int *warpSums, RunRec *runs, RStat *sAcc,
                             int &sLeft, double &sSplit, double *stage)
{
    const unsigned full = 0xFFFFFFFFu;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, warps = blockDim.x >> 5;
    const int n = q.count;
    const bool amb = (__ldcg(&nd.flags) & 1) != 0;
    const int dir = __ldcg(&nd.dir), axis = q.axis;
    if (tid == 0)
        sLeft = 0;
    // members by ascending triangle index: each warp scans one contiguous index range twice (count, then
    // write from its offset), so no block barrier runs per chunk
    {
        const int per = (((nt + warps - 1) / warps) + 31) & ~31;
        const int i0 = min(nt, w * per), i1 = min(nt, i0 + per);
        int cnt = 0;
#pragma unroll 4
        for (int b = i0; b < i1; b += 32) {
            const int i = b + lane;
            const bool m = i < i1 && st_node(__ldcg(&state[posOf[i]])) == id;
            cnt += __popc(__ballot_sync(full, m));
        }
        if (lane == 0)
            warpSums[w] = cnt;
        __syncthreads();
        int off = 0;
        for (int k = 0; k < w; ++k)
            off += warpSums[k];
#pragma unroll 4
        for (int b = i0; b < i1; b += 32) {
            const int i = b + lane;
            int pos = 0;
            bool m = false;
            if (i < i1) {
                pos = posOf[i];
                m = st_node(__ldcg(&state[pos])) == id;
            }
            const unsigned bal = __ballot_sync(full, m);
            const int at = off + __popc(bal & ((1u << lane) - 1u));
            if (m && at < n)
                list[at] = pos;
            off += __popc(bal);
        }
        __threadfence_block();
        __syncthreads();
    }
    if (amb) {
        // the reference's sum: sequential in member order. Warp 0's lane 0 adds one staged chunk while the
        // other warps gather the next one into the other half of `stage`.
        auto gather = [&](int c0, double *buf, int t0, int nthr) {
            const int m = min(kStage, n - c0);
            for (int k = t0; k < m; k += nthr) {
                const int mp = c0 + k;
                buf[k] = ord_to_dbl(rec[__ldcg(&list[dir ? n - 1 - mp : mp])].c[axis]);
            }
        };
        gather(0, stage, tid, blockDim.x);
        __syncthreads();
        double s = 0.0;
        for (int c0 = 0, j = 0; c0 < n; c0 += kStage, ++j) {
            const double *cur = stage + (j & 1) * kStage;
            if (w == 0) {
                if (lane == 0) {
                    const int m = min(kStage, n - c0);
                    int k = 0;
                    for (; k + 8 <= m; k += 8) {
                        const double a0 = cur[k], a1 = cur[k + 1], a2 = cur[k + 2], a3 = cur[k + 3];
                        const double a4 = cur[k + 4], a5 = cur[k + 5], a6 = cur[k + 6], a7 = cur[k + 7];
                        s = s + a0;
                        s = s + a1;
                        s = s + a2;
                        s = s + a3;
                        s = s + a4;
                        s = s + a5;
                        s = s + a6;
                        s = s + a7;
                    }
                    for (; k < m; ++k)
                        s = s + cur[k];
                }
                __syncwarp();
            } else if (c0 + kStage < n) {
                gather(c0 + kStage, stage + ((j + 1) & 1) * kStage, tid - 32, blockDim.x - 32);
            }
            __syncthreads();
        }
        if (tid == 0)
            sSplit = s / (double)(float)n;
        __syncthreads();
    }
    int myLeft = 0;
    for (int k = tid; k < n; k += blockDim.x) {
        const unsigned long long c = rec[__ldcg(&list[k])].c[axis];
        myLeft += (amb ? (ord_to_dbl(c) < sSplit) : (c < q.clo)) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1)
        myLeft += __shfl_xor_sync(0xFFFFFFFFu, myLeft, o);
    if ((tid & 31) == 0)
        atomicAdd(&sLeft, myLeft);
    if (tid < 2)
        rstat_clear(sAcc[tid]);
    __syncthreads();
    const int L = sLeft;
    const int mode = L == 0 ? 1 : (L == n ? 2 : 0);
    for (int k0 = 0; k0 < n; k0 += blockDim.x) {
        const int k = k0 + tid;
        int sd = -1;
        int pos = 0;
        if (k < n) {
            pos = __ldcg(&list[k]);
            const int mp = dir ? n - 1 - k : k; // position in member order
            if (mode == 0) {
                const unsigned long long c = rec[pos].c[axis];
                sd = (amb ? (ord_to_dbl(c) < sSplit) : (c < q.clo)) ? 0 : 1;
            } else if (mode == 1) {
                sd = mp < n / 2 ? 0 : 1;               // all right, in member order: halves
            } else {
                sd = (n - 1 - mp) < n - n / 2 ? 0 : 1; // all left, reversed: halves
            }
            state[pos] = (id << 2) | (sd + 1);
        }
        const EStat e = estat_of(sd >= 0, rec[pos]);
        block_reduce_keys(sd, e, sd >= 0 ? 1 : 0, runs, warpSums, [&](int qq) -> RStat & { return sAcc[qq]; });
    }
    __syncthreads();
    if (tid < 2)
        nd.acc[tid] = sAcc[tid];
    if (tid == 0)
        nd.mode = mode;
    __threadfence(); // state words and accumulators reach L2 before anyone reads them through it
    __syncthreads();
}

// The children of one split node, by one warp (lanes 0 and 1 write one child each; all 32 lanes call it): ids
// and terminal-list slots from atomic counters (node ids carry no order; begin offsets and direction bits
// do), statistics and split parameters.
__device__ void create_children(int id, RNode *nodes, NParam *np, int *counters, int *terms, int maxNodes,
                                const int *sc)
{
    RNode &nd = nodes[id];
    const int lane = threadIdx.x & 31;
    int c = 0;
    if (lane == 0) {
        c = atomicAdd(counters + kCtNodes, 2);
        if (c + 2 > maxNodes) {
            atomicExch(counters + kCtOverflow, 1); // nothing is split further; the host reports the overflow
            c = -1;
        }
    }
    c = __shfl_sync(0xFFFFFFFFu, c, 0);
    const int s2 = lane;
    if (c >= 0 && s2 < 2) {
        const RStat acc = ld_rstat(&nd.acc[s2]);
        const int leftCount = __ldcg(&nd.acc[0].count);
        const int mode = __ldcg(&nd.mode), dir = __ldcg(&nd.dir), begin = __ldcg(&nd.begin);
        const int dl = mode == 1 ? dir : dir ^ 1;
        const int dr = mode == 2 ? dir ^ 1 : dir;
        RNode &ch = nodes[c + s2];
        const int cnt = acc.count;
        ch.begin = s2 == 0 ? begin : begin + leftCount;
        ch.count = cnt;
        ch.dir = s2 == 0 ? dl : dr;
        ch.flags = 0;
        ch.mode = 0;
        ch.pad[0] = ch.pad[1] = ch.pad[2] = 0;
        ch.st = acc;
        rstat_clear(ch.acc[0]);
        rstat_clear(ch.acc[1]);
        NParam cq{-1, cnt, 0, 0, 0ull, 0ull};
        if (cnt > kSub)
            node_params(acc.lo, acc.hi, acc.sum, cnt, sc, cq.axis, cq.clo, cq.chi);
        else
            terms[atomicAdd(counters + kCtTerms, 1)] = c + s2;
        np[c + s2] = cq;
        if (s2 == 0)
            np[id].child = c; // read only after the grid barrier that ends this phase
    }
}

__global__ void __launch_bounds__(kElemThreads, 3)
    k_rr_top(int nt, const RRec *__restrict__ rec, const unsigned long long *__restrict__ soa, int *state, NParam *np,
             RNode *nodes, int *counters, int *terms,
             int maxNodes, const int *__restrict__ posOf, int *pool, const int *__restrict__ scg, GridBar *gb,
             unsigned long long *stamps)
{
    __shared__ RunRec runs[kRunCap];
    __shared__ int warpRuns[32];
    __shared__ RStat sAcc[2];
    __shared__ int sLeft;
    __shared__ double sSplit;
    const int sc[3] = {scg[0], scg[1], scg[2]};
    __shared__ LevelTab tab;
    int first = __ldcg(&counters[kCtFirst]), last = __ldcg(&counters[kCtLast]), prevFirst = first;
    // diagnostic: block 0 stamps the device time at each level's start, after its classification and after
    // its children (levels beyond the 32 recorded are not stamped)
    auto stamp = [&](int level, int k) {
        if (stamps && blockIdx.x == 0 && threadIdx.x == 0 && level < 32)
            stamps[3 * level + k] = global_ns();
    };
    for (int level = 0; level < kMaxLevels && first < last; ++level) {
        stamp(level, 0);
        load_level_tab(tab, np, prevFirst, first, last);
        {
            // contiguous Morton ranges: block slices of whole chunks, split among the block's warps
            const int warps = blockDim.x >> 5, w = threadIdx.x >> 5;
            const int chunks = (nt + 31) >> 5;
            const int perBlock = (chunks + gridDim.x - 1) / gridDim.x;
            const int perWarp = (perBlock + warps - 1) / warps;
            const int c0 = min(chunks, (int)blockIdx.x * perBlock + w * perWarp);
            const int c1 = min(min(chunks, ((int)blockIdx.x + 1) * perBlock), c0 + perWarp);
            classify_range(32 * c0, min(nt, 32 * c1), prevFirst, first, last, soa, nt, state, np, nodes, runs,
                           warpRuns, tab);
        }
        if (!grid_sync(gb))
            return;
        stamp(level, 1);
        // the block's nodes: the rare exact resolutions first (whole block each), then the children, one
        // warp per node
        for (int id = first + blockIdx.x; id < last; id += gridDim.x) {
            RNode &nd = nodes[id];
            const int count = __ldcg(&nd.count);
            if (count <= kSub)
                continue;
            const bool flagged = (__ldcg(&nd.flags) & 1) || __ldcg(&nd.acc[0].count) == 0 ||
                                 __ldcg(&nd.acc[1].count) == 0;
            if (flagged) // members of one level's nodes are disjoint: the node's leaf range is its list space
                resolve_node(id, nt, rec, state, ld_nparam(&np[id]), nd, pool + __ldcg(&nd.begin), posOf, warpRuns,
                             runs, sAcc, sLeft, sSplit, reinterpret_cast<double *>(tab.par));
        }
        __syncthreads();
        {
            const int w = threadIdx.x >> 5, W = blockDim.x >> 5;
            int k = 0;
            for (int id = first + blockIdx.x; id < last; id += gridDim.x, ++k)
                if (k % W == w && __ldcg(&nodes[id].count) > kSub)
                    create_children(id, nodes, np, counters, terms, maxNodes, sc);
        }
        if (!grid_sync(gb))
            return;
        stamp(level, 2);
        prevFirst = first;
        first = last;
        last = min(__ldcg(&counters[kCtNodes]), maxNodes);
        if (__ldcg(&counters[kCtOverflow]))
            break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counters[kCtFirst] = first;
        counters[kCtLast] = last;
    }
}

// After the last level: every member's terminal node, and the sort key (the node's first leaf position)
// stored by triangle index, so that a stable sort lists each node's members by ascending index.
// It also starts the tree's node table with the large nodes: {first leaf position, member count, left child
// (right = left + 1), or -1 while the node is terminal}; the subtree blocks fill in the terminal nodes' own
// subtrees, numbering their nodes from maxNodes up.
__global__ void k_rr_finish(int nt, const int *__restrict__ state, const NParam *__restrict__ np,
                            const RNode *__restrict__ nodes, const int *__restrict__ leafTri, int *key, int *val,
                            int4 *tnode, int *counters, int maxNodes)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < min(counters[kCtNodes], maxNodes)) {
        const int cnt = nodes[q].count;
        tnode[q] = make_int4(nodes[q].begin, cnt, cnt > kSub ? np[q].child : -1, 0);
    }
    if (q == 0)
        counters[kCtTNodes] = maxNodes;
    if (q >= nt)
        return;
    const int v = state[q];
    int node = st_node(v);
    const int tag = st_tag(v);
    if ((tag == 1 || tag == 2) && np[node].child >= 0)
        node = np[node].child + tag - 1;
    const int i = leafTri[q];
    key[i] = nodes[node].begin;
    val[i] = i;
}

// ---------------------------------------------------------------------------------------------------
// One block finishes the subtree of one node with at most kSub members: the same level loop as above, with
// the node records and the member permutation in shared memory and __syncthreads between the steps.
// ---------------------------------------------------------------------------------------------------
struct SNode {
    int begin, count, axis, leftFinal, child, amb;
    unsigned long long clo, chi;
    unsigned long long lo[3], hi[3];
    long long sum[3];
};

__device__ __forceinline__ void snode_init(SNode &n, int begin, int count)
{
    n.begin = begin;
    n.count = count;
    n.axis = 0;
    n.leftFinal = 0;
    n.child = -1;
    n.amb = 0;
    n.clo = n.chi = 0;
    for (int k = 0; k < 3; ++k) {
        n.lo[k] = ~0ull;
        n.hi[k] = 0ull;
        n.sum[k] = 0;
    }
}

// about 55 KB: four blocks per SM
constexpr size_t kSubSmem = sizeof(SNode) * kSubNodes + sizeof(int) * (6 * kSub + 1 + kSubThreads / 32);

// One terminal node of the large-node phase (terms[t]), by the whole block.
__device__ __forceinline__ void subtree_one(int t, const int *__restrict__ terms, const RNode *__restrict__ gnodes,
                                            const int *__restrict__ sorted, const RRec *__restrict__ rec,
                                            const int *__restrict__ posOf, const int *__restrict__ leafTri,
                                            const int *__restrict__ scg, int *rank, int *counters, int4 *tnode,
                                            int tnodeCap)
{
    extern __shared__ __align__(16) unsigned char smem[];
    SNode *nodes = reinterpret_cast<SNode *>(smem);
    int(*nodeOf)[kSub] = reinterpret_cast<int(*)[kSub]>(smem + sizeof(SNode) * kSubNodes);
    int(*perm)[kSub] = reinterpret_cast<int(*)[kSub]>(smem + sizeof(SNode) * kSubNodes + sizeof(int) * 2 * kSub);
    int *flag = reinterpret_cast<int *>(smem + sizeof(SNode) * kSubNodes + sizeof(int) * 4 * kSub);
    int *scan = flag + kSub;
    int *warpSum = scan + kSub + 1;
    __shared__ int nNodes, lFirst, lLast, anyAmb, err, tBase;
    const int tid = threadIdx.x;
    const RNode &g = gnodes[terms[t]];
    const int base = g.begin, n = g.count, dir = g.dir;
    int sc[3] = {scg[0], scg[1], scg[2]};
    // perm holds Morton positions (record indices), in member order
    for (int p = tid; p < n; p += kSubThreads) {
        perm[0][p] = posOf[sorted[base + (dir ? n - 1 - p : p)]];
        nodeOf[0][p] = 0;
    }
    if (n <= kLeaf) {
        __syncthreads();
        for (int p = tid; p < n; p += kSubThreads)
            rank[leafTri[perm[0][p]]] = base + p;
        return;
    }
    if (tid == 0) {
        SNode &r = nodes[0];
        snode_init(r, 0, n);
        for (int k = 0; k < 3; ++k) {
            r.lo[k] = g.st.lo[k];
            r.hi[k] = g.st.hi[k];
            r.sum[k] = g.st.sum[k];
        }
        nNodes = 1;
        lFirst = 0;
        lLast = 1;
        err = 0;
    }
    __syncthreads();
    int cur = 0;
    for (int level = 0; level < 4 * kSub; ++level) {
        const int first = lFirst, last = lLast;
        if (first >= last || err)
            break;
        // split parameters
        for (int id = first + tid; id < last; id += kSubThreads) {
            SNode &nd = nodes[id];
            if (nd.count <= kLeaf) {
                nd.child = -1;
                continue;
            }
            node_params(nd.lo, nd.hi, nd.sum, nd.count, sc, nd.axis, nd.clo, nd.chi);
            nd.amb = 0;
        }
        if (tid == 0)
            anyAmb = 0;
        __syncthreads();
        // classify: flag 1 = left
        for (int p = tid; p < n; p += kSubThreads) {
            const int id = nodeOf[cur][p];
            int f = 0;
            if (id >= first) {
                SNode &nd = nodes[id];
                if (nd.count > kLeaf) {
                    const unsigned long long o = rec[perm[cur][p]].c[nd.axis];
                    if (o < nd.clo)
                        f = 1;
                    else if (o < nd.chi) {
                        nd.amb = 1;
                        anyAmb = 1;
                    }
                }
            }
            flag[p] = f;
        }
        __syncthreads();
        if (anyAmb) {
            // the reference's sequential sum in member order (perm holds the member order)
            for (int id = first + tid; id < last; id += kSubThreads) {
                SNode &nd = nodes[id];
                if (nd.count <= kLeaf || !nd.amb)
                    continue;
                double s = 0.0;
                for (int p = nd.begin; p < nd.begin + nd.count; ++p)
                    s = s + ord_to_dbl(rec[perm[cur][p]].c[nd.axis]);
                const double split = s / (double)(float)nd.count;
                for (int p = nd.begin; p < nd.begin + nd.count; ++p)
                    flag[p] = ord_to_dbl(rec[perm[cur][p]].c[nd.axis]) < split ? 1 : 0;
            }
            __syncthreads();
        }
        // block exclusive scan of flag[0..n): each thread owns a contiguous run of kSub / kSubThreads slots
        {
            const int per = kSub / kSubThreads;
            const int b0 = tid * per;
            int local = 0;
            for (int j = 0; j < per; ++j)
                local += (b0 + j < n) ? flag[b0 + j] : 0;
            int incl = local;
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if ((tid & 31) >= o)
                    incl += v;
            }
            if ((tid & 31) == 31)
                warpSum[tid >> 5] = incl;
            __syncthreads();
            int woff = 0;
            for (int w = 0; w < (tid >> 5); ++w)
                woff += warpSum[w];
            int run = woff + incl - local;
            for (int j = 0; j < per; ++j) {
                if (b0 + j <= n)
                    scan[b0 + j] = run;
                run += (b0 + j < n) ? flag[b0 + j] : 0;
            }
            if (tid == kSubThreads - 1)
                scan[n] = run;
        }
        __syncthreads();
        // children
        for (int id = first + tid; id < last; id += kSubThreads) {
            SNode &nd = nodes[id];
            if (nd.count <= kLeaf)
                continue;
            const int left = scan[nd.begin + nd.count] - scan[nd.begin];
            const int right = nd.count - left;
            int lf = left;
            if (left == 0)
                lf = right / 2;
            else if (right == 0)
                lf = left - left / 2;
            const int c = atomicAdd(&nNodes, 2);
            if (c + 2 > kSubNodes) {
                err = 1;
                nd.count = 0;
                continue;
            }
            nd.leftFinal = lf;
            nd.child = c;
            snode_init(nodes[c], nd.begin, lf);
            snode_init(nodes[c + 1], nd.begin + lf, nd.count - lf);
        }
        __syncthreads();
        // scatter the indices into the other buffer
        for (int p = tid; p < n; p += kSubThreads) {
            const int id = nodeOf[cur][p];
            if (id < first || nodes[id].count <= kLeaf) {
                perm[cur ^ 1][p] = perm[cur][p];
                nodeOf[cur ^ 1][p] = -1;
                continue;
            }
            const SNode &nd = nodes[id];
            const int left = scan[nd.begin + nd.count] - scan[nd.begin];
            const int lrank = scan[p] - scan[nd.begin];
            const int rrank = (p - nd.begin) - lrank;
            int pos;
            if (left == 0)
                pos = rrank;
            else if (left == nd.count)
                pos = nd.count - 1 - lrank;
            else
                pos = flag[p] ? (left - 1 - lrank) : (left + rrank);
            const int q = nd.begin + pos;
            const int ch = pos < nd.leftFinal ? nd.child : nd.child + 1;
            perm[cur ^ 1][q] = perm[cur][p];
            nodeOf[cur ^ 1][q] = nodes[ch].count > kLeaf ? ch : -2; // leaves need no statistics
        }
        __syncthreads();
        // Statistics of the children that split again, read in the new order. A node's members are contiguous
        // and number more than 20, so the kPer consecutive positions of one thread hold at most a head run
        // that ends a node inside the thread and a tail run that continues past it (a run in between can only
        // be of settled members). A segmented scan over the threads' tail runs gives each run's total where it
        // ends: a node's total is written to the node, a run cut at a warp's last position is kept per chunk,
        // and one thread per node then adds the chunk totals inside its range. No atomics.
        {
            constexpr int kPer = kSub / kSubThreads;
            constexpr int kChunk = 32 * kPer; // positions per warp
            EStat *chunk = reinterpret_cast<EStat *>(scan); // the scan is consumed; kSubThreads / 32 entries fit
            const int lane = tid & 31, w = tid >> 5;
            const int lastPos = kPer * tid + kPer - 1;
            int kHead = -1, kTail = -1;
            bool split = false;
            EStat head, tail;
            estat_neutral(head);
            estat_neutral(tail);
            for (int j = 0; j < kPer; ++j) {
                const int p = kPer * tid + j;
                const int id = p < n ? nodeOf[cur ^ 1][p] : -1;
                const int key = id >= 0 ? id : -1;
                if (j == 0) {
                    kTail = key;
                } else if (key != kTail) {
                    if (!split) {
                        kHead = kTail;
                        head = tail;
                        split = true;
                    }
                    kTail = key;
                    estat_neutral(tail);
                }
                if (key >= 0)
                    estat_merge(tail, estat_of(true, rec[perm[cur ^ 1][p]]));
            }
            const int prevKey = __shfl_up_sync(0xFFFFFFFFu, kTail, 1);
            EStat run = tail;
            warp_segmented_scan(lane == 0 || split || prevKey != kTail, run);
            EStat prev;
            for (int k = 0; k < 3; ++k) {
                prev.lo[k] = __shfl_up_sync(0xFFFFFFFFu, run.lo[k], 1);
                prev.hi[k] = __shfl_up_sync(0xFFFFFFFFu, run.hi[k], 1);
                prev.s[k] = __shfl_up_sync(0xFFFFFFFFu, run.s[k], 1);
            }
            if (split && kHead >= 0) {
                if (lane > 0 && prevKey == kHead)
                    estat_merge(head, prev);
                SNode &nd = nodes[kHead];
                for (int k = 0; k < 3; ++k) {
                    nd.lo[k] = head.lo[k];
                    nd.hi[k] = head.hi[k];
                    nd.sum[k] = head.s[k];
                }
            }
            if (kTail >= 0) {
                SNode &nd = nodes[kTail];
                if (nd.begin + nd.count - 1 == lastPos) {
                    for (int k = 0; k < 3; ++k) {
                        nd.lo[k] = run.lo[k];
                        nd.hi[k] = run.hi[k];
                        nd.sum[k] = run.s[k];
                    }
                } else if (lane == 31) {
                    chunk[w] = run;
                }
            }
            __syncthreads();
            for (int id = last + tid; id < nNodes; id += kSubThreads) {
                SNode &nd = nodes[id];
                if (nd.count <= kLeaf)
                    continue;
                const int b = nd.begin, e = nd.begin + nd.count - 1; // chunk ends in [b, e) belong to the node
                for (int j = b / kChunk; kChunk * j + kChunk - 1 < e; ++j) {
                    const EStat &c = chunk[j];
                    for (int k = 0; k < 3; ++k) {
                        nd.lo[k] = min(nd.lo[k], c.lo[k]);
                        nd.hi[k] = max(nd.hi[k], c.hi[k]);
                        nd.sum[k] += c.s[k];
                    }
                }
            }
        }
        __syncthreads();
        if (tid == 0) {
            lFirst = last;
            lLast = nNodes;
        }
        cur ^= 1;
        __syncthreads();
    }
    if (tid == 0 && (err || lFirst < lLast))
        atomicAdd(counters + kCtSubErr, 1);
    for (int p = tid; p < n; p += kSubThreads)
        rank[leafTri[perm[cur][p]]] = base + p;
    // the subtree's nodes in the node table: record k > 0 becomes tBase + k - 1 (children stay adjacent)
    if (tid == 0) {
        tBase = atomicAdd(counters + kCtTNodes, nNodes - 1);
        if (tBase + nNodes - 1 > tnodeCap)
            atomicAdd(counters + kCtSubErr, 1);
    }
    __syncthreads();
    if (tBase + nNodes - 1 <= tnodeCap)
        for (int k = tid; k < nNodes; k += kSubThreads) {
            const SNode &nd = nodes[k];
            const int left = (nd.child >= 0 && nd.count > kLeaf) ? tBase + nd.child - 1 : -1;
            if (k == 0)
                tnode[terms[t]].z = left;
            else
                tnode[tBase + k - 1] = make_int4(base + nd.begin, nd.count, left, 0);
        }
}

// The terminal nodes, a block at a time: the count is known only on the device, so the grid is one resident
// wave (or the largest possible count, if smaller) and every block strides over the list.
__global__ void __launch_bounds__(kSubThreads, 4)
    k_rr_subtree(const int *__restrict__ terms, const RNode *__restrict__ gnodes, const int *__restrict__ sorted,
                 const RRec *__restrict__ rec, const int *__restrict__ posOf, const int *__restrict__ leafTri,
                 const int *__restrict__ scg, int *rank, int *counters, int4 *tnode, int tnodeCap)
{
    const int nTerms = counters[kCtTerms];
    for (int t = blockIdx.x; t < nTerms; t += gridDim.x) {
        subtree_one(t, terms, gnodes, sorted, rec, posOf, leafTri, scg, rank, counters, tnode, tnodeCap);
        __syncthreads(); // shared memory is reused by the next node
    }
}

static int bit_length(int x)
{
    int b = 0;
    while (x > 0) {
        ++b;
        x >>= 1;
    }
    return b;
}

// Cooperative blocks of k_rr_top in flight per device. Cooperative grids launched from several streams at
// once (two meshes of a boolean, batched booleans) must fit on the device together, or resident blocks of
// one could wait at a grid barrier for blocks that cannot be scheduled. A launch takes its blocks from the
// budget before it is issued and records an event after the kernel; blocks come back when a later launch
// finds that event complete. A launch that does not fit waits for the oldest such event (its kernel is
// already queued, so it finishes), never for a launch that has not been issued.
struct CoopBudget {
    std::mutex mu;
    std::condition_variable cv; // a pending launch was held or cancelled
    int capacity[256] = {0}, inFlight[256] = {0}, pending[256] = {0};
    struct Held {
        cudaEvent_t done;
        int dev, blocks;
    };
    std::deque<Held> held;          // in launch order
    std::vector<cudaEvent_t> spare; // events for reuse
};
static CoopBudget g_coop;

// with g_coop.mu held: return the blocks of every launch whose kernel has finished
static void coop_reclaim_locked()
{
    for (auto it = g_coop.held.begin(); it != g_coop.held.end();) {
        if (cudaEventQuery(it->done) == cudaSuccess) {
            g_coop.inFlight[it->dev] -= it->blocks;
            g_coop.spare.push_back(it->done);
            it = g_coop.held.erase(it);
        } else {
            ++it;
        }
    }
}

static cudaError_t coop_acquire(int dev, int blocks)
{
    std::unique_lock<std::mutex> lk(g_coop.mu);
    coop_reclaim_locked();
    while (g_coop.inFlight[dev] + blocks > g_coop.capacity[dev]) {
        if (g_coop.held.empty()) {
            if (g_coop.pending[dev] == 0)
                break; // nothing else holds blocks: a grid fits the device by construction
            g_coop.cv.wait(lk); // launches between acquire and hold: each ends in a hold or a cancel
            coop_reclaim_locked();
            continue;
        }
        const cudaEvent_t oldest = g_coop.held.front().done;
        lk.unlock();
        const cudaError_t e = cudaEventSynchronize(oldest);
        lk.lock();
        if (e != cudaSuccess)
            return e;
        coop_reclaim_locked();
    }
    g_coop.inFlight[dev] += blocks;
    ++g_coop.pending[dev];
    return cudaSuccess;
}

// after a successful cooperative launch on stream s: an event marks when its blocks are free again
static cudaError_t coop_hold(int dev, int blocks, cudaStream_t s)
{
    std::lock_guard<std::mutex> lk(g_coop.mu);
    --g_coop.pending[dev];
    g_coop.cv.notify_all();
    cudaEvent_t e = nullptr;
    if (!g_coop.spare.empty()) {
        e = g_coop.spare.back();
        g_coop.spare.pop_back();
    } else {
        const cudaError_t ce = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        if (ce != cudaSuccess) {
            g_coop.inFlight[dev] -= blocks;
            return ce;
        }
    }
    const cudaError_t re = cudaEventRecord(e, s);
    if (re != cudaSuccess) {
        g_coop.spare.push_back(e);
        g_coop.inFlight[dev] -= blocks;
        return re;
    }
    g_coop.held.push_back(CoopBudget::Held{e, dev, blocks});
    return cudaSuccess;
}

// a launch that failed returns its blocks at once
static void coop_cancel(int dev, int blocks)
{
    std::lock_guard<std::mutex> lk(g_coop.mu);
    g_coop.inFlight[dev] -= blocks;
    --g_coop.pending[dev];
    g_coop.cv.notify_all();
}

// Blocks of the cooperative large-node kernel: a quarter of what can be resident at once, no more than the
// members need. The two meshes of a boolean build their leaf orders concurrently, and each grid holds its SMs'
// whole register file until it ends, while the LBVH builds and the broad and narrow phases run on what is left;
// the share balances the two paths (measured on pair_large L7, boolean step: a third 1.76-1.80 ms, a quarter
// 1.67 ms, a fifth 1.74 ms, a sixth 1.77 ms).
static int top_grid(int nt, int *devOut)
{
    static int perSm[256], sms[256];
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256)
        return -1;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (perSm[dev] == 0) {
            int coop = 0;
            if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
                cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm[dev], k_rr_top, kElemThreads, 0) != cudaSuccess ||
                perSm[dev] <= 0) {
                set_last_error("cooperative launch unavailable for the reference tree build");
                perSm[dev] = 0;
                return -1;
            }
            std::lock_guard<std::mutex> lk2(g_coop.mu);
            g_coop.capacity[dev] = perSm[dev] * sms[dev];
        }
    }
    *devOut = dev;
    const int need = (nt + kElemThreads * 4 - 1) / (kElemThreads * 4); // at least 4 members per thread
    return std::max(1, std::min(need, std::max(1, perSm[dev] * sms[dev] / 4)));
}

// Status of a leaf-order build from its counters and barrier record (12 ints).
static sb_status rank_status(const int *chk)
{
    const int *cnt = chk;
    if (chk[kCtCount + 2]) { // GridBar::err
        set_last_error("reference tree: a grid barrier timed out");
        return SB_ERR_CUDA;
    }
    if (cnt[kCtOverflow]) {
        set_last_error("reference tree node capacity exceeded");
        return SB_ERR_CAPACITY;
    }
    if (cnt[kCtFirst] < cnt[kCtLast]) {
        set_last_error("reference tree deeper than the level limit");
        return SB_ERR_CAPACITY;
    }
    if (cnt[kCtSubErr]) {
        set_last_error("reference tree: a subtree exceeded its node records");
        return SB_ERR_CAPACITY;
    }
    return SB_OK;
}

// Pinned host memory in fixed-size slots, carved from blocks that are allocated on demand and kept for the
// process: pinned allocations are slow and synchronise the device, while meshes and booleans come and go.
namespace {
class PinnedPool {
public:
    PinnedPool(size_t slot, int perBlock) : slot_(slot), per_(perBlock) {}
    void *acquire()
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (free_.empty()) {
            char *blk = nullptr;
            if (cudaMallocHost((void **)&blk, slot_ * (size_t)per_) != cudaSuccess)
                return nullptr;
            for (int i = per_ - 1; i >= 0; --i)
                free_.push_back(blk + slot_ * (size_t)i);
        }
        void *p = free_.back();
        free_.pop_back();
        return p;
    }
    void release(void *p)
    {
        if (!p)
            return;
        std::lock_guard<std::mutex> lk(mu_);
        free_.push_back(static_cast<char *>(p));
    }

private:
    size_t slot_;
    int per_;
    std::mutex mu_;
    std::vector<char *> free_;
};
static_assert(kCtCount + sizeof(GridBar) / sizeof(int) <= 15, "the mesh's pinned slot keeps its last int for validation");
PinnedPool g_slots(16 * sizeof(int), 4096);
PinnedPool g_mail(kMailBytes, 256);
} // namespace

int *pinned_slot_acquire() { return static_cast<int *>(g_slots.acquire()); }
void pinned_slot_release(int *p) { g_slots.release(p); }
char *pinned_mail_acquire() { return static_cast<char *>(g_mail.acquire()); }
void pinned_mail_release(char *p) { g_mail.release(p); }

sb_status reference_rank_result(sb_mesh *m)
{
    if (!m->rankPending)
        return SB_OK;
    m->rankPending = false;
    const sb_status st = rank_status(m->rankCheck);
    if (st != SB_OK)
        m->d.rankValid = false;
    return st;
}

// one resident wave of k_rr_subtree blocks on the current device
static int subtree_grid()
{
    static int grid = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0, sms = 0, per = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            cudaFuncSetAttribute(k_rr_subtree, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSubSmem) ==
                cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rr_subtree, kSubThreads, kSubSmem) == cudaSuccess)
            grid = std::max(1, sms * per);
        else
            grid = 1 << 20; // unknown: no cap (the list is still covered)
    });
    return grid;
}

sb_status build_reference_rank(sb_mesh *m, cudaStream_t s, bool wait)
{
    MeshDev &d = m->d;
    const int nt = d.nt;
    d.rankValid = false;
    if (nt <= 0)
        return SB_OK;
    // large nodes have more than kSub members and are disjoint within a level
    const int maxNodes = 16 * (nt / kSub) + 256;
    const int keyBits = bit_length(nt);
    size_t sortBytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, sortBytes, (int *)nullptr, (int *)nullptr, (int *)nullptr,
                                    (int *)nullptr, nt, 0, keyBits, s);
    Carve c;
    const size_t o_rec = c.take<RRec>(nt), o_soa = c.take<unsigned long long>((size_t)12 * nt),
                 o_state = c.take<int>(nt), o_pos = c.take<int>(nt);
    const size_t o_key = c.take<int>(nt), o_val = c.take<int>(nt), o_skey = c.take<int>(nt),
                 o_sval = c.take<int>(nt), o_pool = c.take<int>(nt);
    const size_t o_np = c.take<NParam>(maxNodes);
    const size_t o_nodes = c.take<RNode>(maxNodes), o_terms = c.take<int>(maxNodes), o_ct = c.take<int>(kCtCount),
                 o_sc = c.take<int>(4), o_bar = c.take<GridBar>(1), o_cub = c.take<char>(sortBytes);
    // node table: the large nodes (ids below maxNodes) and at most 2 nt subtree nodes
    const int tnodeCap = maxNodes + 2 * nt + 2;
    const size_t o_tn = c.take<int4>(tnodeCap), o_stamp = c.take<unsigned long long>(96);
    SB_CUDA_CHECK(m->rankTmp.ensure(c.off));
    char *b = m->rankTmp.as<char>();
    RRec *rec = (RRec *)(b + o_rec);
    unsigned long long *soa = (unsigned long long *)(b + o_soa);
    int *state = (int *)(b + o_state);
    NParam *np = (NParam *)(b + o_np);
    int *key = (int *)(b + o_key), *val = (int *)(b + o_val), *skey = (int *)(b + o_skey), *sval = (int *)(b + o_sval);
    int *pool = (int *)(b + o_pool), *posOf = (int *)(b + o_pos);
    RNode *nodes = (RNode *)(b + o_nodes);
    int *terms = (int *)(b + o_terms), *counters = (int *)(b + o_ct), *scg = (int *)(b + o_sc);
    GridBar *bar = (GridBar *)(b + o_bar);
    int4 *tnode = (int4 *)(b + o_tn);
    d.tnode = tnode;
    d.tnodeCount = tnodeCap;
    unsigned long long *stamps = (unsigned long long *)(b + o_stamp);
    d.levelStamps = stamps;
    SB_CUDA_CHECK(cudaMemsetAsync(stamps, 0, 96 * sizeof(unsigned long long), s));

    const int GE = (nt + kElemThreads - 1) / kElemThreads;
    if (!d.absMax) {
        set_last_error("leaf order: the mesh's coordinate bound is missing");
        return SB_ERR_INVALID;
    }
    SB_COUNT(k_rr_init)<<<1, 1, 0, s>>>(nodes, np, nt, counters, reinterpret_cast<unsigned *>(bar));
    {
        KTime kt("k_rr_elems", s);
        SB_COUNT(k_rr_elems)<<<GE, kElemThreads, 0, s>>>(nt, d.v, d.t, d.box64, d.leafTri, rec, soa, posOf, state,
                                                          nodes, np, counters, terms, scg, d.absMax, &bar->ticket);
    }
    // the large-node phase: one cooperative launch, every block resident
    if (nt > kSub) {
        int dev = 0;
        const int topBlocks = top_grid(nt, &dev);
        if (topBlocks <= 0)
            return SB_ERR_CUDA;
        SB_CUDA_CHECK(coop_acquire(dev, topBlocks));
        void *args[] = {(void *)&nt, (void *)&rec, (void *)&soa, (void *)&state, (void *)&np, (void *)&nodes, (void *)&counters,
                        (void *)&terms, (void *)&maxNodes, (void *)&posOf, (void *)&pool, (void *)&scg, (void *)&bar,
                        (void *)&stamps};
        count_launch();
        KTime kt("k_rr_top", s);
        const cudaError_t le =
            cudaLaunchCooperativeKernel((const void *)k_rr_top, dim3(topBlocks), dim3(kElemThreads), args, 0, s);
        if (le != cudaSuccess) {
            coop_cancel(dev, topBlocks);
            SB_CUDA_CHECK(le);
        }
        SB_CUDA_CHECK(coop_hold(dev, topBlocks, s));
    }
    SB_COUNT(k_rr_finish)<<<GE, kElemThreads, 0, s>>>(nt, state, np, nodes, d.leafTri, key, val, tnode, counters,
                                                       maxNodes);
    SB_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(b + o_cub, sortBytes, key, skey, val, sval, nt, 0, keyBits, s));
    {
        static std::once_flag smemOnce; // a per-call attribute set is a driver call every build
        static cudaError_t smemErr = cudaSuccess;
        std::call_once(smemOnce, [] {
            smemErr = cudaFuncSetAttribute(k_rr_subtree, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSubSmem);
        });
        SB_CUDA_CHECK(smemErr);
    }
    // the terminal nodes, a resident wave of blocks striding over the device-side list
    {
        KTime kt("k_rr_subtree", s);
        SB_COUNT(k_rr_subtree)<<<std::min(maxNodes, subtree_grid()), kSubThreads, kSubSmem, s>>>(terms, nodes, sval, rec, posOf, d.leafTri,
                                                                        scg, d.rank, counters, tnode, tnodeCap);
    }
    // counters and barrier record to pinned host memory; read now, or by reference_rank_result once the
    // caller has synchronised past this stream
    if (!m->rankCheck) {
        m->rankCheck = pinned_slot_acquire();
        if (!m->rankCheck) {
            set_last_error("no pinned host memory for the leaf-order status");
            return SB_ERR_CUDA;
        }
    }
    SB_CUDA_CHECK(cudaMemcpyAsync(m->rankCheck, counters, kCtCount * sizeof(int), cudaMemcpyDeviceToHost, s));
    SB_CUDA_CHECK(cudaMemcpyAsync(m->rankCheck + kCtCount, bar, sizeof(GridBar), cudaMemcpyDeviceToHost, s));
    SB_CUDA_CHECK(cudaGetLastError());
    d.rankValid = true;
    m->rankPending = true;
    if (!wait)
        return SB_OK;
    SB_CUDA_CHECK(cudaStreamSynchronize(s));
    return reference_rank_result(m);
}

} // namespace sbg
