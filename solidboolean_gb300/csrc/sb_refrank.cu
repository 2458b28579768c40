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
// resolution, children); one radix sort then lists each remaining node's members in order, and one block per
// such node finishes its subtree in shared memory and writes the final positions.
#include <cub/cub.cuh>

#include "sb_common.cuh"
#include "sb_internal.h"
#include "sb_ktime.h"

namespace sbg {

constexpr int kLeaf = 20;        // reference leaf size (src/axisalignedboundingboxtree.cpp:25)
constexpr int kSub = 1024;       // nodes with at most this many members finish in one block
constexpr int kSubThreads = 256;
constexpr int kSubNodes = 272;   // node records per subtree block (shared memory)
constexpr int kWide = 1024;      // block size of the large-node phase

// counters[] slots
enum {
    kCtNodes = 0,   // node records allocated
    kCtTerms = 1,   // terminal nodes listed
    kCtOverflow = 2,
    kCtPool = 3,    // member-list pool use of the current level (exact resolution)
    kCtFirst = 4,   // current level: first node
    kCtLast = 5,    //                one past the last node
    kCtSubErr = 6,  // subtree blocks that ran out of node records
    kCtCount = 8
};

// one triangle: its box centre and box, in triangle index order
struct RRec {
    double c[3];
    double lo[3], hi[3];
};

// box (order-preserving keys) and fixed-point centre sum of a set of members
struct RStat {
    unsigned long long lo[3], hi[3];
    long long sum[3];
    int count, pad;
};

struct RNode {
    int begin, count;  // begin: position of the node's first member in the final leaf order
    int child;         // left child id (right = child + 1), -1 while unsplit or terminal
    int dir;           // member order: 0 ascending triangle index, 1 descending
    int axis, flags;   // flags bit 0: a member fell inside the interval
    int mode, pad;     // 0 regular split, 1 left side was empty, 2 right side was empty
    unsigned long long clo, chi; // order-preserving keys of an interval holding the reference's split value
    RStat st;                    // the node's own members
    RStat acc[2];                // left / right members, accumulated while classifying
};

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

__device__ __forceinline__ EStat estat_of(bool valid, const RRec &r, const int *sc)
{
    EStat e;
    for (int k = 0; k < 3; ++k) {
        e.lo[k] = valid ? ordc(r.lo[k]) : ~0ull;
        e.hi[k] = valid ? ordc(r.hi[k]) : 0ull;
        e.s[k] = valid ? to_fixed(r.c[k], sc[k]) : 0;
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

// Segmented inclusive reduction over runs of equal `key` among the 32 lanes. Returns true on the last lane
// of each run, which then holds the run's total and its length in `len`. All 32 lanes must call it.
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
        if (lane - o >= head)
            estat_merge(r, t);
    }
    len = lane - head + 1;
    const int nextKey = __shfl_down_sync(full, key, 1);
    return lane == 31 || nextKey != key;
}

// merges a run's box and sum into a node (global or shared); sums add as two's complement
template <class Stat>
__device__ __forceinline__ void stat_atomic_box(Stat &dst, const EStat &e)
{
    for (int k = 0; k < 3; ++k) {
        atomicMin(&dst.lo[k], e.lo[k]);
        atomicMax(&dst.hi[k], e.hi[k]);
        atomicAdd(reinterpret_cast<unsigned long long *>(&dst.sum[k]), (unsigned long long)e.s[k]);
    }
}

__device__ __forceinline__ void stat_atomic(RStat &dst, const EStat &e, int len)
{
    stat_atomic_box(dst, e);
    atomicAdd(&dst.count, len);
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
__global__ void k_rr_init(RNode *nodes, int nt, int *counters)
{
    RNode &r = nodes[0];
    r.begin = 0;
    r.count = nt;
    r.child = -1;
    r.dir = 0;
    r.axis = 0;
    r.flags = 0;
    r.mode = 0;
    r.pad = 0;
    r.clo = r.chi = 0;
    rstat_clear(r.st);
    rstat_clear(r.acc[0]);
    rstat_clear(r.acc[1]);
    r.st.count = nt;
    for (int i = 0; i < kCtCount; ++i)
        counters[i] = 0;
    counters[kCtNodes] = 1;
}

// box centre of each triangle as AxisAlignedBoudingBox::updateCenter computes it, (((0 + v0) + v1) + v2) /
// (float)3 (src/axisalignedboundingbox.h:31-53), its box, and the root box (src/solidmesh.cpp:68-72)
__global__ void __launch_bounds__(kWide) k_rr_elems(int nt, const double *__restrict__ v,
                                                    const uint32_t *__restrict__ t,
                                                    const double *__restrict__ box64, RRec *rec, int *nodeOf,
                                                    int8_t *side, RNode *nodes)
{
    __shared__ unsigned long long sLo[3], sHi[3];
    if (threadIdx.x < 3) {
        sLo[threadIdx.x] = ~0ull;
        sHi[threadIdx.x] = 0ull;
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    if (i < nt) {
        RRec r;
        for (int a = 0; a < 3; ++a) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                s = s + v[3 * (size_t)t[3 * (size_t)i + k] + a];
            r.c[a] = s / 3.0;
            r.lo[a] = box64[6 * (size_t)i + a];
            r.hi[a] = box64[6 * (size_t)i + 3 + a];
            lo[a] = ordc(r.lo[a]);
            hi[a] = ordc(r.hi[a]);
        }
        rec[i] = r;
        nodeOf[i] = 0;
        side[i] = -1;
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int a = 0; a < 3; ++a) {
            lo[a] = min(lo[a], __shfl_xor_sync(0xFFFFFFFFu, lo[a], o));
            hi[a] = max(hi[a], __shfl_xor_sync(0xFFFFFFFFu, hi[a], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; ++a) {
            atomicMin(&sLo[a], lo[a]);
            atomicMax(&sHi[a], hi[a]);
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        atomicMin(&nodes[0].st.lo[threadIdx.x], sLo[threadIdx.x]);
        atomicMax(&nodes[0].st.hi[threadIdx.x], sHi[threadIdx.x]);
    }
}

__global__ void __launch_bounds__(kWide) k_rr_root_sum(int nt, const RRec *__restrict__ rec, RNode *nodes,
                                                       int *scg)
{
    __shared__ long long sSum[3];
    __shared__ int sc[3];
    if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        double M = fmax(fabs(ord_to_dbl(nodes[0].st.lo[a])), fabs(ord_to_dbl(nodes[0].st.hi[a])));
        sc[a] = fixed_scale(M, nt);
        sSum[a] = 0;
        if (blockIdx.x == 0)
            scg[a] = sc[a];
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    long long s[3] = {0, 0, 0};
    if (i < nt)
        for (int a = 0; a < 3; ++a)
            s[a] = to_fixed(rec[i].c[a], sc[a]);
    for (int o = 16; o > 0; o >>= 1)
        for (int a = 0; a < 3; ++a)
            s[a] += __shfl_xor_sync(0xFFFFFFFFu, s[a], o);
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; ++a)
            atomicAdd(reinterpret_cast<unsigned long long *>(&sSum[a]), (unsigned long long)s[a]);
    __syncthreads();
    if (threadIdx.x < 3)
        atomicAdd(reinterpret_cast<unsigned long long *>(&nodes[0].st.sum[threadIdx.x]),
                  (unsigned long long)sSum[threadIdx.x]);
}

__global__ void k_rr_root_params(RNode *nodes, int nt, const int *scg, int *counters, int *terms)
{
    RNode &r = nodes[0];
    if (nt > kSub) {
        node_params(r.st.lo, r.st.hi, r.st.sum, nt, scg, r.axis, r.clo, r.chi);
        counters[kCtFirst] = 0;
        counters[kCtLast] = 1;
    } else {
        terms[0] = 0;
        counters[kCtTerms] = 1;
        counters[kCtFirst] = 1;
        counters[kCtLast] = 1;
    }
}

// ---------------------------------------------------------------------------------------------------
// Large-node phase, one level per (classify, resolve, children)
// ---------------------------------------------------------------------------------------------------

// Moves every member decided at the previous level into its child, then classifies the members of this
// level's large nodes against their intervals and accumulates the children's statistics. side[i]: -1 none
// pending, 0 left, 1 right, 2 inside the interval (resolved exactly by k_rr_resolve).
__global__ void __launch_bounds__(kWide) k_rr_classify(int nt, const int *__restrict__ counters,
                                                       const RRec *__restrict__ rec, int *nodeOf, int8_t *side,
                                                       RNode *nodes, const int *__restrict__ scg)
{
    constexpr int kTab = 64; // per-block table for levels with at most 32 nodes
    __shared__ RStat tab[kTab];
    __shared__ int sc[3];
    const int first = counters[kCtFirst], last = counters[kCtLast];
    if (first >= last)
        return;
    const bool small = last - first <= kTab / 2;
    if (threadIdx.x < 3)
        sc[threadIdx.x] = scg[threadIdx.x];
    if (small)
        for (int j = threadIdx.x; j < kTab; j += blockDim.x)
            rstat_clear(tab[j]);
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1;
    if (i < nt) {
        int p = nodeOf[i];
        const int s = side[i];
        if (s >= 0) {
            const int c = nodes[p].child;
            if (c >= 0) {
                p = c + s;
                nodeOf[i] = p;
            }
            side[i] = -1;
        }
        if (p >= first && p < last) {
            const RNode &nd = nodes[p];
            if (nd.count > kSub) {
                const unsigned long long o = ordc(rec[i].c[nd.axis]);
                const int sd = o < nd.clo ? 0 : (o >= nd.chi ? 1 : 2);
                side[i] = (int8_t)sd;
                if (sd == 2)
                    atomicOr(&nodes[p].flags, 1);
                else
                    key = (p - first) * 2 + sd;
            }
        }
    }
    EStat e = estat_of(key >= 0, rec[i < nt ? i : 0], sc);
    int len = 0;
    const bool tail = warp_segment_reduce(key, e, len);
    if (small) {
        if (tail && key >= 0)
            stat_atomic(tab[key], e, len);
        __syncthreads();
        for (int j = threadIdx.x; j < 2 * (last - first); j += blockDim.x)
            if (tab[j].count > 0) {
                EStat t;
                for (int k = 0; k < 3; ++k) {
                    t.lo[k] = tab[j].lo[k];
                    t.hi[k] = tab[j].hi[k];
                    t.s[k] = tab[j].sum[k];
                }
                stat_atomic(nodes[first + (j >> 1)].acc[j & 1], t, tab[j].count);
            }
    } else if (tail && key >= 0) {
        stat_atomic(nodes[first + (key >> 1)].acc[key & 1], e, len);
    }
}

// Nodes that need their member order: a member inside the interval (the reference's sequential sum in member
// order decides), or an empty side (the split takes halves of the member order). One block per such node
// lists its members by triangle index, then rewrites their sides and the children's statistics. Rare.
__global__ void __launch_bounds__(kWide) k_rr_resolve(int nt, int *counters, const RRec *__restrict__ rec,
                                                      const int *__restrict__ nodeOf, int8_t *side, RNode *nodes,
                                                      int *pool, const int *__restrict__ scg)
{
    __shared__ int warpSums[32];
    __shared__ int sOff, sLeft;
    __shared__ double sSplit;
    __shared__ RStat sAcc[2];
    const int first = counters[kCtFirst], last = counters[kCtLast];
    const int tid = threadIdx.x;
    int sc[3] = {scg[0], scg[1], scg[2]};
    for (int id = first + blockIdx.x; id < last; id += gridDim.x) {
        RNode &nd = nodes[id];
        const int n = nd.count;
        if (n <= kSub)
            continue;
        const bool amb = (nd.flags & 1) != 0;
        if (!amb && nd.acc[0].count > 0 && nd.acc[1].count > 0)
            continue;
        // members by ascending triangle index
        if (tid == 0) {
            sOff = atomicAdd(counters + kCtPool, n);
            sLeft = 0;
        }
        __syncthreads();
        int *list = pool + sOff;
        int got = 0;
        for (int b = 0; b < nt; b += blockDim.x) {
            const int i = b + tid;
            const int m = (i < nt && nodeOf[i] == id) ? 1 : 0;
            int tot;
            const int pos = block_exclusive_scan(m, tot, warpSums);
            if (m && got + pos < n)
                list[got + pos] = i;
            got += tot;
        }
        const int dir = nd.dir, axis = nd.axis;
        if (amb) {
            if (tid == 0) {
                double s = 0.0;
                for (int k = 0; k < n; ++k)
                    s = s + rec[list[dir ? n - 1 - k : k]].c[axis];
                sSplit = s / (double)(float)n;
            }
            __syncthreads();
        }
        // exact sides; count the left ones
        int myLeft = 0;
        for (int k = tid; k < n; k += blockDim.x) {
            const double c = rec[list[k]].c[axis];
            const bool left = amb ? (c < sSplit) : (ordc(c) < nd.clo);
            myLeft += left ? 1 : 0;
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
            if (k < n) {
                const int i = list[k];
                const int mp = dir ? n - 1 - k : k; // position in member order
                if (mode == 0) {
                    const double c = rec[i].c[axis];
                    sd = (amb ? (c < sSplit) : (ordc(c) < nd.clo)) ? 0 : 1;
                } else if (mode == 1) {
                    sd = mp < n / 2 ? 0 : 1;                  // all right, in member order: halves
                } else {
                    sd = (n - 1 - mp) < n - n / 2 ? 0 : 1;    // all left, reversed: halves
                }
                side[i] = (int8_t)sd;
            }
            // per-side statistics (list order is by index, so runs of equal side are common)
            EStat e = estat_of(sd >= 0, rec[k < n ? list[k] : 0], sc);
            int len = 0;
            if (warp_segment_reduce(sd, e, len) && sd >= 0)
                stat_atomic(sAcc[sd], e, len);
        }
        __syncthreads();
        if (tid < 2)
            nd.acc[tid] = sAcc[tid];
        if (tid == 0)
            nd.mode = mode;
        __syncthreads();
    }
}

// One block: allocates the children of every node split at this level, fills their statistics and split
// parameters, lists the terminal ones, and advances the level bounds.
__global__ void __launch_bounds__(kWide) k_rr_children(RNode *nodes, int *counters, int *terms, int maxNodes,
                                                       const int *__restrict__ scg)
{
    const int first = counters[kCtFirst], last = counters[kCtLast];
    if (first >= last)
        return;
    int sc[3] = {scg[0], scg[1], scg[2]};
    for (int id = first + threadIdx.x; id < last; id += blockDim.x) {
        RNode &nd = nodes[id];
        if (nd.count <= kSub)
            continue;
        const int c = atomicAdd(counters + kCtNodes, 2);
        if (c + 2 > maxNodes) {
            atomicAdd(counters + kCtOverflow, 1); // nothing is split further; the host reports the overflow
            continue;
        }
        const int mode = nd.mode, dir = nd.dir;
        const int dl = mode == 1 ? dir : dir ^ 1;
        const int dr = mode == 2 ? dir ^ 1 : dir;
        for (int s = 0; s < 2; ++s) {
            RNode &ch = nodes[c + s];
            ch.begin = s == 0 ? nd.begin : nd.begin + nd.acc[0].count;
            ch.count = nd.acc[s].count;
            ch.child = -1;
            ch.dir = s == 0 ? dl : dr;
            ch.axis = 0;
            ch.flags = 0;
            ch.mode = 0;
            ch.pad = 0;
            ch.st = nd.acc[s];
            rstat_clear(ch.acc[0]);
            rstat_clear(ch.acc[1]);
            if (ch.count > kSub)
                node_params(ch.st.lo, ch.st.hi, ch.st.sum, ch.count, sc, ch.axis, ch.clo, ch.chi);
            else
                terms[atomicAdd(counters + kCtTerms, 1)] = c + s;
        }
        nd.child = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        counters[kCtFirst] = last;
        counters[kCtLast] = counters[kCtNodes];
        counters[kCtPool] = 0;
    }
}

// after the last level: every member's terminal node and the sort key (the node's first leaf position)
__global__ void k_rr_finish(int nt, int *nodeOf, int8_t *side, const RNode *__restrict__ nodes, int *key,
                            int *val)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt)
        return;
    int p = nodeOf[i];
    const int s = side[i];
    if (s >= 0 && nodes[p].child >= 0) {
        p = nodes[p].child + s;
        nodeOf[i] = p;
    }
    key[i] = nodes[p].begin;
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

__global__ void __launch_bounds__(kSubThreads)
    k_rr_subtree(const int *__restrict__ terms, const RNode *__restrict__ gnodes, const int *__restrict__ sorted,
                 const RRec *__restrict__ rec, const int *__restrict__ scg, int *rank, int *counters)
{
    extern __shared__ __align__(16) unsigned char smem[];
    SNode *nodes = reinterpret_cast<SNode *>(smem);
    int(*nodeOf)[kSub] = reinterpret_cast<int(*)[kSub]>(smem + sizeof(SNode) * kSubNodes);
    int(*perm)[kSub] = reinterpret_cast<int(*)[kSub]>(smem + sizeof(SNode) * kSubNodes + sizeof(int) * 2 * kSub);
    int *flag = reinterpret_cast<int *>(smem + sizeof(SNode) * kSubNodes + sizeof(int) * 4 * kSub);
    int *scan = flag + kSub;
    int *warpSum = scan + kSub + 1;
    __shared__ int nNodes, lFirst, lLast, anyAmb, err;
    const int tid = threadIdx.x;
    const RNode &g = gnodes[terms[blockIdx.x]];
    const int base = g.begin, n = g.count, dir = g.dir;
    int sc[3] = {scg[0], scg[1], scg[2]};
    for (int p = tid; p < n; p += kSubThreads) {
        perm[0][p] = sorted[base + (dir ? n - 1 - p : p)];
        nodeOf[0][p] = 0;
    }
    if (n <= kLeaf) {
        __syncthreads();
        for (int p = tid; p < n; p += kSubThreads)
            rank[perm[0][p]] = base + p;
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
                    const unsigned long long o = ordc(rec[perm[cur][p]].c[nd.axis]);
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
                    s = s + rec[perm[cur][p]].c[nd.axis];
                const double split = s / (double)(float)nd.count;
                for (int p = nd.begin; p < nd.begin + nd.count; ++p)
                    flag[p] = rec[perm[cur][p]].c[nd.axis] < split ? 1 : 0;
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
        // statistics of the children that split again, read in the new order (members of a node are
        // contiguous, so the warp reduction sees runs)
        for (int p0 = 0; p0 < n; p0 += kSubThreads) {
            const int p = p0 + tid;
            const int id = p < n ? nodeOf[cur ^ 1][p] : -1;
            const int key = id >= 0 ? id : -1;
            EStat e = estat_of(key >= 0, rec[key >= 0 ? perm[cur ^ 1][p] : 0], sc);
            int len = 0;
            if (warp_segment_reduce(key, e, len) && key >= 0)
                stat_atomic_box(nodes[key], e);
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
        rank[perm[cur][p]] = base + p;
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

sb_status build_reference_rank(sb_mesh *m, cudaStream_t s)
{
    MeshDev &d = m->d;
    const int nt = d.nt;
    d.rankValid = false;
    if (nt <= 0)
        return SB_OK;
    KTime kt("reference_leaf_order", s);
    // large nodes have more than kSub members and are disjoint within a level
    const int maxNodes = 16 * (nt / kSub) + 256;
    const int keyBits = bit_length(nt);
    size_t sortBytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, sortBytes, (int *)nullptr, (int *)nullptr, (int *)nullptr,
                                    (int *)nullptr, nt, 0, keyBits, s);
    Carve c;
    const size_t o_rec = c.take<RRec>(nt), o_nodeOf = c.take<int>(nt), o_side = c.take<int8_t>(nt);
    const size_t o_key = c.take<int>(nt), o_val = c.take<int>(nt), o_skey = c.take<int>(nt),
                 o_sval = c.take<int>(nt), o_pool = c.take<int>(nt);
    const size_t o_nodes = c.take<RNode>(maxNodes), o_terms = c.take<int>(maxNodes), o_ct = c.take<int>(kCtCount),
                 o_sc = c.take<int>(4), o_cub = c.take<char>(sortBytes);
    SB_CUDA_CHECK(m->tmp.ensure(c.off));
    char *b = m->tmp.as<char>();
    RRec *rec = (RRec *)(b + o_rec);
    int *nodeOf = (int *)(b + o_nodeOf);
    int8_t *side = (int8_t *)(b + o_side);
    int *key = (int *)(b + o_key), *val = (int *)(b + o_val), *skey = (int *)(b + o_skey), *sval = (int *)(b + o_sval);
    int *pool = (int *)(b + o_pool);
    RNode *nodes = (RNode *)(b + o_nodes);
    int *terms = (int *)(b + o_terms), *counters = (int *)(b + o_ct), *scg = (int *)(b + o_sc);

    const int GW = (nt + kWide - 1) / kWide;
    SB_COUNT(k_rr_init)<<<1, 1, 0, s>>>(nodes, nt, counters);
    SB_COUNT(k_rr_elems)<<<GW, kWide, 0, s>>>(nt, d.v, d.t, d.box64, rec, nodeOf, side, nodes);
    SB_COUNT(k_rr_root_sum)<<<GW, kWide, 0, s>>>(nt, rec, nodes, scg);
    SB_COUNT(k_rr_root_params)<<<1, 1, 0, s>>>(nodes, nt, scg, counters, terms);
    // levels run in batches; the host looks at the level bounds only between batches. The first batch
    // covers the expected depth of the large-node phase (a mean split roughly halves); empty levels cost
    // only their launches.
    int expected = 0;
    while ((nt >> expected) > kSub)
        ++expected;
    bool done = nt <= kSub;
    int cnt[kCtCount] = {0};
    for (int level = 0, batch = expected + 1; level < 4096 && !done; level += batch, batch = 2) {
        for (int j = 0; j < batch; ++j) {
            SB_COUNT(k_rr_classify)<<<GW, kWide, 0, s>>>(nt, counters, rec, nodeOf, side, nodes, scg);
            SB_COUNT(k_rr_resolve)<<<152, kWide, 0, s>>>(nt, counters, rec, nodeOf, side, nodes, pool, scg);
            SB_COUNT(k_rr_children)<<<1, kWide, 0, s>>>(nodes, counters, terms, maxNodes, scg);
        }
        SB_CUDA_CHECK(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, s));
        SB_CUDA_CHECK(cudaStreamSynchronize(s));
        if (cnt[kCtOverflow] != 0) {
            set_last_error("reference tree node capacity exceeded");
            return SB_ERR_CAPACITY;
        }
        done = cnt[kCtFirst] >= cnt[kCtLast];
    }
    if (!done) {
        set_last_error("reference tree deeper than 4096 levels");
        return SB_ERR_CAPACITY;
    }
    if (nt <= kSub)
        cnt[kCtTerms] = 1;
    SB_COUNT(k_rr_finish)<<<GW, kWide, 0, s>>>(nt, nodeOf, side, nodes, key, val);
    SB_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(b + o_cub, sortBytes, key, skey, val, sval, nt, 0, keyBits, s));
    SB_CUDA_CHECK(cudaFuncSetAttribute(k_rr_subtree, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSubSmem));
    SB_COUNT(k_rr_subtree)<<<cnt[kCtTerms], kSubThreads, kSubSmem, s>>>(terms, nodes, sval, rec, scg, d.rank,
                                                                        counters);
    int errs = 0;
    SB_CUDA_CHECK(cudaMemcpyAsync(&errs, counters + kCtSubErr, sizeof errs, cudaMemcpyDeviceToHost, s));
    SB_CUDA_CHECK(cudaStreamSynchronize(s));
    if (errs) {
        set_last_error("reference tree: a subtree exceeded its node records");
        return SB_ERR_CAPACITY;
    }
    SB_CUDA_CHECK(cudaGetLastError());
    d.rankValid = true;
    return SB_OK;
}

} // namespace sbg
