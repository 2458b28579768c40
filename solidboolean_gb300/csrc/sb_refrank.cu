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
    kCtFirst = 4,   // current level: first node
    kCtLast = 5,    //                one past the last node
    kCtSubErr = 6,  // subtree blocks that ran out of node records
    kCtCount = 8
};

// one triangle: its box centre and box (stored by Morton position)
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

// Merges a run's box and sum into an accumulator; sums add as two's complement. A box bound only moves one
// way, so a bound that the stored value already beats needs no atomic (a stale read only costs one).
__device__ __forceinline__ void stat_atomic(RStat &dst, const EStat &e, int len)
{
    // all six reads in flight together; plain loads, since the accumulator may live in shared memory
    unsigned long long curLo[3], curHi[3];
    for (int k = 0; k < 3; ++k) {
        curLo[k] = dst.lo[k];
        curHi[k] = dst.hi[k];
    }
    for (int k = 0; k < 3; ++k) {
        if (e.lo[k] < curLo[k])
            atomicMin(&dst.lo[k], e.lo[k]);
        if (e.hi[k] > curHi[k])
            atomicMax(&dst.hi[k], e.hi[k]);
        if (e.s[k] != 0)
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
// it; `target(key)` names the accumulator of a key.
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
    __syncthreads();
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

__global__ void k_rr_init(RNode *nodes, NParam *np, int nt, int *counters)
{
    node_clear(nodes[0], 0, nt, 0);
    np[0] = NParam{-1, nt, 0, 0, 0ull, 0ull};
    for (int i = 0; i < kCtCount; ++i)
        counters[i] = 0;
    counters[kCtNodes] = 1;
}

// Box centre of each triangle as AxisAlignedBoudingBox::updateCenter computes it, (((0 + v0) + v1) + v2) /
// (float)3 (src/axisalignedboundingbox.h:31-53), its box, and the root box (src/solidmesh.cpp:68-72).
// Records are stored in Morton order (position p holds triangle leafTri[p]): member order is carried by the
// direction bits, so the processing order is free, and in Morton order a node's members form long runs.
__global__ void __launch_bounds__(kElemThreads) k_rr_elems(int nt, const double *__restrict__ v,
                                                           const uint32_t *__restrict__ t,
                                                           const double *__restrict__ box64,
                                                           const int *__restrict__ leafTri, RRec *rec, int *posOf,
                                                           int *state, RNode *nodes)
{
    __shared__ unsigned long long sLo[3], sHi[3];
    if (threadIdx.x < 3) {
        sLo[threadIdx.x] = ~0ull;
        sHi[threadIdx.x] = 0ull;
    }
    __syncthreads();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    if (p < nt) {
        const int i = leafTri[p];
        RRec r;
        for (int a = 0; a < 3; ++a) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                s = s + v[3 * (size_t)t[3 * (size_t)i + k] + a];
            r.c[a] = div3_rn(s);
            r.lo[a] = box64[6 * (size_t)i + a];
            r.hi[a] = box64[6 * (size_t)i + 3 + a];
            lo[a] = ordc(r.lo[a]);
            hi[a] = ordc(r.hi[a]);
        }
        rec[p] = r;
        posOf[i] = p;
        state[p] = 0;
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

__global__ void __launch_bounds__(kElemThreads) k_rr_root_sum(int nt, const RRec *__restrict__ rec, RNode *nodes,
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

__global__ void k_rr_root_params(RNode *nodes, NParam *np, int nt, const int *scg, int *counters, int *terms)
{
    RNode &r = nodes[0];
    if (nt > kSub) {
        NParam q{-1, nt, 0, 0, 0ull, 0ull};
        node_params(r.st.lo, r.st.hi, r.st.sum, nt, scg, q.axis, q.clo, q.chi);
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

// ---------------------------------------------------------------------------------------------------
// Large-node phase, one level per (classify, children)
// ---------------------------------------------------------------------------------------------------

// Moves every member decided at the previous level into its child, then classifies the members of this
// level's large nodes against their intervals and accumulates the children's statistics. Indexed by Morton
// position.
__global__ void __launch_bounds__(kElemThreads, 4) k_rr_classify(int nt, const int *__restrict__ counters,
                                                                 const RRec *__restrict__ rec, int *state,
                                                                 const NParam *__restrict__ np, RNode *nodes,
                                                                 const int *__restrict__ scg)
{
    __shared__ RunRec runs[kRunCap];
    __shared__ int warpRuns[kElemThreads / 32];
    const int first = counters[kCtFirst], last = counters[kCtLast];
    if (first >= last)
        return;
    const int sc[3] = {scg[0], scg[1], scg[2]};
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    RRec r;
    if (p < nt)
        r = rec[p];
    int key = -1;
    if (p < nt) {
        const int v = state[p];
        int node = st_node(v), tag = st_tag(v);
        if (tag == 1 || tag == 2) {
            const int c = np[node].child;
            if (c >= 0)
                node = c + tag - 1;
            tag = 0;
        }
        if (node >= first && node < last) {
            const NParam q = np[node];
            if (q.count > kSub) {
                const double c = q.axis == 0 ? r.c[0] : (q.axis == 1 ? r.c[1] : r.c[2]); // no local array
                const unsigned long long o = ordc(c);
                const int sd = o < q.clo ? 0 : (o >= q.chi ? 1 : 2);
                tag = sd + 1;
                if (sd == 2)
                    atomicOr(&nodes[node].flags, 1);
                else
                    key = (node - first) * 2 + sd;
            }
        }
        const int nv = (node << 2) | tag;
        if (nv != v)
            state[p] = nv;
    }
    const EStat e = estat_of(key >= 0, r, sc);
    block_reduce_keys(key, e, key >= 0 ? 1 : 0, runs, warpRuns,
                      [&](int k) -> RStat & { return nodes[first + (k >> 1)].acc[k & 1]; });
}

// Exact sides of one node whose member order matters: a member inside the interval (the reference's
// sequential sum in member order decides), or an empty side (the split takes halves of the member order).
// Run by the whole block; lists the members by triangle index, rewrites their state words and the children's
// statistics. Rare.
__device__ void resolve_node(int id, int nt, const RRec *__restrict__ rec, int *state, const NParam &q,
                             RNode &nd, int *list, const int *__restrict__ posOf, const int *sc, int *warpSums,
                             RunRec *runs, RStat *sAcc, int &sLeft, double &sSplit)
{
    const int tid = threadIdx.x;
    const int n = q.count;
    const bool amb = (nd.flags & 1) != 0;
    if (tid == 0)
        sLeft = 0;
    int got = 0;
    for (int b = 0; b < nt; b += blockDim.x) {
        const int i = b + tid; // triangle index
        const int pos = i < nt ? posOf[i] : 0;
        const int m = (i < nt && st_node(state[pos]) == id) ? 1 : 0;
        int tot;
        const int at = block_exclusive_scan(m, tot, warpSums);
        if (m && got + at < n)
            list[got + at] = pos;
        got += tot;
    }
    const int dir = nd.dir, axis = q.axis;
    if (amb) {
        if (tid == 0) {
            double s = 0.0;
            for (int k = 0; k < n; ++k)
                s = s + rec[list[dir ? n - 1 - k : k]].c[axis];
            sSplit = s / (double)(float)n;
        }
        __syncthreads();
    }
    int myLeft = 0;
    for (int k = tid; k < n; k += blockDim.x) {
        const double c = rec[list[k]].c[axis];
        myLeft += (amb ? (c < sSplit) : (ordc(c) < q.clo)) ? 1 : 0;
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
            const int pos = list[k];
            const int mp = dir ? n - 1 - k : k; // position in member order
            if (mode == 0) {
                const double c = rec[pos].c[axis];
                sd = (amb ? (c < sSplit) : (ordc(c) < q.clo)) ? 0 : 1;
            } else if (mode == 1) {
                sd = mp < n / 2 ? 0 : 1;               // all right, in member order: halves
            } else {
                sd = (n - 1 - mp) < n - n / 2 ? 0 : 1; // all left, reversed: halves
            }
            state[pos] = (id << 2) | (sd + 1);
        }
        const EStat e = estat_of(sd >= 0, rec[k < n ? list[k] : 0], sc);
        block_reduce_keys(sd, e, sd >= 0 ? 1 : 0, runs, warpSums, [&](int qq) -> RStat & { return sAcc[qq]; });
    }
    if (tid < 2)
        nd.acc[tid] = sAcc[tid];
    if (tid == 0) {
        nd.mode = mode;
        nd.flags = 0;
    }
    __syncthreads();
}

// One block per level: resolves the rare nodes that need their member order, allocates the children of every
// node split at this level (block scans, no atomics), fills their statistics and split parameters, lists the
// terminal ones, and advances the level bounds.
__global__ void __launch_bounds__(kWide) k_rr_children(int nt, RNode *nodes, NParam *np, int *counters, int *terms,
                                                       int maxNodes, const RRec *__restrict__ rec, int *state,
                                                       const int *__restrict__ posOf, int *pool,
                                                       const int *__restrict__ scg)
{
    __shared__ int warpSums[32];
    __shared__ RunRec runs[kRunCap];
    __shared__ RStat sAcc[2];
    __shared__ int sLeft, nFlag;
    __shared__ double sSplit;
    __shared__ int flagged[kWide];
    const int first = counters[kCtFirst], last = counters[kCtLast];
    if (first >= last)
        return;
    const int tid = threadIdx.x;
    const int sc[3] = {scg[0], scg[1], scg[2]};
    // nodes that need the exact, order-aware resolution
    for (int b = first; b < last; b += kWide) {
        if (tid == 0)
            nFlag = 0;
        __syncthreads();
        const int id = b + tid;
        if (id < last) {
            const RNode &nd = nodes[id];
            if (nd.count > kSub && ((nd.flags & 1) || nd.acc[0].count == 0 || nd.acc[1].count == 0))
                flagged[atomicAdd(&nFlag, 1)] = id;
        }
        __syncthreads();
        const int nf = nFlag;
        for (int f = 0; f < nf; ++f) {
            const int fid = flagged[f];
            const NParam q = np[fid];
            resolve_node(fid, nt, rec, state, q, nodes[fid], pool, posOf, sc, warpSums, runs, sAcc, sLeft, sSplit);
        }
        __syncthreads();
    }
    // children
    int nodeBase = counters[kCtNodes], termBase = counters[kCtTerms];
    bool overflow = false;
    for (int b = first; b < last; b += kWide) {
        const int id = b + tid;
        const RNode *nd = id < last ? &nodes[id] : nullptr;
        const int split = (nd && nd->count > kSub) ? 1 : 0;
        int totSplit;
        const int at = block_exclusive_scan(split, totSplit, warpSums);
        const int c = nodeBase + 2 * at;
        const bool ok = split && c + 2 <= maxNodes;
        overflow |= split && !ok;
        int nTerm = 0, cnt[2] = {0, 0};
        if (ok) {
            const int mode = nd->mode, dir = nd->dir;
            const int dl = mode == 1 ? dir : dir ^ 1;
            const int dr = mode == 2 ? dir ^ 1 : dir;
            for (int s2 = 0; s2 < 2; ++s2) {
                cnt[s2] = nd->acc[s2].count;
                RNode &ch = nodes[c + s2];
                ch.begin = s2 == 0 ? nd->begin : nd->begin + nd->acc[0].count;
                ch.count = cnt[s2];
                ch.dir = s2 == 0 ? dl : dr;
                ch.flags = 0;
                ch.mode = 0;
                ch.pad[0] = ch.pad[1] = ch.pad[2] = 0;
                ch.st = nd->acc[s2];
                rstat_clear(ch.acc[0]);
                rstat_clear(ch.acc[1]);
                NParam cq{-1, cnt[s2], 0, 0, 0ull, 0ull};
                if (cnt[s2] > kSub)
                    node_params(ch.st.lo, ch.st.hi, ch.st.sum, cnt[s2], sc, cq.axis, cq.clo, cq.chi);
                else
                    ++nTerm;
                np[c + s2] = cq;
            }
            np[id].child = c;
        }
        int totTerm;
        const int tat = block_exclusive_scan(nTerm, totTerm, warpSums);
        if (ok) {
            int t2 = termBase + tat;
            for (int s2 = 0; s2 < 2; ++s2)
                if (cnt[s2] <= kSub)
                    terms[t2++] = c + s2;
        }
        nodeBase += 2 * totSplit;
        termBase += totTerm;
    }
    overflow = __syncthreads_or(overflow);
    if (tid == 0) {
        counters[kCtNodes] = nodeBase < maxNodes ? nodeBase : maxNodes;
        counters[kCtTerms] = termBase;
        if (overflow)
            counters[kCtOverflow] = 1;
        counters[kCtFirst] = last;
        counters[kCtLast] = overflow ? last : counters[kCtNodes];
    }
}

// After the last level: every member's terminal node, and the sort key (the node's first leaf position)
// stored by triangle index, so that a stable sort lists each node's members by ascending index.
__global__ void k_rr_finish(int nt, const int *__restrict__ state, const NParam *__restrict__ np,
                            const RNode *__restrict__ nodes, const int *__restrict__ leafTri, int *key, int *val)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
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

__global__ void __launch_bounds__(kSubThreads)
    k_rr_subtree(const int *__restrict__ terms, const RNode *__restrict__ gnodes, const int *__restrict__ sorted,
                 const RRec *__restrict__ rec, const int *__restrict__ posOf, const int *__restrict__ leafTri,
                 const int *__restrict__ scg, int *rank, int *counters)
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
        // Statistics of the children that split again, read in the new order. A node's members are
        // contiguous, so each warp's runs end either at a node's last member (that run's total goes to the
        // node) or at the warp's last lane (kept per 32-position chunk); one thread per node then adds the
        // chunk totals inside its range. No atomics.
        EStat *chunk = reinterpret_cast<EStat *>(scan); // the scan is consumed; kSub / 32 entries fit
        for (int p0 = 0; p0 < n; p0 += kSubThreads) {
            const int p = p0 + tid;
            const int id = p < n ? nodeOf[cur ^ 1][p] : -1;
            const int key = id >= 0 ? id : -1;
            EStat e = estat_of(key >= 0, rec[key >= 0 ? perm[cur ^ 1][p] : 0], sc);
            int len = 1;
            if (warp_segment_reduce(key, e, len) && key >= 0) {
                SNode &nd = nodes[key];
                if (p == nd.begin + nd.count - 1) {
                    for (int k = 0; k < 3; ++k) {
                        nd.lo[k] = e.lo[k];
                        nd.hi[k] = e.hi[k];
                        nd.sum[k] = e.s[k];
                    }
                } else {
                    chunk[p >> 5] = e; // p is the last position of its chunk
                }
            }
        }
        __syncthreads();
        for (int id = last + tid; id < nNodes; id += kSubThreads) {
            SNode &nd = nodes[id];
            if (nd.count <= kLeaf)
                continue;
            const int b = nd.begin, e = nd.begin + nd.count - 1; // chunk ends in [b, e) belong to the node
            for (int j = b >> 5; 32 * j + 31 < e; ++j) { // 32 (b / 32) + 31 is the first chunk end >= b
                const EStat &c = chunk[j];
                for (int k = 0; k < 3; ++k) {
                    nd.lo[k] = min(nd.lo[k], c.lo[k]);
                    nd.hi[k] = max(nd.hi[k], c.hi[k]);
                    nd.sum[k] += c.s[k];
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
    const size_t o_rec = c.take<RRec>(nt), o_state = c.take<int>(nt), o_pos = c.take<int>(nt);
    const size_t o_key = c.take<int>(nt), o_val = c.take<int>(nt), o_skey = c.take<int>(nt),
                 o_sval = c.take<int>(nt), o_pool = c.take<int>(nt);
    const size_t o_np = c.take<NParam>(maxNodes);
    const size_t o_nodes = c.take<RNode>(maxNodes), o_terms = c.take<int>(maxNodes), o_ct = c.take<int>(kCtCount),
                 o_sc = c.take<int>(4), o_cub = c.take<char>(sortBytes);
    SB_CUDA_CHECK(m->tmp.ensure(c.off));
    char *b = m->tmp.as<char>();
    RRec *rec = (RRec *)(b + o_rec);
    int *state = (int *)(b + o_state);
    NParam *np = (NParam *)(b + o_np);
    int *key = (int *)(b + o_key), *val = (int *)(b + o_val), *skey = (int *)(b + o_skey), *sval = (int *)(b + o_sval);
    int *pool = (int *)(b + o_pool), *posOf = (int *)(b + o_pos);
    RNode *nodes = (RNode *)(b + o_nodes);
    int *terms = (int *)(b + o_terms), *counters = (int *)(b + o_ct), *scg = (int *)(b + o_sc);

    const int GE = (nt + kElemThreads - 1) / kElemThreads;
    SB_COUNT(k_rr_init)<<<1, 1, 0, s>>>(nodes, np, nt, counters);
    SB_COUNT(k_rr_elems)<<<GE, kElemThreads, 0, s>>>(nt, d.v, d.t, d.box64, d.leafTri, rec, posOf, state, nodes);
    SB_COUNT(k_rr_root_sum)<<<GE, kElemThreads, 0, s>>>(nt, rec, nodes, scg);
    SB_COUNT(k_rr_root_params)<<<1, 1, 0, s>>>(nodes, np, nt, scg, counters, terms);
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
            SB_COUNT(k_rr_classify)<<<GE, kElemThreads, 0, s>>>(nt, counters, rec, state, np, nodes, scg);
            SB_COUNT(k_rr_children)<<<1, kWide, 0, s>>>(nt, nodes, np, counters, terms, maxNodes, rec, state, posOf,
                                                        pool, scg);
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
    SB_COUNT(k_rr_finish)<<<GE, kElemThreads, 0, s>>>(nt, state, np, nodes, d.leafTri, key, val);
    SB_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(b + o_cub, sortBytes, key, skey, val, sval, nt, 0, keyBits, s));
    SB_CUDA_CHECK(cudaFuncSetAttribute(k_rr_subtree, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSubSmem));
    SB_COUNT(k_rr_subtree)<<<cnt[kCtTerms], kSubThreads, kSubSmem, s>>>(terms, nodes, sval, rec, posOf, d.leafTri, scg, d.rank,
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
