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
// The tree (src/axisalignedboundingboxtree.cpp:27-45, 71-141): a node with more than 20 boxes splits on the
// longest axis of its box (spans compared as float, first maximum wins) at the mean of its box centres
// (sequential sum in member order divided by (float)count); boxes with centre < mean go left in reverse
// order of appearance, the others right in order; an empty side takes half of the other.
//
// Built level by level: every node's members are a contiguous segment of one permutation. The mean is
// needed exactly only through the comparisons centre < mean. Each node's sum is accumulated in parallel
// with a rigorous bound on its distance to the sequential sum (2 gamma_n sum|c|), giving an interval that
// contains the reference's mean; a member outside the interval is classified exactly, and a node with any
// member inside it recomputes the sequential sum in member order (one thread) before classifying.
#include <cub/cub.cuh>

#include "sb_common.cuh"
#include "sb_internal.h"
#include "sb_ktime.h"

namespace sbg {

// nodes with at most kSub members are finished by one block each (k_rr_subtree)
constexpr int kSub = 2048;
constexpr int kSubThreads = 256;
constexpr int kSubNodes = 512;

struct RNode {
    int begin, count;
    int axis, leftFinal, child; // child: id of the left child (right = child + 1), -1 for a leaf
    int ambiguous;
    double clo, chi;            // interval holding the reference's split value on `axis`
    unsigned long long lo[3], hi[3]; // box (order-preserving integer encoding of doubles)
    double sum[3], asum[3];          // approximate sum of member centres and of their magnitudes
};

// one triangle's data, kept physically in the current permutation order so every pass reads it coalesced
struct RElem {
    double c[3];   // box centre
    double bx[6];  // box lo xyz, hi xyz
    int tri;
    int pad;
};

__device__ __forceinline__ void rnode_init(RNode &n, int begin, int count)
{
    n.begin = begin;
    n.count = count;
    n.axis = 0;
    n.leftFinal = 0;
    n.child = -1;
    n.ambiguous = 0;
    n.clo = n.chi = 0.0;
    for (int k = 0; k < 3; ++k) {
        n.lo[k] = ~0ull;
        n.hi[k] = 0ull;
        n.sum[k] = 0.0;
        n.asum[k] = 0.0;
    }
}

// box centre of each triangle, exactly as AxisAlignedBoudingBox::updateCenter computes it
// (((0 + v0) + v1) + v2) / (float)3 (src/axisalignedboundingbox.h:31-53)
__global__ void k_rr_centres(int nt, const double *__restrict__ v, const uint32_t *__restrict__ t,
                             const double *__restrict__ box64, RElem *rec, int *nodeOf)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt)
        return;
    RElem e;
    for (int a = 0; a < 3; ++a) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k)
            s = s + v[3 * (size_t)t[3 * (size_t)i + k] + a];
        e.c[a] = s / 3.0;
    }
    for (int k = 0; k < 6; ++k)
        e.bx[k] = box64[6 * (size_t)i + k];
    e.tri = i;
    e.pad = 0;
    rec[i] = e;
    nodeOf[i] = 0;
}

// adds the members of node `node` (positions p) into that node's box and sums, one atomic per warp when
// the whole warp belongs to the same node
__device__ __forceinline__ void rr_accumulate(RNode *nodes, int node, const double *c, const double *bx)
{
    const unsigned full = 0xFFFFFFFFu;
    unsigned mask = __activemask();
    int lead = __shfl_sync(mask, node, __ffs(mask) - 1);
    bool uniform = (mask == full) && __all_sync(full, node == lead);
    unsigned long long lo[3], hi[3];
    double s[3], as[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = dbl_to_ord(bx[k]);
        hi[k] = dbl_to_ord(bx[3 + k]);
        s[k] = c[k];
        as[k] = fabs(c[k]);
    }
    if (uniform) {
        for (int o = 16; o > 0; o >>= 1)
            for (int k = 0; k < 3; ++k) {
                lo[k] = min(lo[k], __shfl_xor_sync(full, lo[k], o));
                hi[k] = max(hi[k], __shfl_xor_sync(full, hi[k], o));
                s[k] += __shfl_xor_sync(full, s[k], o);
                as[k] += __shfl_xor_sync(full, as[k], o);
            }
        if ((threadIdx.x & 31) != 0)
            return;
    }
    RNode &n = nodes[node];
    for (int k = 0; k < 3; ++k) {
        atomicMin(&n.lo[k], lo[k]);
        atomicMax(&n.hi[k], hi[k]);
        atomicAdd(&n.sum[k], s[k]);
        atomicAdd(&n.asum[k], as[k]);
    }
}

// all threads of the block call this; a block whose valid threads all belong to one node reduces in
// shared memory first (one set of atomics per block), other blocks fall back to warp-level reduction
__device__ void rr_block_accumulate(RNode *nodes, int node, const double *c, const double *bx)
{
    __shared__ int sNode;
    __shared__ unsigned long long sLo[32][3], sHi[32][3];
    __shared__ double sSum[32][3], sAbs[32][3];
    if (threadIdx.x == 0)
        sNode = node;
    __syncthreads();
    const bool uniform = __syncthreads_and(node == sNode) && sNode >= 0;
    if (!uniform) {
        if (node >= 0)
            rr_accumulate(nodes, node, c, bx);
        return;
    }
    const unsigned full = 0xFFFFFFFFu;
    unsigned long long lo[3], hi[3];
    double sm[3], as[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = dbl_to_ord(bx[k]);
        hi[k] = dbl_to_ord(bx[3 + k]);
        sm[k] = c[k];
        as[k] = fabs(c[k]);
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 3; ++k) {
            lo[k] = min(lo[k], __shfl_xor_sync(full, lo[k], o));
            hi[k] = max(hi[k], __shfl_xor_sync(full, hi[k], o));
            sm[k] += __shfl_xor_sync(full, sm[k], o);
            as[k] += __shfl_xor_sync(full, as[k], o);
        }
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; ++k) {
            sLo[w][k] = lo[k];
            sHi[w][k] = hi[k];
            sSum[w][k] = sm[k];
            sAbs[w][k] = as[k];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        unsigned long long l = ~0ull, h = 0ull;
        double a = 0.0, b = 0.0;
        for (int i = 0; i < nw; ++i) {
            l = min(l, sLo[i][k]);
            h = max(h, sHi[i][k]);
            a += sSum[i][k];
            b += sAbs[i][k];
        }
        RNode &n = nodes[node];
        atomicMin(&n.lo[k], l);
        atomicMax(&n.hi[k], h);
        atomicAdd(&n.sum[k], a);
        atomicAdd(&n.asum[k], b);
    }
}

__global__ void k_rr_root(int nt, const RElem *__restrict__ rec, RNode *nodes)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int node = i < nt ? 0 : -1;
    const RElem &e = rec[i < nt ? i : 0];
    rr_block_accumulate(nodes, node, e.c, e.bx);
}

// gamma_n = n u / (1 - n u), rounded up
__device__ __forceinline__ double rr_gamma(int n)
{
    const double u = 1.1102230246251565e-16;
    double nu = __dmul_ru((double)n, u);
    return __ddiv_ru(nu, __dsub_rd(1.0, nu));
}

// bounds[0..1]: first and one-past-last node of the current level; counters[1] counts leaves
__global__ void k_rr_prep(const int *__restrict__ bounds, RNode *nodes, int *counters, int *deferred)
{
    const int first = bounds[0], last = bounds[1];
    for (int id = first + blockIdx.x * blockDim.x + threadIdx.x; id < last; id += gridDim.x * blockDim.x) {
        RNode &n = nodes[id];
        if (n.count <= kSub) {
            n.child = -1;
            if (n.count <= 20)
                atomicAdd(counters + 1, 1);
            else
                deferred[atomicAdd(counters + 6, 1)] = id;
            continue;
        }
        float span[3];
        for (int k = 0; k < 3; ++k)
            span[k] = __double2float_rn(ord_to_dbl(n.hi[k]) - ord_to_dbl(n.lo[k]));
        int axis = 0;
        for (int k = 1; k < 3; ++k)
            if (span[axis] < span[k])
                axis = k;
        n.axis = axis;
        // |sequential - approximate| <= 2 gamma_n sum|c|, with sum|c| itself known to within gamma_n
        double g = rr_gamma(n.count + 1);
        double aup = __dmul_ru(n.asum[axis], __dadd_ru(1.0, __dmul_ru(2.0, g)));
        double err = __dmul_ru(__dmul_ru(2.0, g), aup);
        err = __dadd_ru(err, 1e-300);
        double cnt = (double)(float)n.count;
        n.clo = __ddiv_rd(__dsub_rd(n.sum[axis], err), cnt);
        n.chi = __ddiv_ru(__dadd_ru(n.sum[axis], err), cnt);
        n.ambiguous = 0;
    }
}

// flag: 1 = left, 0 = right; positions of leaves are left untouched (flag 0)
__global__ void k_rr_classify(int nt, const int *__restrict__ bounds, const RElem *__restrict__ rec,
                              const int *__restrict__ nodeOf, RNode *nodes, int *flag)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nt || bounds[0] >= bounds[1])
        return;
    int id = nodeOf[p];
    int f = 0;
    if (id >= bounds[0]) {
        RNode &n = nodes[id];
        if (n.count > kSub) {
            double c = rec[p].c[n.axis];
            if (c < n.clo)
                f = 1;
            else if (!(c >= n.chi))
                atomicOr(&n.ambiguous, 1);
        }
    }
    flag[p] = f;
}

// nodes whose interval could not decide every member: the reference's sequential sum, in member order
__global__ void k_rr_resolve(const int *__restrict__ bounds, const RElem *__restrict__ rec, RNode *nodes,
                             int *flag)
{
    const int first = bounds[0], last = bounds[1];
    for (int id = first + blockIdx.x * blockDim.x + threadIdx.x; id < last; id += gridDim.x * blockDim.x) {
        RNode &n = nodes[id];
        if (n.count <= kSub || !n.ambiguous)
            continue;
        double s = 0.0;
        for (int p = n.begin; p < n.begin + n.count; ++p)
            s = s + rec[p].c[n.axis];
        double split = s / (double)(float)n.count;
        for (int p = n.begin; p < n.begin + n.count; ++p)
            flag[p] = rec[p].c[n.axis] < split ? 1 : 0;
    }
}

__global__ void k_rr_children(const int *__restrict__ bounds, const int *__restrict__ scan, RNode *nodes,
                              int *counters, int maxNodes)
{
    const int first = bounds[0], last = bounds[1];
    for (int id = first + blockIdx.x * blockDim.x + threadIdx.x; id < last; id += gridDim.x * blockDim.x) {
        RNode &n = nodes[id];
        if (n.count <= kSub)
            continue;
        int left = scan[n.begin + n.count] - scan[n.begin];
        int right = n.count - left;
        int leftFinal = left;
        if (left == 0)
            leftFinal = right / 2;
        else if (right == 0)
            leftFinal = left - left / 2;
        int c = atomicAdd(counters, 2);
        if (c + 2 > maxNodes) {
            // out of node records: nothing is written, the host reports a capacity error
            n.count = 0;
            atomicAdd(counters + 3, 1);
            continue;
        }
        n.leftFinal = leftFinal;
        n.child = c;
        rnode_init(nodes[c], n.begin, leftFinal);
        rnode_init(nodes[c + 1], n.begin + leftFinal, n.count - leftFinal);
    }
}

// nodeOf: >= 0 node of the current level, -2 settled in a leaf with its record already in both buffers
__global__ void k_rr_scatter(int nt, const int *__restrict__ bounds, const RElem *__restrict__ rec,
                             const int *__restrict__ nodeOf, const int *__restrict__ flag,
                             const int *__restrict__ scan, const RNode *nodes, RElem *rec2, int *nodeOf2)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nt || bounds[0] >= bounds[1])
        return;
    int id = nodeOf[p];
    if (id == -2) {
        nodeOf2[p] = -2;
        return;
    }
    if (id < 0 || id < bounds[0] || nodes[id].count <= kSub) {
        rec2[p] = rec[p]; // settled in a leaf: one copy makes it final in both buffers
        nodeOf2[p] = -2;
        return;
    }
    const RNode &n = nodes[id];
    int left = scan[n.begin + n.count] - scan[n.begin];
    int lrank = scan[p] - scan[n.begin];
    int rrank = (p - n.begin) - lrank;
    int pos;
    if (left == 0)
        pos = rrank;
    else if (left == n.count)
        pos = n.count - 1 - lrank;
    else
        pos = flag[p] ? (left - 1 - lrank) : (left + rrank);
    int q = n.begin + pos;
    rec2[q] = rec[p];
    nodeOf2[q] = pos < n.leftFinal ? n.child : n.child + 1;
}

__global__ void k_rr_child_stats(int nt, const int *__restrict__ bounds, const RElem *__restrict__ rec,
                                 const int *__restrict__ nodeOf, RNode *nodes)
{
    // an empty level wrote no indices: the other buffer still holds an older level's (block-uniform exit)
    if (bounds[0] >= bounds[1])
        return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int id = p < nt ? nodeOf[p] : -1;
    const RElem &e = rec[id >= 0 ? p : 0];
    rr_block_accumulate(nodes, id < 0 ? -1 : id, e.c, e.bx);
}


// ---------------------------------------------------------------------------------------------------
// One block finishes the subtree of one node with at most kSub members: the same level loop as above,
// with the node records and per-element state in shared memory and __syncthreads between the steps.
// ---------------------------------------------------------------------------------------------------
struct SNode {
    int begin, count, axis, leftFinal, child, ambiguous;
    double clo, chi;
    unsigned long long lo[3], hi[3];
    double sum[3], asum[3];
};

__device__ __forceinline__ void snode_init(SNode &n, int begin, int count)
{
    n.begin = begin;
    n.count = count;
    n.axis = 0;
    n.leftFinal = 0;
    n.child = -1;
    n.ambiguous = 0;
    n.clo = n.chi = 0.0;
    for (int k = 0; k < 3; ++k) {
        n.lo[k] = ~0ull;
        n.hi[k] = 0ull;
        n.sum[k] = 0.0;
        n.asum[k] = 0.0;
    }
}

// warp-reduced accumulation into a shared-memory node (lanes of one node combine first)
__device__ __forceinline__ void snode_accumulate(SNode *nodes, int node, const RElem &e, bool valid)
{
    const unsigned full = 0xFFFFFFFFu;
    int key = valid ? node : -1;
    int lead = __shfl_sync(full, key, 0);
    bool uniform = __all_sync(full, key == lead) && lead >= 0;
    unsigned long long lo[3], hi[3];
    double sm[3], as[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = valid ? dbl_to_ord(e.bx[k]) : ~0ull;
        hi[k] = valid ? dbl_to_ord(e.bx[3 + k]) : 0ull;
        sm[k] = valid ? e.c[k] : 0.0;
        as[k] = valid ? fabs(e.c[k]) : 0.0;
    }
    if (uniform) {
        for (int o = 16; o > 0; o >>= 1)
            for (int k = 0; k < 3; ++k) {
                lo[k] = min(lo[k], __shfl_xor_sync(full, lo[k], o));
                hi[k] = max(hi[k], __shfl_xor_sync(full, hi[k], o));
                sm[k] += __shfl_xor_sync(full, sm[k], o);
                as[k] += __shfl_xor_sync(full, as[k], o);
            }
        if ((threadIdx.x & 31) != 0)
            return;
    } else if (!valid) {
        return;
    }
    SNode &n = nodes[node];
    for (int k = 0; k < 3; ++k) {
        atomicMin(&n.lo[k], lo[k]);
        atomicMax(&n.hi[k], hi[k]);
        atomicAdd(&n.sum[k], sm[k]);
        atomicAdd(&n.asum[k], as[k]);
    }
}

__global__ void __launch_bounds__(kSubThreads)
    k_rr_subtree(const int *__restrict__ deferred, const RNode *__restrict__ gnodes, RElem *recA, RElem *recB,
                 int *rank, int *errors)
{
    // ~102 KB of dynamic shared memory (opted in by the host)
    extern __shared__ __align__(16) unsigned char smem[];
    SNode *nodes = reinterpret_cast<SNode *>(smem);
    int(*nodeOf)[kSub] = reinterpret_cast<int(*)[kSub]>(smem + sizeof(SNode) * kSubNodes);
    int(*perm)[kSub] = reinterpret_cast<int(*)[kSub]>(smem + sizeof(SNode) * kSubNodes + sizeof(int) * 2 * kSub);
    int *flag = reinterpret_cast<int *>(smem + sizeof(SNode) * kSubNodes + sizeof(int) * 4 * kSub);
    int *scan = flag + kSub;
    int *warpSum = scan + kSub + 1;
    __shared__ int nNodes, lFirst, lLast, anyAmb, err;
    const int tid = threadIdx.x;
    const RNode &g = gnodes[deferred[blockIdx.x]];
    const int base = g.begin, n = g.count;
    const RElem *rc = recA + base; // the segment's records stay in place; only indices move
    (void)recB;
    if (tid == 0) {
        SNode &r = nodes[0];
        r.begin = 0;
        r.count = n;
        r.axis = 0;
        r.leftFinal = 0;
        r.child = -1;
        r.ambiguous = 0;
        for (int k = 0; k < 3; ++k) {
            r.lo[k] = g.lo[k];
            r.hi[k] = g.hi[k];
            r.sum[k] = g.sum[k];
            r.asum[k] = g.asum[k];
        }
        nNodes = 1;
        lFirst = 0;
        lLast = 1;
        err = 0;
    }
    for (int p = tid; p < n; p += kSubThreads) {
        nodeOf[0][p] = 0;
        perm[0][p] = p;
    }
    __syncthreads();
    int cur = 0;
    for (int level = 0; level < 4 * kSub; ++level) {
        const int first = lFirst, last = lLast;
        if (first >= last || err)
            break;
        // prep
        for (int id = first + tid; id < last; id += kSubThreads) {
            SNode &nd = nodes[id];
            if (nd.count <= 20) {
                nd.child = -1;
                continue;
            }
            float span[3];
            for (int k = 0; k < 3; ++k)
                span[k] = __double2float_rn(ord_to_dbl(nd.hi[k]) - ord_to_dbl(nd.lo[k]));
            int axis = 0;
            for (int k = 1; k < 3; ++k)
                if (span[axis] < span[k])
                    axis = k;
            nd.axis = axis;
            double gm = rr_gamma(nd.count + 1);
            double aup = __dmul_ru(nd.asum[axis], __dadd_ru(1.0, __dmul_ru(2.0, gm)));
            double e = __dadd_ru(__dmul_ru(__dmul_ru(2.0, gm), aup), 1e-300);
            double cnt = (double)(float)nd.count;
            nd.clo = __ddiv_rd(__dsub_rd(nd.sum[axis], e), cnt);
            nd.chi = __ddiv_ru(__dadd_ru(nd.sum[axis], e), cnt);
            nd.ambiguous = 0;
        }
        if (tid == 0)
            anyAmb = 0;
        __syncthreads();
        // classify
        for (int p = tid; p < n; p += kSubThreads) {
            int id = nodeOf[cur][p];
            int f = 0;
            if (id >= first) {
                SNode &nd = nodes[id];
                if (nd.count > 20) {
                    double c = rc[perm[cur][p]].c[nd.axis];
                    if (c < nd.clo)
                        f = 1;
                    else if (!(c >= nd.chi)) {
                        nd.ambiguous = 1;
                        anyAmb = 1;
                    }
                }
            }
            flag[p] = f;
        }
        __syncthreads();
        if (anyAmb) {
            for (int id = first + tid; id < last; id += kSubThreads) {
                SNode &nd = nodes[id];
                if (nd.count <= 20 || !nd.ambiguous)
                    continue;
                double sacc = 0.0;
                for (int p = nd.begin; p < nd.begin + nd.count; ++p)
                    sacc = sacc + rc[perm[cur][p]].c[nd.axis];
                double split = sacc / (double)(float)nd.count;
                for (int p = nd.begin; p < nd.begin + nd.count; ++p)
                    flag[p] = rc[perm[cur][p]].c[nd.axis] < split ? 1 : 0;
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
            if (nd.count <= 20)
                continue;
            int left = scan[nd.begin + nd.count] - scan[nd.begin];
            int right = nd.count - left;
            int lf = left;
            if (left == 0)
                lf = right / 2;
            else if (right == 0)
                lf = left - left / 2;
            int c = atomicAdd(&nNodes, 2);
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
            int id = nodeOf[cur][p];
            if (id < first || nodes[id].count <= 20) {
                perm[cur ^ 1][p] = perm[cur][p];
                nodeOf[cur ^ 1][p] = -1;
                continue;
            }
            const SNode &nd = nodes[id];
            int left = scan[nd.begin + nd.count] - scan[nd.begin];
            int lrank = scan[p] - scan[nd.begin];
            int rrank = (p - nd.begin) - lrank;
            int pos;
            if (left == 0)
                pos = rrank;
            else if (left == nd.count)
                pos = nd.count - 1 - lrank;
            else
                pos = flag[p] ? (left - 1 - lrank) : (left + rrank);
            int q = nd.begin + pos;
            perm[cur ^ 1][q] = perm[cur][p];
            nodeOf[cur ^ 1][q] = pos < nd.leftFinal ? nd.child : nd.child + 1;
        }
        __syncthreads();
        // statistics of the new nodes, read back in the new order
        for (int p0 = 0; p0 < n; p0 += kSubThreads) {
            int p = p0 + tid;
            bool valid = p < n && nodeOf[cur ^ 1][p] >= 0;
            RElem e;
            if (valid)
                e = rc[perm[cur ^ 1][p]];
            snode_accumulate(nodes, valid ? nodeOf[cur ^ 1][p] : 0, e, valid);
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
        atomicAdd(errors, 1);
    for (int p = tid; p < n; p += kSubThreads)
        rank[rc[perm[cur][p]].tri] = base + p;
}

// next level: [last, nodes allocated so far)
__global__ void k_rr_advance(int *bounds, const int *counters)
{
    bounds[0] = bounds[1];
    bounds[1] = counters[0];
}

__global__ void k_rr_rank(int nt, const RElem *__restrict__ rec, int *rank)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < nt)
        rank[rec[p].tri] = p;
}

__global__ void k_rr_init_root(RNode *nodes, int nt, int *counters)
{
    rnode_init(nodes[0], 0, nt);
    counters[0] = 1; // nodes allocated
    counters[1] = 0; // leaves
    counters[3] = 0; // capacity overflow
    counters[4] = 0; // level bounds: first
    counters[5] = 1; //               one past last
    counters[6] = 0; // deferred subtrees
    counters[7] = 0; // subtree errors
}

sb_status build_reference_rank(sb_mesh *m, cudaStream_t s)
{
    MeshDev &d = m->d;
    const int nt = d.nt;
    d.rankValid = false;
    if (nt <= 0)
        return SB_OK;
    KTime kt("reference_leaf_order", s);
    const int maxNodes = 2 * (nt / 4 + 8) + 64;
    size_t scanBytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, (int *)nullptr, (int *)nullptr, nt + 1, s);
    Carve c;
    size_t o_r1 = c.take<RElem>(nt), o_r2 = c.take<RElem>(nt), o_n1 = c.take<int>(nt), o_n2 = c.take<int>(nt);
    size_t o_fl = c.take<int>(nt + 1), o_sc = c.take<int>(nt + 1);
    size_t o_nd = c.take<RNode>(maxNodes), o_ct = c.take<int>(8), o_cub = c.take<char>(scanBytes);
    size_t o_df = c.take<int>(maxNodes);
    SB_CUDA_CHECK(m->tmp.ensure(c.off));
    char *b = m->tmp.as<char>();
    RElem *rec = (RElem *)(b + o_r1), *rec2 = (RElem *)(b + o_r2);
    int *nodeOf = (int *)(b + o_n1), *nodeOf2 = (int *)(b + o_n2);
    int *flag = (int *)(b + o_fl), *scan = (int *)(b + o_sc);
    RNode *nodes = (RNode *)(b + o_nd);
    int *counters = (int *)(b + o_ct); // [0] nodes, [1] leaves, [3] overflow, [4..5] level bounds
    int *bounds = counters + 4;
    int *deferred = (int *)(b + o_df);
    const int BS = 256, G = (nt + BS - 1) / BS, GN = 152 * 4;
    SB_COUNT(k_rr_centres)<<<G, BS, 0, s>>>(nt, d.v, d.t, d.box64, rec, nodeOf);
    SB_COUNT(k_rr_init_root)<<<1, 1, 0, s>>>(nodes, nt, counters);
    SB_COUNT(k_rr_root)<<<G, BS, 0, s>>>(nt, rec, nodes);
    SB_CUDA_CHECK(cudaMemsetAsync(flag + nt, 0, sizeof(int), s));
    // levels run in batches; the host looks at the level bounds only between batches
    // the first batch covers the expected depth of the large-node phase (a mean split roughly halves),
    // later batches are short; empty levels cost only their launches
    int expected = 1;
    while ((nt >> expected) > kSub)
        ++expected;
    bool done = false;
    for (int level = 0, batch = expected + 1; level < 4096 && !done; level += batch, batch = 2) {
        for (int j = 0; j < batch; ++j) {
            SB_COUNT(k_rr_prep)<<<GN, 128, 0, s>>>(bounds, nodes, counters, deferred);
            SB_COUNT(k_rr_classify)<<<G, BS, 0, s>>>(nt, bounds, rec, nodeOf, nodes, flag);
            SB_COUNT(k_rr_resolve)<<<GN, 128, 0, s>>>(bounds, rec, nodes, flag);
            SB_CUDA_CHECK(cub::DeviceScan::ExclusiveSum(b + o_cub, scanBytes, flag, scan, nt + 1, s));
            SB_COUNT(k_rr_children)<<<GN, 128, 0, s>>>(bounds, scan, nodes, counters, maxNodes);
            SB_COUNT(k_rr_scatter)<<<G, BS, 0, s>>>(nt, bounds, rec, nodeOf, flag, scan, nodes, rec2, nodeOf2);
            SB_COUNT(k_rr_child_stats)<<<G, BS, 0, s>>>(nt, bounds, rec2, nodeOf2, nodes);
            SB_COUNT(k_rr_advance)<<<1, 1, 0, s>>>(bounds, counters);
            std::swap(rec, rec2);
            std::swap(nodeOf, nodeOf2);
        }
        int cnt[8];
        SB_CUDA_CHECK(cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, s));
        SB_CUDA_CHECK(cudaStreamSynchronize(s));
        if (cnt[3] != 0) {
            set_last_error("reference tree node capacity exceeded");
            return SB_ERR_CAPACITY;
        }
        done = cnt[4] >= cnt[5];
    }
    if (!done) {
        set_last_error("reference tree deeper than 4096 levels");
        return SB_ERR_CAPACITY;
    }
    SB_COUNT(k_rr_rank)<<<G, BS, 0, s>>>(nt, rec, d.rank);
    int cnt2[8];
    SB_CUDA_CHECK(cudaMemcpyAsync(cnt2, counters, sizeof cnt2, cudaMemcpyDeviceToHost, s));
    SB_CUDA_CHECK(cudaStreamSynchronize(s));
    if (cnt2[6] > 0) {
        const size_t smemBytes = sizeof(SNode) * kSubNodes + sizeof(int) * (4 * kSub + kSub + kSub + 1 + kSubThreads / 32);
        SB_CUDA_CHECK(cudaFuncSetAttribute(k_rr_subtree, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemBytes));
        SB_COUNT(k_rr_subtree)<<<cnt2[6], kSubThreads, smemBytes, s>>>(deferred, nodes, rec, rec2, d.rank,
                                                                       counters + 7);
        int errs = 0;
        SB_CUDA_CHECK(cudaMemcpyAsync(&errs, counters + 7, sizeof errs, cudaMemcpyDeviceToHost, s));
        SB_CUDA_CHECK(cudaStreamSynchronize(s));
        if (errs) {
            set_last_error("reference tree: a subtree exceeded its node records");
            return SB_ERR_CAPACITY;
        }
    }
    SB_CUDA_CHECK(cudaGetLastError());
    d.rankValid = true;
    return SB_OK;
}

} // namespace sbg
