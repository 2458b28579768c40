// Candidate search and triangle-triangle intersection.
//
// Broad phase: the reference's dual-tree descent (src/axisalignedboundingboxtree.h:54-95, called from
// src/solidboolean.cpp:94-101) emits exactly the pairs whose triangle AABBs overlap under closed intervals;
// here one thread per first-mesh triangle (taken in Morton order, so neighbouring threads query
// neighbouring boxes) walks the second mesh's LBVH with a private stack and writes hits through
// warp-aggregated atomics. The set is the same; its order is not used (every later ordering is by unique
// keys), so runs are deterministic without sorting it.
//
// Narrow phase: Guigue-Devillers (thirdparty/GuigueDevillers03/tri_tri_intersect.c:285-472) one thread per
// candidate. Every orientation sign the reference tests is first evaluated in FP32 from rounded copies of
// the vertices together with a static forward-error bound that covers the FP32 rounding of the inputs,
// the FP32 arithmetic and the FP64 arithmetic of the reference; a sign is used only when |v32| exceeds
// that bound, otherwise the value is recomputed in FP64 with the reference's exact operation order. The
// segment end points are always constructed in FP64 with the reference's formulas.
#include <cooperative_groups.h>
#include <cub/cub.cuh>

#include "sb_common.cuh"
#include "sb_internal.h"
#include "sb_ktime.h"
#include "sb_pairs.cuh"

namespace cg = cooperative_groups;

namespace sbg {

__device__ __forceinline__ void emit_u64(uint64_t v, uint64_t *out, unsigned int *count, unsigned int cap)
{
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned int base = 0;
    if (g.thread_rank() == 0)
        base = atomicAdd(count, g.size());
    base = g.shfl(base, 0);
    unsigned int pos = base + g.thread_rank();
    if (pos < cap)
        out[pos] = v;
}

// closed-interval overlap of triangle boxes (src/axisalignedboundingbox.h:95-105)
template <bool FP64>
__device__ __forceinline__ bool leaf_overlap(const float *qa32, const double *qa64, const MeshDev &B, int tb,
                                             unsigned int &fallbacks)
{
    if (FP64) {
        const double *b = B.box64 + 6 * (size_t)tb;
        for (int k = 0; k < 3; ++k)
            if (!(qa64[k] <= b[3 + k] && qa64[3 + k] >= b[k]))
                return false;
        return true;
    }
    // round-to-nearest is monotonic: FP32 order decides unless the two rounded values are equal
    const float *b = B.box32 + 6 * (size_t)tb;
    bool tie = false;
    for (int k = 0; k < 3; ++k) {
        float alo = qa32[k], ahi = qa32[3 + k], blo = b[k], bhi = b[3 + k];
        if (alo > bhi || ahi < blo)
            return false;
        if (alo == bhi || ahi == blo)
            tie = true;
    }
    if (!tie)
        return true;
    ++fallbacks;
    const double *b64 = B.box64 + 6 * (size_t)tb;
    for (int k = 0; k < 3; ++k)
        if (!(qa64[k] <= b64[3 + k] && qa64[3 + k] >= b64[k]))
            return false;
    return true;
}

template <bool FP64>
__global__ void __launch_bounds__(128) k_broad(MeshDev A, MeshDev B, uint64_t *out, unsigned int *count,
                                               unsigned int cap, unsigned long long *stats)
{
    int li = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int tests = 0, fallbacks = 0;
    if (li < A.nt && B.nt > 0) {
        int a = A.leafTri[li];
        double q64[6];
        float q32[6], qo[6];
        for (int k = 0; k < 6; ++k) {
            q64[k] = A.box64[6 * (size_t)a + k];
            q32[k] = A.box32[6 * (size_t)a + k];
        }
        for (int k = 0; k < 3; ++k) {
            qo[k] = __double2float_rd(q64[k]);
            qo[3 + k] = __double2float_ru(q64[3 + k]);
        }
        const uint64_t nb = (uint64_t)B.nt;
        if (B.root < 0) {
            int tb = B.leafTri[0];
            ++tests;
            if (leaf_overlap<FP64>(q32, q64, B, tb, fallbacks))
                emit_u64((uint64_t)a * nb + (uint64_t)tb, out, count, cap);
        } else {
            int stack[96];
            int sp = 0;
            stack[sp++] = B.root;
            while (sp > 0) {
                int node = stack[--sp];
                int2 ch = B.child[node];
                int cs[2] = {ch.x, ch.y};
                for (int k = 0; k < 2; ++k) {
                    int c = cs[k];
                    if (c < 0) {
                        int tb = B.leafTri[~c];
                        ++tests;
                        if (leaf_overlap<FP64>(q32, q64, B, tb, fallbacks))
                            emit_u64((uint64_t)a * nb + (uint64_t)tb, out, count, cap);
                    } else {
                        bool hit;
                        if (FP64) {
                            const double *bx = B.nbox64 + 6 * (size_t)c;
                            hit = q64[0] <= bx[3] && q64[3] >= bx[0] && q64[1] <= bx[4] && q64[4] >= bx[1] &&
                                  q64[2] <= bx[5] && q64[5] >= bx[2];
                        } else {
                            const float4 *bx = reinterpret_cast<const float4 *>(B.nbox32) + 2 * (size_t)c;
                            const float4 lo = __ldg(bx), hi = __ldg(bx + 1);
                            hit = qo[0] <= hi.x && qo[3] >= lo.x && qo[1] <= hi.y && qo[4] >= lo.y &&
                                  qo[2] <= hi.z && qo[5] >= lo.z;
                        }
                        if (hit) {
                            if (sp < 96)
                                stack[sp++] = c;
                            else
                                atomicAdd(stats + 4, 1ull); // reported as a capacity error, never dropped
                        }
                    }
                }
            }
        }
    }
    // warp totals into the stats counters
    for (int s = 16; s > 0; s >>= 1) {
        tests += __shfl_xor_sync(0xFFFFFFFFu, tests, s);
        fallbacks += __shfl_xor_sync(0xFFFFFFFFu, fallbacks, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(stats + 0, (unsigned long long)tests);
        atomicAdd(stats + 1, (unsigned long long)fallbacks);
    }
}

template <bool FP64>
__global__ void __launch_bounds__(128) k_narrow(MeshDev A, MeshDev B, const uint64_t *__restrict__ cand, int n,
                                                uint8_t *__restrict__ hit, double *__restrict__ seg,
                                                uint32_t *__restrict__ perm, unsigned long long *stats)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int tests = 0, fallbacks = 0;
    if (i < n) {
        uint64_t key = cand[i];
        int a = (int)(key / (uint64_t)B.nt);
        int b = (int)(key - (uint64_t)a * (uint64_t)B.nt);
        TriTri<FP64> tt;
        tt.load(A, B, a, b);
        double s[6];
        int r = tt.run(s);
        hit[i] = r == 1 ? 1 : 0;
        if (r == 1) {
            for (int k = 0; k < 6; ++k)
                seg[6 * (size_t)i + k] = s[k];
            perm[i] = tt.permCode;
        }
        tests = tt.tests;
        fallbacks = tt.fallbacks;
    }
    for (int s = 16; s > 0; s >>= 1) {
        tests += __shfl_xor_sync(0xFFFFFFFFu, tests, s);
        fallbacks += __shfl_xor_sync(0xFFFFFFFFu, fallbacks, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(stats + 2, (unsigned long long)tests);
        atomicAdd(stats + 3, (unsigned long long)fallbacks);
    }
}

// launch wrappers ----------------------------------------------------------------------------------------
void launch_broad(bool fp64, const MeshDev &A, const MeshDev &B, uint64_t *out, unsigned int *count,
                  unsigned int cap, unsigned long long *stats, cudaStream_t s)
{
    if (A.nt <= 0)
        return;
    int bs = 128, g = (A.nt + bs - 1) / bs;
    KTime kt("k_broad", s);
    count_launch();
    if (fp64)
        k_broad<true><<<g, bs, 0, s>>>(A, B, out, count, cap, stats);
    else
        k_broad<false><<<g, bs, 0, s>>>(A, B, out, count, cap, stats);
}

void launch_narrow(bool fp64, const MeshDev &A, const MeshDev &B, const uint64_t *cand, int n, uint8_t *hit,
                   double *seg, uint32_t *perm, unsigned long long *stats, cudaStream_t s)
{
    if (n <= 0)
        return;
    int bs = 128, g = (n + bs - 1) / bs;
    KTime kt("k_narrow", s);
    count_launch();
    if (fp64)
        k_narrow<true><<<g, bs, 0, s>>>(A, B, cand, n, hit, seg, perm, stats);
    else
        k_narrow<false><<<g, bs, 0, s>>>(A, B, cand, n, hit, seg, perm, stats);
}

} // namespace sbg
