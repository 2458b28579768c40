// Guigue-Devillers triangle-triangle intersection for one candidate pair, in two arithmetic forms:
//   TriTri<true>  : plain FP64, the reference's operations in the reference's order;
//   TriTri<false> : every orientation sign first from FP32 with a static forward-error bound, FP64 only
//                   where the bound does not certify the sign of the FP64 expression.
// The permutation logic works on vertex slots 0..5 = (p1, q1, r1, p2, q2, r2) so one decision tree serves
// both forms (tri_tri_intersect.c:360-385 and 443-471).
#pragma once
#include "sb_common.cuh"
#include "sb_internal.h"

namespace sbg {

// ---- FP32 value with a forward-error bound -----------------------------------------------------------
struct F3e {
    float x, y, z;    // computed FP32 value
    float ex, ey, ez; // |computed - exact| bound
    float mx, my, mz; // bound on both |computed| and |exact|
};

// u = 2^-24; c_diff >= u / (1 - u) rounded up
#define SB_U32 5.9604645e-08f
#define SB_CDIFF 5.9604652e-08f

// difference of two FP32-rounded inputs, with the bound relative to the exact FP64 difference
__device__ __forceinline__ F3e fdiff(float4 a, float4 b)
{
    F3e r;
    r.x = a.x - b.x;
    r.y = a.y - b.y;
    r.z = a.z - b.z;
    r.ex = SB_CDIFF * (fabsf(a.x) + fabsf(b.x) + fabsf(r.x));
    r.ey = SB_CDIFF * (fabsf(a.y) + fabsf(b.y) + fabsf(r.y));
    r.ez = SB_CDIFF * (fabsf(a.z) + fabsf(b.z) + fabsf(r.z));
    r.mx = fabsf(r.x) + r.ex;
    r.my = fabsf(r.y) + r.ey;
    r.mz = fabsf(r.z) + r.ez;
    return r;
}

// one cross component c = a1*b2 - a2*b1 with perturbation and rounding bounds
__device__ __forceinline__ void fcross1(float a1, float ea1, float ma1, float b2, float eb2, float mb2, float a2,
                                        float ea2, float ma2, float b1, float eb1, float mb1, float &c, float &e,
                                        float &m)
{
    c = __fsub_rn(__fmul_rn(a1, b2), __fmul_rn(a2, b1));
    float perm = ma1 * mb2 + ma2 * mb1;
    e = ma1 * eb2 + ea1 * mb2 + ma2 * eb1 + ea2 * mb1 + 3.0f * SB_U32 * perm;
    m = perm * (1.0f + 4.0f * SB_U32);
}

__device__ __forceinline__ F3e fcross(const F3e &a, const F3e &b)
{
    F3e r;
    fcross1(a.y, a.ey, a.my, b.z, b.ez, b.mz, a.z, a.ez, a.mz, b.y, b.ey, b.my, r.x, r.ex, r.mx);
    fcross1(a.z, a.ez, a.mz, b.x, b.ex, b.mx, a.x, a.ex, a.mx, b.z, b.ez, b.mz, r.y, r.ey, r.my);
    fcross1(a.x, a.ex, a.mx, b.y, b.ey, b.my, a.y, a.ey, a.my, b.x, b.ex, b.mx, r.z, r.ez, r.mz);
    return r;
}

// certified sign of the FP64 evaluation of dot(u, n): +1 / -1, or 0 when not certified
__device__ __forceinline__ int fdot_sign(const F3e &u, const F3e &n)
{
    float v = __fadd_rn(__fadd_rn(__fmul_rn(u.x, n.x), __fmul_rn(u.y, n.y)), __fmul_rn(u.z, n.z));
    float perm = u.mx * n.mx + u.my * n.my + u.mz * n.mz;
    float err = u.mx * n.ex + u.ex * n.mx + u.my * n.ey + u.ey * n.my + u.mz * n.ez + u.ez * n.mz +
                4.0f * SB_U32 * perm  // FP32 dot rounding
                + 1.2e-15f * perm;    // the reference's own FP64 rounding
    err = err * (1.0f + 16.0f * SB_U32) + 1e-36f;
    float av = fabsf(v);
    if (!(av > err) || !(av >= 1e-30f))
        return 0;
    return v > 0.0f ? 1 : -1;
}

// ---- FP64, reference operation order ----------------------------------------------------------------
__device__ __forceinline__ int sign64(double v) { return (v > 0.0) ? 1 : ((v < 0.0) ? -1 : 0); }

template <bool FP64> struct TriTri {
    d3 P[6];
    float4 F[6];
    bool have64 = false;
    unsigned int tests = 0, fallbacks = 0;
    // how the segment was built (kept for the adjoint): the six slots in construction order, 3 bits each,
    // and the case `which` in bits 18-19
    uint32_t permCode = 0;
    const MeshDev *pA = nullptr, *pB = nullptr;
    int ia[3], ib[3];

    __device__ __forceinline__ void load(const MeshDev &A, const MeshDev &B, int a, int b)
    {
        pA = &A;
        pB = &B;
        for (int k = 0; k < 3; ++k) {
            ia[k] = (int)A.t[3 * (size_t)a + k];
            ib[k] = (int)B.t[3 * (size_t)b + k];
        }
        if (FP64) {
            load64();
        } else {
            for (int k = 0; k < 3; ++k) {
                F[k] = A.vf[ia[k]];
                F[3 + k] = B.vf[ib[k]];
            }
        }
    }
    __device__ __forceinline__ void load64()
    {
        if (have64)
            return;
        for (int k = 0; k < 3; ++k) {
            const double *pa = pA->v + 3 * (size_t)ia[k];
            const double *pb = pB->v + 3 * (size_t)ib[k];
            P[k] = mk(pa[0], pa[1], pa[2]);
            P[3 + k] = mk(pb[0], pb[1], pb[2]);
        }
        have64 = true;
    }


    // register-resident selection of slot i (runtime index into the arrays would spill them to local memory)
    __device__ __forceinline__ float4 fs(int i) const
    {
        float4 r = F[0];
        r = i == 1 ? F[1] : r;
        r = i == 2 ? F[2] : r;
        r = i == 3 ? F[3] : r;
        r = i == 4 ? F[4] : r;
        r = i == 5 ? F[5] : r;
        return r;
    }
    __device__ __forceinline__ d3 ps(int i) const
    {
        d3 r = P[0];
        r = i == 1 ? P[1] : r;
        r = i == 2 ? P[2] : r;
        r = i == 3 ? P[3] : r;
        r = i == 4 ? P[4] : r;
        r = i == 5 ? P[5] : r;
        return r;
    }

    // Signs of dot(X - base, cross(V0 - V1, W0 - W1)) for X in x[0..2]; `reject` reproduces
    // ((d0 * d1) > 0) && ((d0 * d2) > 0) (tri_tri_intersect.c:421, 438).
    __device__ __forceinline__ void stage(int V0, int V1, int W0, int W1, int base, const int *x, int *s,
                                          bool &reject)
    {
        tests += 3;
        if (!FP64) {
            F3e n = fcross(fdiff(fs(V0), fs(V1)), fdiff(fs(W0), fs(W1)));
            int ok = 1;
            for (int k = 0; k < 3; ++k) {
                s[k] = fdot_sign(fdiff(fs(x[k]), fs(base)), n);
                ok &= (s[k] != 0);
            }
            if (ok) {
                reject = (s[0] * s[1] > 0) && (s[0] * s[2] > 0);
                return;
            }
            fallbacks += 3;
            load64();
        }
        d3 n = cross(ps(V0) - ps(V1), ps(W0) - ps(W1));
        double d[3];
        for (int k = 0; k < 3; ++k) {
            d[k] = dot(ps(x[k]) - ps(base), n);
            s[k] = sign64(d[k]);
        }
        reject = ((d[0] * d[1]) > 0.0) && ((d[0] * d[2]) > 0.0);
    }

    // sign of dot(U0 - U1, cross(V0 - V1, W0 - W1)), as the FP64 expression evaluates it
    __device__ __forceinline__ int orient(int U0, int U1, int V0, int V1, int W0, int W1)
    {
        ++tests;
        if (!FP64) {
            F3e n = fcross(fdiff(fs(V0), fs(V1)), fdiff(fs(W0), fs(W1)));
            int s = fdot_sign(fdiff(fs(U0), fs(U1)), n);
            if (s != 0)
                return s;
            ++fallbacks;
            load64();
        }
        d3 n = cross(ps(V0) - ps(V1), ps(W0) - ps(W1));
        return sign64(dot(ps(U0) - ps(U1), n));
    }

    // out = base - alpha * (base - other), alpha = dot(base - ref, n) / dot(base - other, n)
    __device__ __forceinline__ d3 along(int base, int ref, int other, d3 n)
    {
        d3 v1 = ps(base) - ps(ref);
        d3 v2 = ps(base) - ps(other);
        double alpha = dot(v1, n) / dot(v2, n);
        d3 sv = scale(alpha, v2);
        return ps(base) - sv;
    }

    // CONSTRUCT_INTERSECTION (tri_tri_intersect.c:285-356) on slots already in canonical order. The four
    // outcomes differ only in which vertices and which normal the two end points use, so they are chosen as
    // data and computed once (one copy of the code keeps the kernel small).
    __device__ int construct(const int *v, double *out)
    {
        const int p1 = v[0], q1 = v[1], r1 = v[2], p2 = v[3], q2 = v[4], r2 = v[5];
        int which; // 0: (p1 r1 N2, p2 r2 N1)  1: (p2 q2 N1, p2 r2 N1)  2: (p1 r1 N2, p1 q1 N2)  3: (p2 q2 N1, p1 q1 N2)
        if (orient(p2, p1, q1, p1, r2, p1) > 0) {
            if (orient(p2, p1, r1, p1, r2, p1) > 0)
                return 0;
            which = orient(p2, p1, r1, p1, q2, p1) > 0 ? 0 : 1;
        } else {
            if (orient(p2, p1, q1, p1, q2, p1) < 0)
                return 0;
            which = orient(p2, p1, r1, p1, q2, p1) >= 0 ? 2 : 3;
        }
        load64();
        permCode = (uint32_t)v[0] | (uint32_t)v[1] << 3 | (uint32_t)v[2] << 6 | (uint32_t)v[3] << 9 |
                   (uint32_t)v[4] << 12 | (uint32_t)v[5] << 15 | (uint32_t)which << 18;
        const d3 N1 = cross(ps(1) - ps(0), ps(2) - ps(0));
        const d3 N2 = cross(ps(3) - ps(5), ps(4) - ps(5));
        // first end point: which 0, 2 -> along(p1, p2, r1, N2); 1, 3 -> along(p2, p1, q2, N1)
        const bool sOn1 = which == 0 || which == 2;
        const d3 s = along(sOn1 ? p1 : p2, sOn1 ? p2 : p1, sOn1 ? r1 : q2, sOn1 ? N2 : N1);
        // second end point: which 0, 1 -> along(p2, p1, r2, N1); 2, 3 -> along(p1, p2, q1, N2)
        const bool tOn2 = which <= 1;
        const d3 t = along(tOn2 ? p2 : p1, tOn2 ? p1 : p2, tOn2 ? r2 : q1, tOn2 ? N1 : N2);
        out[0] = s.x;
        out[1] = s.y;
        out[2] = s.z;
        out[3] = t.x;
        out[4] = t.y;
        out[5] = t.z;
        return 1;
    }

    // TRI_TRI_INTER_3D (tri_tri_intersect.c:360-385): the slot order handed to CONSTRUCT_INTERSECTION, or
    // false for the coplanar case
    __device__ __forceinline__ static bool second(int p1, int q1, int r1, int p2, int q2, int r2, int dp2, int dq2,
                                                  int dr2, int *v)
    {
        // tri 1 either as given (p1 q1 r1) or swapped (p1 r1 q1); tri 2 in one of three rotations
        int t1 = 0, rot = 0; // t1: 0 keep, 1 swap q1/r1; rot: 0 (p2 q2 r2), 1 (r2 p2 q2), 2 (q2 r2 p2)
        if (dp2 > 0) {
            if (dq2 > 0) {
                t1 = 1;
                rot = 1;
            } else if (dr2 > 0) {
                t1 = 1;
                rot = 2;
            } else {
                t1 = 0;
                rot = 0;
            }
        } else if (dp2 < 0) {
            if (dq2 < 0) {
                t1 = 0;
                rot = 1;
            } else if (dr2 < 0) {
                t1 = 0;
                rot = 2;
            } else {
                t1 = 1;
                rot = 0;
            }
        } else if (dq2 < 0) {
            if (dr2 >= 0) {
                t1 = 1;
                rot = 2;
            } else {
                t1 = 0;
                rot = 0;
            }
        } else if (dq2 > 0) {
            if (dr2 > 0) {
                t1 = 1;
                rot = 0;
            } else {
                t1 = 0;
                rot = 2;
            }
        } else if (dr2 > 0) {
            t1 = 0;
            rot = 1;
        } else if (dr2 < 0) {
            t1 = 1;
            rot = 1;
        } else {
            return false;
        }
        v[0] = p1;
        v[1] = t1 ? r1 : q1;
        v[2] = t1 ? q1 : r1;
        v[3] = rot == 0 ? p2 : (rot == 1 ? r2 : q2);
        v[4] = rot == 0 ? q2 : (rot == 1 ? p2 : r2);
        v[5] = rot == 0 ? r2 : (rot == 1 ? q2 : p2);
        return true;
    }

    // tri_tri_intersection_test_3d (tri_tri_intersect.c:395-472): 1 segment, 0 none, -1 coplanar
    __device__ int run(double *out)
    {
        const int p1 = 0, q1 = 1, r1 = 2, p2 = 3, q2 = 4, r2 = 5;
        int s1[3], s2[3];
        bool rej;
        const int x1[3] = {p1, q1, r1};
        stage(p2, r2, q2, r2, r2, x1, s1, rej);
        if (rej)
            return 0;
        const int x2[3] = {p2, q2, r2};
        stage(q1, p1, r1, p1, r1, x2, s2, rej);
        if (rej)
            return 0;
        const int dp1 = s1[0], dq1 = s1[1], dr1 = s1[2];
        const int dp2 = s2[0], dq2 = s2[1], dr2 = s2[2];
        // tri 1 rotated to (r1 p1 q1), (q1 r1 p1) or kept; tri 2 kept or swapped (p2 r2 q2) with its signs
        int rot1 = 0, sw2 = 0; // rot1: 0 (p1 q1 r1), 1 (r1 p1 q1), 2 (q1 r1 p1); sw2: 1 swaps q2/r2
        if (dp1 > 0) {
            if (dq1 > 0) {
                rot1 = 1;
                sw2 = 1;
            } else if (dr1 > 0) {
                rot1 = 2;
                sw2 = 1;
            } else {
                rot1 = 0;
                sw2 = 0;
            }
        } else if (dp1 < 0) {
            if (dq1 < 0) {
                rot1 = 1;
                sw2 = 0;
            } else if (dr1 < 0) {
                rot1 = 2;
                sw2 = 0;
            } else {
                rot1 = 0;
                sw2 = 1;
            }
        } else if (dq1 < 0) {
            if (dr1 >= 0) {
                rot1 = 2;
                sw2 = 1;
            } else {
                rot1 = 0;
                sw2 = 0;
            }
        } else if (dq1 > 0) {
            if (dr1 > 0) {
                rot1 = 0;
                sw2 = 1;
            } else {
                rot1 = 2;
                sw2 = 0;
            }
        } else if (dr1 > 0) {
            rot1 = 1;
            sw2 = 0;
        } else if (dr1 < 0) {
            rot1 = 1;
            sw2 = 1;
        } else {
            return -1;
        }
        const int a = rot1 == 0 ? p1 : (rot1 == 1 ? r1 : q1);
        const int b = rot1 == 0 ? q1 : (rot1 == 1 ? p1 : r1);
        const int c = rot1 == 0 ? r1 : (rot1 == 1 ? q1 : p1);
        int v[6];
        if (!second(a, b, c, p2, sw2 ? r2 : q2, sw2 ? q2 : r2, dp2, sw2 ? dr2 : dq2, sw2 ? dq2 : dr2, v))
            return -1;
        return construct(v, out);
    }
};

void launch_broad(bool fp64, const MeshDev &A, const MeshDev &B, uint64_t *out, unsigned int *count,
                  unsigned int cap, unsigned long long *stats, cudaStream_t s);
void launch_narrow(bool fp64, const MeshDev &A, const MeshDev &B, const uint64_t *cand, int n, uint8_t *hit,
                   double *seg, uint32_t *perm, unsigned long long *stats, cudaStream_t s);

} // namespace sbg
