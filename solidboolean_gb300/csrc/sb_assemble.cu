// Assembly of the combined arrangement and the inside/outside labelling.
//
//   global weld       addNewPoint (src/solidboolean.cpp:241-248): cut points of all faces, first mesh's faces
//                     first, keyed by PositionKey in a device hash table; the first occurrence in that order
//                     keeps its coordinates and the new vertices are numbered in first-occurrence order
//   arrangement       addUnintersectedTriangles (:250-286) and the reTriangulate lambda (:352-407): uncut
//                     triangles of each mesh (index order) and the re-triangulated faces, with their
//                     half-edges in per-mesh device hash tables (first owner wins)
//   cut loops         buildPolygonsFromEdges (:124-165): every loop vertex must have exactly two neighbours
//   face groups       buildFaceGroups (:167-239): the flood fill crosses every half-edge that is not a cut
//                     edge and has a twin; its connected components are found with a lock-free union-find
//   sides             decideGroupSide / isPointInMesh (:482-510, 48-92): three axis rays from the centroid
//                     of each region's representative triangle, hit points deduplicated by PositionKey,
//                     inside when at least two of the three parities are odd
#include <algorithm>

#include <cub/cub.cuh>

#include "sb_assemble.cuh"
#include "sb_common.cuh"
#include "sb_ktime.h"

namespace sbg {

// ---- global weld ----------------------------------------------------------------------------------
// A cut point's place in the reference's sequence is ptRef[f] + k: faces in their processing order (the
// first mesh's, then the second's), points in each face's local order. Slots are claimed by the first
// storage position to arrive (for the key comparison) and keep the smallest sequence position of the key.
__global__ void k_weld_insert(int nFaces, const int *__restrict__ ptOff, const int *__restrict__ ptRef,
                              const int *__restrict__ faceNpts, const Key *__restrict__ keys, int *slotOwner,
                              int *slotMin, uint32_t mask, int *pointSlot)
{
    int f = blockIdx.x;
    if (f >= nFaces)
        return;
    int n = faceNpts[f];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        int seq = ptOff[f] + k;
        Key key = keys[seq];
        uint32_t s = (uint32_t)(key_hash(key) & mask);
        for (uint32_t probe = 0; probe <= mask; ++probe) {
            int o = atomicCAS(slotOwner + s, -1, seq);
            if (o == -1 || key_eq(keys[o], key)) {
                atomicMin(slotMin + s, ptRef[f] + k);
                pointSlot[seq] = (int)s;
                break;
            }
            s = (s + 1) & mask;
        }
    }
}

// first occurrences flagged at their sequence positions (capacity slots past a face's points stay 0)
__global__ void k_weld_first(int nFaces, const int *__restrict__ ptOff, const int *__restrict__ ptRef,
                             const int *__restrict__ faceNpts, const int *__restrict__ pointSlot,
                             const int *__restrict__ slotMin, int *isFirst)
{
    int f = blockIdx.x;
    if (f >= nFaces)
        return;
    int n = faceNpts[f];
    for (int k = threadIdx.x; k < ptOff[f + 1] - ptOff[f]; k += blockDim.x) {
        const int rs = ptRef[f] + k;
        isFirst[rs] = (k < n && slotMin[pointSlot[ptOff[f] + k]] == rs) ? 1 : 0;
    }
}

// appended vertex r = rank of its first occurrence in the sequence (addNewPoint numbering), with the
// coordinates of that occurrence
__global__ void k_weld_number(int nFaces, const int *__restrict__ ptOff, const int *__restrict__ ptRef,
                              const int *__restrict__ faceNpts, const int *__restrict__ isFirst,
                              const int *__restrict__ firstRank, const int *__restrict__ pointSlot, int *slotRank,
                              const d3 *__restrict__ pts, double *newV, int vbase, const int *__restrict__ ptSrc,
                              int *newSrc)
{
    int f = blockIdx.x;
    if (f >= nFaces)
        return;
    int n = faceNpts[f];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int rs = ptRef[f] + k, seq = ptOff[f] + k;
        if (!isFirst[rs])
            continue;
        const int r = firstRank[rs];
        slotRank[pointSlot[seq]] = r;
        newSrc[r] = ptSrc[seq];
        const d3 p = pts[seq];
        double *o = newV + 3 * (size_t)(vbase + r);
        o[0] = p.x;
        o[1] = p.y;
        o[2] = p.z;
    }
}

// ---- arrangement ------------------------------------------------------------------------------------
__global__ void k_mark_cut(int nFaces, const int *__restrict__ faceSide, const int *__restrict__ faceTri,
                           int *cutA, int *cutB)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces)
        return;
    if (faceSide[f] == 0)
        cutA[faceTri[f]] = 1;
    else
        cutB[faceTri[f]] = 1;
}

// uncut triangles of one mesh, in index order, offset into the arrangement
__global__ void k_uncut(int nt, const uint32_t *__restrict__ t, const int *__restrict__ cut,
                        const int *__restrict__ uncutRank, uint32_t vbase, uint32_t outBase, uint32_t *newT,
                        int *origUncut, const int *__restrict__ truncOcc)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt || cut[i] || i > *truncOcc / 3)
        return;
    uint32_t o = outBase + (uint32_t)uncutRank[i];
    origUncut[o] = i;
    newT[3 * (size_t)o] = t[3 * (size_t)i] + vbase;
    newT[3 * (size_t)o + 1] = t[3 * (size_t)i + 1] + vbase;
    newT[3 * (size_t)o + 2] = t[3 * (size_t)i + 2] + vbase;
}

__device__ __forceinline__ uint32_t local_to_global(int local, const uint32_t *tri, uint32_t vbase, int ptBase,
                                                   const int *pointSlot, const int *slotRank, uint32_t newBase)
{
    if (local < 3)
        return tri[local] + vbase;
    return newBase + (uint32_t)slotRank[pointSlot[ptBase + local - 3]];
}

__global__ void k_retri(int nFaces, const int *__restrict__ faceSide, const int *__restrict__ faceTri,
                        const int *__restrict__ faceNtris, const int *__restrict__ triOff,
                        const int *__restrict__ retriRank, const int *__restrict__ faceTris,
                        const int *__restrict__ ptOff, const int *__restrict__ pointSlot,
                        const int *__restrict__ slotRank, MeshDev A, MeshDev B, uint32_t newBase, uint32_t outBase,
                        uint32_t *newT, int *retriFace)
{
    int f = blockIdx.x;
    if (f >= nFaces)
        return;
    const MeshDev &M = faceSide[f] == 0 ? A : B;
    uint32_t vbase = faceSide[f] == 0 ? 0u : (uint32_t)A.nv;
    const uint32_t *tri = M.t + 3 * (size_t)faceTri[f];
    int n = faceNtris[f];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int *lt = faceTris + 3 * (size_t)(triOff[f] + k);
        uint32_t o = outBase + (uint32_t)(retriRank[f] + k);
        retriFace[retriRank[f] + k] = f;
        for (int c = 0; c < 3; ++c)
            newT[3 * (size_t)o + c] = local_to_global(lt[c], tri, vbase, ptOff[f], pointSlot, slotRank, newBase);
    }
}

// ---- cut loops (first mesh's cut edges) ----------------------------------------------------------------
// Directed entry e of first-mesh face f, (u -> v), is the reference's `edges[u].insert(v); edges[v].insert(u)`
// at sequence slots 2 (edgeRef[f] + e) and that + 1 (src/solidboolean.cpp:397-404): u becomes a key of the
// loop map at the first slot, v at the second, v joins u's set at the first, u joins v's set at the second.
// Per undirected edge (lo, hi) of the table: slotLo = when hi joined lo's set, slotHi = when lo joined hi's.
__global__ void k_cut_edges(int nFaces, const int *__restrict__ faceSide, const int *__restrict__ faceNedges,
                            const int *__restrict__ edgeOff, const int *__restrict__ edgeRef,
                            const int *__restrict__ faceEdges, const int *__restrict__ ptOff,
                            const int *__restrict__ pointSlot, const int *__restrict__ slotRank, uint64_t *edgeKeys,
                            int *edgeVals, uint32_t mask, int *slotLo, int *slotHi, int *firstOcc, int sideWanted)
{
    int f = blockIdx.x;
    if (f >= nFaces || faceSide[f] != sideWanted)
        return;
    for (int k = threadIdx.x; k < faceNedges[f]; k += blockDim.x) {
        const int *e = faceEdges + 2 * (size_t)(edgeOff[f] + k);
        uint32_t u = (uint32_t)slotRank[pointSlot[ptOff[f] + e[0] - 3]];
        uint32_t v = (uint32_t)slotRank[pointSlot[ptOff[f] + e[1] - 3]];
        if (u == v)
            continue;
        const int slot = 2 * (edgeRef[f] + k);
        uint32_t lo = min(u, v), hi = max(u, v);
        const int s = u64map_insert_min_slot(edgeKeys, edgeVals, mask, ((uint64_t)lo << 32) | hi, 0);
        if (s >= 0) {
            atomicMin(slotLo + s, u == lo ? slot : slot + 1);
            atomicMin(slotHi + s, u == lo ? slot + 1 : slot);
        }
        atomicMin(firstOcc + u, slot);
        atomicMin(firstOcc + v, slot + 1);
    }
}

// neighbour count of every loop vertex, and its first two neighbours with the slot at which each joined
// its set
__global__ void k_loop_degree(uint32_t cap, const uint64_t *__restrict__ edgeKeys, const int *__restrict__ slotLo,
                              const int *__restrict__ slotHi, int *degree, int *nbr, int *nbrSlot)
{
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cap)
        return;
    uint64_t k = edgeKeys[s];
    if (k == kEmpty64)
        return;
    const int lo = (int)(k >> 32), hi = (int)(k & 0xFFFFFFFFu);
    const int a = atomicAdd(degree + lo, 1);
    if (a < 2) {
        nbr[2 * lo + a] = hi;
        nbrSlot[2 * lo + a] = slotLo[s];
    }
    const int b = atomicAdd(degree + hi, 1);
    if (b < 2) {
        nbr[2 * hi + b] = lo;
        nbrSlot[2 * hi + b] = slotHi[s];
    }
}

__global__ void k_loop_check(int n, const int *__restrict__ degree, unsigned int *counters)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    int d = degree[i];
    if (d > 0)
        atomicAdd(counters + 0, 1u);
    if (d > 0 && d != 2)
        atomicAdd(counters + 1, 1u);
}

// ---- half-edge tables, union-find ---------------------------------------------------------------------

__global__ void k_halfedges(int nTri, const uint32_t *__restrict__ newT, const int8_t *__restrict__ triMesh,
                            uint64_t *keysA, int *valsA, uint64_t *keysB, int *valsB, uint32_t mask, int uncutAll,
                            const int *__restrict__ origUncut, const int *__restrict__ truncOcc)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nTri)
        return;
    const uint32_t *v = newT + 3 * (size_t)t;
    const int m = triMesh[t];
    uint64_t *keys = m == 0 ? keysA : keysB;
    int *vals = m == 0 ? valsA : valsB;
    // the last uncut triangle of a truncated mesh inserted its half-edges only up to the repeated one
    const int lastEdge = t < uncutAll ? truncOcc[m] - 3 * origUncut[t] : 2;
    for (int i = 0; i < 3 && i <= lastEdge; ++i)
        u64map_insert_min(keys, vals, mask, he_key(v[i], v[(i + 1) % 3]), t);
}

__device__ int uf_find(int *parent, int x)
{
    while (true) {
        int p = parent[x];
        if (p == x)
            return x;
        int gp = parent[p];
        if (gp != p)
            atomicCAS(parent + x, p, gp); // path halving
        x = gp;
    }
}

__device__ void uf_union(int *parent, int a, int b)
{
    while (true) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b)
            return;
        if (a < b) {
            int t = a;
            a = b;
            b = t;
        }
        if (atomicCAS(parent + a, a, b) == a)
            return;
    }
}

__global__ void k_union(int nTri, const uint32_t *__restrict__ newT, const int8_t *__restrict__ triMesh,
                        const uint64_t *keysA, const int *valsA, const uint64_t *keysB, const int *valsB,
                        uint32_t mask, const uint64_t *edgeKeys, const int *edgeVals, uint32_t emask,
                        uint32_t newBase, int *parent, int *seedFlag, unsigned int *dupCount)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nTri)
        return;
    const uint32_t *v = newT + 3 * (size_t)t;
    const uint64_t *keys = triMesh[t] == 0 ? keysA : keysB;
    const int *vals = triMesh[t] == 0 ? valsA : valsB;
    int seed = 0;
    for (int i = 0; i < 3; ++i) {
        uint32_t a = v[i], b = v[(i + 1) % 3];
        int owner = u64map_find(keys, vals, mask, he_key(a, b));
        if (owner != t)
            atomicAdd(dupCount, 1u);
        if (is_cut_edge(edgeKeys, edgeVals, emask, a, b, newBase)) {
            if (owner == t)
                seed = 1;
            continue;
        }
        if (owner != t)
            continue; // a repeated half-edge was already crossed by its first owner
        int tw = u64map_find(keys, vals, mask, he_key(b, a));
        if (tw >= 0)
            uf_union(parent, t, tw);
    }
    seedFlag[t] = seed;
}

// Grouping through the input adjacency (both input meshes hold every directed edge once). The per-mesh
// half-edge tables hold only the re-triangulated triangles (first owner wins; the meshes need separate tables
// because the cut points are shared vertices of both). The twin of an uncut triangle's edge is its input neighbour when that one is
// uncut, else a re-triangulated triangle of the neighbour found in the table; the twin of a re-triangulated
// triangle's edge is found in the table, or, on an original edge of its face, is the uncut neighbour across
// it. With every directed edge held once per mesh this crosses exactly the half-edges k_union crosses.
__global__ void k_halfedges_retri(int nRetri, int retriBase, const uint32_t *__restrict__ newT,
                                  const int8_t *__restrict__ triMesh, uint64_t *keysA, int *valsA, uint64_t *keysB,
                                  int *valsB, uint32_t mask)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nRetri)
        return;
    const int t = retriBase + r;
    const uint32_t *v = newT + 3 * (size_t)t;
    uint64_t *keys = triMesh[t] == 0 ? keysA : keysB;
    int *vals = triMesh[t] == 0 ? valsA : valsB;
    for (int i = 0; i < 3; ++i)
        u64map_insert_min(keys, vals, mask, he_key(v[i], v[(i + 1) % 3]), t);
}

__global__ void k_union_adj(int nTri, int uncutA, int uncutB, const uint32_t *__restrict__ newT,
                            const int8_t *__restrict__ triMesh, const int *__restrict__ origUncut,
                            const int *__restrict__ retriFace, const int *__restrict__ faceTri, MeshDev A, MeshDev B,
                            const int *__restrict__ cutA, const int *__restrict__ cutB,
                            const int *__restrict__ uncutRankA, const int *__restrict__ uncutRankB,
                            const uint64_t *keysA, const int *valsA, const uint64_t *keysB, const int *valsB,
                            uint32_t mask, const uint64_t *edgeKeys,
                            const int *edgeVals, uint32_t emask, uint32_t newBase, int *parent, int *seedFlag,
                            unsigned int *dupCount)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nTri)
        return;
    const int retriBase = uncutA + uncutB;
    const uint32_t *v = newT + 3 * (size_t)t;
    const int side = triMesh[t];
    const MeshDev &M = side == 0 ? A : B;
    const int *cut = side == 0 ? cutA : cutB;
    const int *urank = side == 0 ? uncutRankA : uncutRankB;
    const int outBase = side == 0 ? 0 : uncutA;
    const uint32_t vbase = side == 0 ? 0u : (uint32_t)A.nv;
    const uint64_t *keys = side == 0 ? keysA : keysB;
    const int *vals = side == 0 ? valsA : valsB;
    int seed = 0;
    if (t < retriBase) {
        const int i = origUncut[t];
        for (int k = 0; k < 3; ++k) {
            const int j = M.adj[3 * (size_t)i + k];
            if (j < 0)
                continue;
            // two uncut neighbours see each other (every directed edge is held once, so the adjacency is
            // symmetric): the edge is joined from its higher end only
            const int tw = !cut[j] ? outBase + urank[j]
                                   : u64map_find(keys, vals, mask, he_key(v[(k + 1) % 3], v[k]));
            if (tw >= 0 && (cut[j] || tw < t))
                uf_union(parent, t, tw);
        }
    } else {
        const int face = faceTri[retriFace[t - retriBase]];
        const uint32_t *c = M.t + 3 * (size_t)face;
        for (int i = 0; i < 3; ++i) {
            const uint32_t a = v[i], b = v[(i + 1) % 3];
            const int owner = u64map_find(keys, vals, mask, he_key(a, b));
            if (owner != t)
                atomicAdd(dupCount, 1u);
            if (is_cut_edge(edgeKeys, edgeVals, emask, a, b, newBase)) {
                if (owner == t)
                    seed = 1;
                continue;
            }
            if (owner != t)
                continue; // a repeated half-edge was already crossed by its first owner
            int tw = u64map_find(keys, vals, mask, he_key(b, a));
            if (tw < 0 && a < newBase && b < newBase) {
                for (int kk = 0; kk < 3; ++kk)
                    if (c[kk] + vbase == a && c[(kk + 1) % 3] + vbase == b) {
                        const int j = M.adj[3 * (size_t)face + kk];
                        if (j >= 0 && !cut[j])
                            tw = outBase + urank[j];
                        break;
                    }
            }
            if (tw >= 0)
                uf_union(parent, t, tw);
        }
    }
    seedFlag[t] = seed;
}

__global__ void k_uf_flatten(int n, int *parent)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n)
        return;
    parent[t] = uf_find(parent, t);
}

// representative triangle of each region: the smallest seed triangle, else the smallest uncut triangle
__global__ void k_region_rep(int nTri, const int *__restrict__ root, const int *__restrict__ seedFlag,
                             const int8_t *__restrict__ isUncut, int *seedMin, int *remMin)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nTri)
        return;
    int r = root[t];
    // lanes with the same root reduce first, so a big region costs one atomic per warp, not per triangle
    unsigned mask = __match_any_sync(__activemask(), r);
    int sv = (int)__reduce_min_sync(mask, (unsigned)(seedFlag[t] ? t : INT_MAX));
    int rv = (int)__reduce_min_sync(mask, (unsigned)(isUncut[t] ? t : INT_MAX));
    if ((threadIdx.x & 31) == __ffs(mask) - 1) {
        if (sv != INT_MAX)
            atomicMin(seedMin + r, sv);
        if (rv != INT_MAX)
            atomicMin(remMin + r, rv);
    }
}

// isPointInMesh (src/solidboolean.cpp:48-92) for one (region, axis) per warp: the 32 lanes pop up to 32
// LBVH nodes at a time from a per-warp shared-memory stack, test the children against the ray's box
// (FP32 boxes rounded outward, or exact FP64 boxes in the plain form), test reached triangles exactly in
// FP64 (closed-interval box test, plane hit, three same-sign normals) and collect the hit points; the
// parity of the number of distinct PositionKeys decides the axis.
// One axis ray of a region's representative triangle (src/solidboolean.cpp:482-510, 48-92): from the
// triangle's centroid p to e = p + (DBL_MAX on the axis, DBL_EPSILON on the others), its query box as the
// reference's tree query builds it (update with p then e), and the FP32 box rounded outward.
struct SideRay {
    d3 p, u;
    double qlo[3], qhi[3];
    float olo[3], ohi[3];
    int target; // mesh whose triangles the ray tests (the other mesh): 0 first, 1 second
    int region;
};

__device__ SideRay side_ray(int rep, int axis, int region, const uint32_t *__restrict__ newT,
                            const double *__restrict__ newV, const int8_t *__restrict__ triMesh)
{
    SideRay r;
    const uint32_t *tv = newT + 3 * (size_t)rep;
    const d3 v0 = mk(newV[3 * (size_t)tv[0]], newV[3 * (size_t)tv[0] + 1], newV[3 * (size_t)tv[0] + 2]);
    const d3 v1 = mk(newV[3 * (size_t)tv[1]], newV[3 * (size_t)tv[1] + 1], newV[3 * (size_t)tv[1] + 2]);
    const d3 v2 = mk(newV[3 * (size_t)tv[2]], newV[3 * (size_t)tv[2] + 1], newV[3 * (size_t)tv[2] + 2]);
    r.p = divs((v0 + v1) + v2, 3.0);
    const d3 ax = mk(axis == 0 ? kDblMax : kDblEps, axis == 1 ? kDblMax : kDblEps, axis == 2 ? kDblMax : kDblEps);
    const d3 e = r.p + ax;
    for (int k = 0; k < 3; ++k) {
        const double a = comp(r.p, k), b = comp(e, k);
        double lo = kDblMax, hi = -kDblMax; // AxisAlignedBoudingBox::update with p then e
        if (a > hi)
            hi = a;
        if (a < lo)
            lo = a;
        if (b > hi)
            hi = b;
        if (b < lo)
            lo = b;
        r.qlo[k] = lo;
        r.qhi[k] = hi;
        r.olo[k] = __double2float_rd(lo);
        r.ohi[k] = __double2float_ru(hi);
    }
    r.u = e - r.p;
    r.target = triMesh[rep] == 0 ? 1 : 0;
    r.region = region;
    return r;
}

// The reference's test of one triangle against the ray: box overlap in FP64, then the segment-plane
// intersection and the point-in-triangle test by normals. Writes the hit's PositionKey.
__device__ bool side_hit(const MeshDev &M, int ti, const SideRay &ray, double factor, Key &key)
{
    const double *bx = M.box64 + 6 * (size_t)ti;
    for (int k = 0; k < 3; ++k)
        if (!(bx[k] <= ray.qhi[k] && bx[3 + k] >= ray.qlo[k]))
            return false;
    const uint32_t *t = M.t + 3 * (size_t)ti;
    d3 tp[3];
    for (int k = 0; k < 3; ++k)
        tp[k] = mk(M.v[3 * (size_t)t[k]], M.v[3 * (size_t)t[k] + 1], M.v[3 * (size_t)t[k] + 2]);
    const d3 n = unit_normal(tp[0], tp[1], tp[2]);
    const d3 wv = ray.p - tp[0];
    const double d = dot(n, ray.u);
    const double nn = dot(neg(n), wv);
    if (fabs(d) <= kDblEps)
        return false;
    const double s = nn / d;
    if (s < 0 || s > 1 || isnan(s) || isinf(s))
        return false;
    const d3 x = ray.p + scale(s, ray.u);
    const d3 n0 = unit_normal(x, tp[0], tp[1]);
    const d3 n1 = unit_normal(x, tp[1], tp[2]);
    const d3 n2 = unit_normal(x, tp[2], tp[0]);
    if (!(dot(n0, n1) > 0 && dot(n0, n2) > 0))
        return false;
    key = make_key(x, factor);
    return true;
}

constexpr int kSideHits = 128; // hit keys kept per ray (more sets the side-error counter)

__device__ __forceinline__ void side_record(const SideRay &ray, int rayId, const MeshDev &M, int ti, double factor,
                                            Key *hits, int *hitCount, unsigned int *errors)
{
    Key key;
    if (!side_hit(M, ti, ray, factor, key))
        return;
    const int slot = atomicAdd(hitCount + rayId, 1);
    if (slot < kSideHits)
        hits[(size_t)rayId * kSideHits + slot] = key;
    else
        atomicAdd(errors, 1u);
}


// Few rays: every triangle of the target mesh against all rays, one thread per triangle (the triangle's box
// read once, the rays from shared memory), instead of one latency-bound tree walk per ray. The FP32 box
// against the outward-rounded query is conservative; side_hit then applies the reference's FP64 box test.
constexpr int kBruteRays = 96;

// three rays per side query (a group's first triangle, or a remaining region's smallest uncut triangle)
__global__ void k_side_rays(int nRays, const int *__restrict__ qTri, const uint32_t *__restrict__ newT,
                            const double *__restrict__ newV, const int8_t *__restrict__ triMesh, SideRay *rays,
                            int *hitCount)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nRays)
        return;
    const int q = w / 3;
    rays[w] = side_ray(qTri[q], w % 3, q, newT, newV, triMesh);
    hitCount[w] = 0;
}

template <bool FP64>
__global__ void __launch_bounds__(256) k_side_brute(int target, MeshDev M, int nRays, const SideRay *__restrict__ rays,
                                                    double factor, Key *hits, int *hitCount, unsigned int *errors)
{
    __shared__ SideRay sr[kBruteRays];
    __shared__ int ids[kBruteRays], nMine;
    if (threadIdx.x == 0) {
        int c = 0;
        for (int k = 0; k < nRays; ++k)
            if (rays[k].target == target)
                ids[c++] = k;
        nMine = c;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nMine; k += blockDim.x)
        sr[k] = rays[ids[k]];
    __syncthreads();
    const int n = nMine;
    for (int ti = blockIdx.x * blockDim.x + threadIdx.x; ti < M.nt; ti += gridDim.x * blockDim.x) {
        float b32[6];
        double b64[6];
        if (FP64)
            for (int k = 0; k < 6; ++k)
                b64[k] = M.box64[6 * (size_t)ti + k];
        else
            for (int k = 0; k < 6; ++k)
                b32[k] = M.box32[6 * (size_t)ti + k];
        for (int k = 0; k < n; ++k) {
            const SideRay &ray = sr[k];
            bool over = true;
            for (int a = 0; a < 3; ++a)
                over = over && (FP64 ? (b64[a] <= ray.qhi[a] && b64[3 + a] >= ray.qlo[a])
                                     : (b32[a] <= ray.ohi[a] && b32[3 + a] >= ray.olo[a]));
            if (!over)
                continue;
            Key key;
            if (!side_hit(M, ti, ray, factor, key))
                continue;
            const int id = ids[k];
            const int slot = atomicAdd(hitCount + id, 1);
            if (slot < kSideHits)
                hits[(size_t)id * kSideHits + slot] = key;
            else
                atomicAdd(errors, 1u);
        }
    }
}

// the exact test of the listed (ray, triangle) pairs, one per thread
__global__ void k_side_pairs(const int *__restrict__ pairCount, int pairCap, const int2 *__restrict__ pairs,
                             const SideRay *__restrict__ rays, MeshDev A, MeshDev B, double factor, Key *hits,
                             int *hitCount, unsigned int *errors)
{
    const int n = min(*pairCount, pairCap);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int2 pr = pairs[q];
        const SideRay ray = rays[pr.x];
        side_record(ray, pr.x, ray.target == 0 ? A : B, pr.y, factor, hits, hitCount, errors);
    }
}

// one warp per ray: distinct hit keys (the reference's std::set<PositionKey>), odd count = inside
__global__ void k_side_parity(int nRays, const SideRay *__restrict__ rays, const Key *__restrict__ hits,
                              const int *__restrict__ hitCount, int *insideCount)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nRays)
        return;
    const Key *h = hits + (size_t)w * kSideHits;
    const int nh = min(hitCount[w], kSideHits);
    int distinct = 0;
    for (int i = lane; i < nh; i += 32) {
        bool dup = false;
        for (int j = 0; j < i && !dup; ++j)
            dup = key_eq(h[j], h[i]);
        distinct += dup ? 0 : 1;
    }
    for (int o = 16; o > 0; o >>= 1)
        distinct += __shfl_xor_sync(0xFFFFFFFFu, distinct, o);
    if (lane == 0 && distinct % 2 != 0)
        atomicAdd(insideCount + rays[w].region, 1);
}

// Many rays: one warp per ray walks the other mesh's LBVH (a node stack in shared memory, up to 32 nodes per
// step) with the query box, FP32 node boxes and FP32 leaf boxes rounded conservatively (FP64 boxes in the
// plain FP64 form), and lists the leaves that pass as (ray, triangle) pairs; the exact test then runs one pair
// per lane in k_side_pairs. Pairs beyond the list's capacity are tested in place.
constexpr int kTreeWarps = 4;
constexpr int kSideStack = 1536; // nodes per warp

template <bool FP64>
__global__ void __launch_bounds__(32 * kTreeWarps)
    k_tree_rays(int nRays, const SideRay *__restrict__ rays, MeshDev A, MeshDev B, double factor, Key *hits,
                int *hitCount, unsigned int *errors, int2 *pairs, int *pairCount, int pairCap)
{
    __shared__ int stack[kTreeWarps][kSideStack];
    __shared__ int spS[kTreeWarps];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned full = 0xFFFFFFFFu;
    const int w = blockIdx.x * kTreeWarps + wl;
    if (w >= nRays)
        return;
    const SideRay ray = rays[w];
    const MeshDev &M = ray.target == 0 ? A : B;
    if (M.nt <= 0)
        return;
    auto leaf = [&](int ti) {
        bool over = true;
        for (int k = 0; k < 3; ++k) {
            if (FP64) {
                const double *bx = M.box64 + 6 * (size_t)ti;
                over = over && bx[k] <= ray.qhi[k] && bx[3 + k] >= ray.qlo[k];
            } else {
                const float *bx = M.box32 + 6 * (size_t)ti;
                over = over && bx[k] <= ray.ohi[k] && bx[3 + k] >= ray.olo[k];
            }
        }
        if (!over)
            return;
        const int slot = atomicAdd(pairCount, 1);
        if (slot < pairCap)
            pairs[slot] = make_int2(w, ti);
        else
            side_record(ray, w, M, ti, factor, hits, hitCount, errors);
    };
    if (M.root < 0) {
        if (lane == 0)
            leaf(M.leafTri[0]);
        return;
    }
    if (lane == 0) {
        stack[wl][0] = M.root;
        spS[wl] = 1;
    }
    __syncwarp();
    for (int iter = 0; iter < (1 << 20); ++iter) {
        const int sp = spS[wl];
        const int n = min(sp, 32);
        if (n == 0)
            break;
        const int node = lane < n ? stack[wl][sp - n + lane] : -1;
        __syncwarp();
        int push[2] = {-1, -1};
        if (node >= 0) {
            const int2 ch = M.child[node];
            const int cs[2] = {ch.x, ch.y};
            for (int k = 0; k < 2; ++k) {
                const int c = cs[k];
                if (c < 0) {
                    leaf(M.leafTri[~c]);
                    continue;
                }
                bool hit;
                if (FP64) {
                    const double *bx = M.nbox64 + 6 * (size_t)c;
                    hit = ray.qlo[0] <= bx[3] && ray.qhi[0] >= bx[0] && ray.qlo[1] <= bx[4] && ray.qhi[1] >= bx[1] &&
                          ray.qlo[2] <= bx[5] && ray.qhi[2] >= bx[2];
                } else {
                    const float4 *bx = reinterpret_cast<const float4 *>(M.nbox32) + 2 * (size_t)c;
                    const float4 lo = __ldg(bx), hi = __ldg(bx + 1);
                    hit = ray.olo[0] <= hi.x && ray.ohi[0] >= lo.x && ray.olo[1] <= hi.y && ray.ohi[1] >= lo.y &&
                          ray.olo[2] <= hi.z && ray.ohi[2] >= lo.z;
                }
                if (hit)
                    push[k] = c;
            }
        }
        const int cnt = (push[0] >= 0) + (push[1] >= 0);
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(full, incl, o);
            if (lane >= o)
                incl += v;
        }
        const int total = __shfl_sync(full, incl, 31);
        const int base = sp - n;
        if (base + total > kSideStack) {
            if (lane == 0)
                atomicAdd(errors, 1u);
            break;
        }
        int pos = base + incl - cnt;
        for (int k = 0; k < 2; ++k)
            if (push[k] >= 0)
                stack[wl][pos++] = push[k];
        __syncwarp();
        if (lane == 0)
            spS[wl] = base + total;
        __syncwarp();
    }
}

// fetch flags: union keeps outside of both, intersect inside of both, diff outside of the first and
// inside of the second (reversed) (src/solidboolean.cpp:512-565)
// Selection of the three results (src/solidboolean.cpp:512-570): union keeps the first mesh's outside and the
// second's outside, intersect both insides, diff the first's outside and the second's inside with its
// winding reversed. Flags of the three ops are laid out back to back, [op * (nTri + 1) + t], each run ending
// in a zero, so one exclusive scan ranks all three: op k's output position is its rank minus the rank at the
// start of its run.
__device__ __forceinline__ int fetch_keep(int l, int mesh, int op)
{
    if (l < 0)
        return 0;
    if (op == 0)
        return l == 0;
    if (op == 2)
        return l == 1;
    return mesh == 0 ? (l == 0) : (l == 1);
}

__global__ void k_fetch_flags(int nTri, const int8_t *__restrict__ label, const int8_t *__restrict__ triMesh,
                              int *flag)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > nTri)
        return;
    const size_t stride = (size_t)nTri + 1;
    if (t == nTri) {
        for (int op = 0; op < 3; ++op)
            flag[op * stride + t] = 0;
        return;
    }
    const int l = label[t], m = triMesh[t];
    for (int op = 0; op < 3; ++op)
        flag[op * stride + t] = fetch_keep(l, m, op);
}

__global__ void k_fetch_write(int nTri, const int *__restrict__ flag, const int *__restrict__ rank,
                              const uint32_t *__restrict__ newT, const int8_t *__restrict__ triMesh, uint32_t *out0,
                              uint32_t *out1, uint32_t *out2)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nTri)
        return;
    const size_t stride = (size_t)nTri + 1;
    const uint32_t *v = newT + 3 * (size_t)t;
    const uint32_t a = v[0], b = v[1], c = v[2];
    const bool flip = triMesh[t] == 1;
    uint32_t *outs[3] = {out0, out1, out2};
    for (int op = 0; op < 3; ++op) {
        if (!flag[op * stride + t])
            continue;
        uint32_t *o = outs[op] + 3 * (size_t)(rank[op * stride + t] - rank[op * stride]);
        if (op == 1 && flip) {
            o[0] = c;
            o[1] = b;
            o[2] = a;
        } else {
            o[0] = a;
            o[1] = b;
            o[2] = c;
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------------------------------
static inline int nb(size_t n, int bs) { return (int)((n + bs - 1) / bs); }

void launch_weld(const AsmArgs &g, cudaStream_t s)
{
    if (g.nFaces <= 0)
        return;
    {
        KTime kt("k_weld_insert", s);
        SB_COUNT(k_weld_insert)<<<g.nFaces, 32, 0, s>>>(g.nFaces, g.ptOff, g.ptRef, g.faceNpts, g.cutKeys, g.weldOwner,
                                                        g.weldMin, g.weldMask, g.pointSlot);
    }
    {
        KTime kt("k_weld_first", s);
        SB_COUNT(k_weld_first)<<<g.nFaces, 32, 0, s>>>(g.nFaces, g.ptOff, g.ptRef, g.faceNpts, g.pointSlot, g.weldMin,
                                                       g.isFirst);
    }
}

void launch_weld_number(const AsmArgs &g, int nSeq, cudaStream_t s)
{
    if (nSeq <= 0 || g.nFaces <= 0)
        return;
    {
        KTime kt("k_weld_number", s);
        SB_COUNT(k_weld_number)<<<g.nFaces, 32, 0, s>>>(g.nFaces, g.ptOff, g.ptRef, g.faceNpts, g.isFirst, g.firstRank,
                                                        g.pointSlot, g.slotRank, g.cutPts, g.newV, g.newBase, g.ptSrc,
                                                        g.newSrc);
    }
}

void launch_mark_cut(const AsmArgs &g, cudaStream_t s)
{
    if (g.nFaces > 0)
        {
            KTime kt("k_mark_cut", s);
            SB_COUNT(k_mark_cut)<<<nb(g.nFaces, 256), 256, 0, s>>>(g.nFaces, g.faceSide, g.faceTri, g.cutA, g.cutB);
        }
}

void launch_arrangement(const AsmArgs &g, cudaStream_t s)
{
    if (g.A.nt > 0)
        {
            KTime kt("k_uncut", s);
            SB_COUNT(k_uncut)<<<nb(g.A.nt, 256), 256, 0, s>>>(g.A.nt, g.A.t, g.cutA, g.uncutRankA, 0u, 0u, g.newT,
                                                              g.origUncut, g.truncOcc);
        }
    if (g.B.nt > 0)
        {
            KTime kt("k_uncut", s);
            SB_COUNT(k_uncut)<<<nb(g.B.nt, 256), 256, 0, s>>>(g.B.nt, g.B.t, g.cutB, g.uncutRankB, (uint32_t)g.A.nv,
                                                (uint32_t)g.uncutA, g.newT, g.origUncut, g.truncOcc + 1);
        }
    if (g.nFaces > 0)
        {
            KTime kt("k_retri", s);
            SB_COUNT(k_retri)<<<g.nFaces, 32, 0, s>>>(g.nFaces, g.faceSide, g.faceTri, g.faceNtris, g.triOff, g.retriRank,
                                        g.faceTris, g.ptOff, g.pointSlot, g.slotRank, g.A, g.B,
                                        (uint32_t)g.newBase, (uint32_t)(g.uncutA + g.uncutB), g.newT, g.retriFace);
        }
}

void launch_loops(const AsmArgs &g, cudaStream_t s)
{
    if (g.nFaces > 0)
        {
            KTime kt("k_cut_edges", s);
            SB_COUNT(k_cut_edges)<<<g.nFaces, 32, 0, s>>>(g.nFaces, g.faceSide, g.faceNedges, g.edgeOff, g.edgeRef,
                                                          g.faceEdges, g.ptOff, g.pointSlot, g.slotRank, g.edgeKeys,
                                                          g.edgeVals, g.edgeMask, g.edgeSlotLo, g.edgeSlotHi,
                                                          g.firstOcc, 0);
        }
    {
        KTime kt("k_loop_degree", s);
        SB_COUNT(k_loop_degree)<<<nb((size_t)g.edgeMask + 1, 256), 256, 0, s>>>(g.edgeMask + 1, g.edgeKeys, g.edgeSlotLo,
                                                                               g.edgeSlotHi, g.degree, g.nbr,
                                                                               g.nbrSlot);
    }
    if (g.nNew > 0)
        {
            KTime kt("k_loop_check", s);
            SB_COUNT(k_loop_check)<<<nb(g.nNew, 256), 256, 0, s>>>(g.nNew, g.degree, g.counters + kCntLoopVerts);
        }
}

void launch_halfedges(const AsmArgs &g, cudaStream_t s)
{
    if (g.nTri <= 0)
        return;
    if (g.useAdj) {
        const int retriBase = g.uncutA + g.uncutB, nRetri = g.nTri - retriBase;
        if (nRetri > 0) {
            KTime kt("k_halfedges", s);
            SB_COUNT(k_halfedges_retri)<<<nb(nRetri, 256), 256, 0, s>>>(nRetri, retriBase, g.newT, g.triMesh,
                                                                       g.heKeysA, g.heValsA, g.heKeysB, g.heValsB,
                                                                       g.heMask);
        }
    } else {
        KTime kt("k_halfedges", s);
        SB_COUNT(k_halfedges)<<<nb(g.nTri, 256), 256, 0, s>>>(g.nTri, g.newT, g.triMesh, g.heKeysA, g.heValsA,
                                                             g.heKeysB, g.heValsB, g.heMask, g.uncutA + g.uncutB,
                                                             g.origUncut, g.truncOcc);
    }
}

void launch_groups(const AsmArgs &g, cudaStream_t s)
{
    if (g.nTri <= 0)
        return;
    if (g.useAdj) {
        KTime kt("k_union", s);
        SB_COUNT(k_union_adj)<<<nb(g.nTri, 256), 256, 0, s>>>(
            g.nTri, g.uncutA, g.uncutB, g.newT, g.triMesh, g.origUncut, g.retriFace, g.faceTri, g.A, g.B, g.cutA,
            g.cutB, g.uncutRankA, g.uncutRankB, g.heKeysA, g.heValsA, g.heKeysB, g.heValsB, g.heMask, g.edgeKeys,
            g.edgeVals, g.edgeMask,
            (uint32_t)g.newBase, g.parent, g.seedFlag, g.counters + kCntDupHalfedge);
    } else {
        KTime kt("k_union", s);
        SB_COUNT(k_union)<<<nb(g.nTri, 256), 256, 0, s>>>(g.nTri, g.newT, g.triMesh, g.heKeysA, g.heValsA, g.heKeysB,
                                                         g.heValsB, g.heMask, g.edgeKeys, g.edgeVals, g.edgeMask,
                                                         (uint32_t)g.newBase, g.parent, g.seedFlag,
                                                         g.counters + kCntDupHalfedge);
    }
    {
        KTime kt("k_uf_flatten", s);
        SB_COUNT(k_uf_flatten)<<<nb(g.nTri, 256), 256, 0, s>>>(g.nTri, g.parent);
    }
    {
        KTime kt("k_region_rep", s);
        SB_COUNT(k_region_rep)<<<nb(g.nTri, 256), 256, 0, s>>>(g.nTri, g.parent, g.seedFlag, g.isUncut, g.seedMin, g.remMin);
    }
}

constexpr int kPairsPerRay = 64; // pair-list capacity per ray (more are tested in place)

size_t side_layout(AsmArgs &g, int nRays, char *base)
{
    Carve c;
    const size_t n = (size_t)std::max(nRays, 1);
    const size_t oRays = c.take<SideRay>(n), oHits = c.take<Key>(n * kSideHits), oCnt = c.take<int>(n + 1);
    const size_t oPairs = c.take<int2>(kPairsPerRay * n);
    if (base) {
        g.sideRays = base + oRays;
        g.sideHits = base + oHits;
        g.sideHitCount = reinterpret_cast<int *>(base + oCnt);
        g.sidePairs = base + oPairs;
        g.sidePairCap = (int)(kPairsPerRay * n);
    }
    return c.off;
}

void launch_sides(const AsmArgs &g, unsigned int nQueries, bool fp64, cudaStream_t s)
{
    const int nRays = 3 * (int)nQueries;
    if (nQueries > 0) {
        KTime kt("k_sides", s);
        SideRay *rays = reinterpret_cast<SideRay *>(g.sideRays);
        Key *hits = reinterpret_cast<Key *>(g.sideHits);
        int *pairCount = g.sideHitCount + nRays; // one past the per-ray counts
        cudaMemsetAsync(pairCount, 0, sizeof(int), s);
        SB_COUNT(k_side_rays)<<<nb(nRays, 128), 128, 0, s>>>(nRays, g.qTri, g.newT, g.newV, g.triMesh, rays,
                                                             g.sideHitCount);
        if (nRays <= kBruteRays) {
            // few rays: every triangle against all of them
            for (int target = 0; target < 2; ++target) {
                const MeshDev &M = target == 0 ? g.A : g.B;
                if (M.nt <= 0)
                    continue;
                const int grid = std::min(nb(M.nt, 256), 152 * 8);
                count_launch();
                if (fp64)
                    k_side_brute<true><<<grid, 256, 0, s>>>(target, M, nRays, rays, g.factor, hits, g.sideHitCount,
                                                            g.counters + kCntSideErrors);
                else
                    k_side_brute<false><<<grid, 256, 0, s>>>(target, M, nRays, rays, g.factor, hits, g.sideHitCount,
                                                             g.counters + kCntSideErrors);
            }
        } else {
            int2 *pairs = reinterpret_cast<int2 *>(g.sidePairs);
            count_launch();
            if (fp64)
                k_tree_rays<true><<<nb(nRays, kTreeWarps), 32 * kTreeWarps, 0, s>>>(
                    nRays, rays, g.A, g.B, g.factor, hits, g.sideHitCount, g.counters + kCntSideErrors, pairs,
                    pairCount, g.sidePairCap);
            else
                k_tree_rays<false><<<nb(nRays, kTreeWarps), 32 * kTreeWarps, 0, s>>>(
                    nRays, rays, g.A, g.B, g.factor, hits, g.sideHitCount, g.counters + kCntSideErrors, pairs,
                    pairCount, g.sidePairCap);
            SB_COUNT(k_side_pairs)<<<nb(g.sidePairCap, 128), 128, 0, s>>>(pairCount, g.sidePairCap, pairs, rays, g.A,
                                                                          g.B, g.factor, hits, g.sideHitCount,
                                                                          g.counters + kCntSideErrors);
        }
        SB_COUNT(k_side_parity)<<<nb(32 * (size_t)nRays, 128), 128, 0, s>>>(nRays, rays, hits, g.sideHitCount,
                                                                            g.insideCount);
    }
}

void launch_fetch_flags(const AsmArgs &g, int *flag, cudaStream_t s)
{
    KTime kt("k_fetch_flags", s);
    SB_COUNT(k_fetch_flags)<<<nb((size_t)g.nTri + 1, 256), 256, 0, s>>>(g.nTri, g.label, g.triMesh, flag);
}

void launch_fetch_write(const AsmArgs &g, const int *flag, const int *rank, uint32_t *const out[3], cudaStream_t s)
{
    if (g.nTri > 0) {
        KTime kt("k_fetch_write", s);
        SB_COUNT(k_fetch_write)<<<nb(g.nTri, 256), 256, 0, s>>>(g.nTri, flag, rank, g.newT, g.triMesh, out[0], out[1],
                                                                 out[2]);
    }
}

} // namespace sbg
