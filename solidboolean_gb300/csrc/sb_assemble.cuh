// Assembly / labelling launch interface.
#pragma once
#include "sb_common.cuh"
#include "sb_hash.cuh"
#include "sb_internal.h"

namespace sbg {

// device counters (unsigned int) used by the assembly kernels
enum {
    kCntLoopVerts = 0,   // [0] loop vertices, [1] loop vertices with degree != 2
    kCntDupHalfedge = 2, // triangles' half-edges whose table owner is another triangle
    kCntReps = 3,        // number of side queries (groups' first triangles, remaining regions)
    kCntRegionsA = 4,    // [4] first mesh, [5] second mesh
    kCntSideErrors = 6,  // hit-buffer or stack overflow in the side rays
    kCntCount = 8
};

struct AsmArgs {
    MeshDev A, B;
    double factor;
    int nFaces;
    const int *faceSide, *faceTri, *faceNpts, *faceNtris, *faceNedges;
    const int *ptOff, *triOff, *edgeOff;
    const d3 *cutPts;
    const Key *cutKeys;
    const int *faceTris, *faceEdges;
    // weld
    int *weldOwner, *weldMin;
    uint32_t weldMask;
    int *pointSlot, *isFirst, *firstRank, *slotRank;
    const int *ptRef;   // per face: its points' first position in the reference's sequence (processing order)
    int newBase; // = A.nv + B.nv
    const int *ptSrc; // per cut point: 2 x (intersecting pair) + segment end (see FaceArgs::ptSrc)
    int *newSrc;      // per appended vertex: the source of the point that represents its weld class
    int nNew;    // unique cut points
    double *newV;
    // arrangement
    int *cutA, *cutB, *uncutRankA, *uncutRankB;
    int uncutA, uncutB;
    const int *retriRank; // per face: offset of its triangles within the re-triangulated block
    uint32_t *newT;
    int nTri;
    int8_t *triMesh, *isUncut;
    // loops
    uint64_t *edgeKeys;
    int *edgeVals;
    uint32_t edgeMask;
    int *degree;
    const int *edgeRef;          // per face: its directed cut edges' first position in the processing order
    int *edgeSlotLo, *edgeSlotHi; // per edge-table slot: when each end joined the other's neighbour set
    int *firstOcc;               // per appended vertex: its first slot in the loop map's insertion sequence
    int *nbr, *nbrSlot;          // per appended vertex: two neighbours on the loops and their joining slots
    // groups
    uint64_t *heKeysA, *heKeysB;
    int *heValsA, *heValsB;
    uint32_t heMask;
    // repOfRoot: per region root, its side query (-1: none); qTri: each side query's triangle; insideCount: per
    // query, the rays (of three) that found the point inside
    int *parent, *seedFlag, *seedMin, *remMin, *repOfRoot, *qTri, *insideCount;
    // grouping through the input meshes' edge adjacency (both meshes hold every directed edge once): the
    // per-mesh half-edge tables then hold the re-triangulated triangles only
    int useAdj;
    int *origUncut;  // [uncutA + uncutB] input triangle of each uncut arrangement triangle
    // [2] per mesh, 3 i + k of the first uncut triangle edge whose half-edge repeats an earlier one (INT_MAX:
    // none): the reference stops adding that mesh's uncut triangles there, keeping triangle i and the
    // half-edges inserted before the repeat (src/solidboolean.cpp:250-286)
    const int *truncOcc;
    int *retriFace;  // [nTri - uncutA - uncutB] face of each re-triangulated triangle
    int8_t *label;
    unsigned int *counters;
    // side rays: per ray its setup, hit keys and hit count, and the (ray, triangle) pairs for the exact test
    void *sideRays, *sideHits, *sidePairs;
    int *sideHitCount; // nRays + 1: the last one counts the pairs
    int sidePairCap;
};

#ifdef __CUDACC__
// (u, v) lies on a cut loop: both are appended vertices and the first mesh's cut edges hold the pair
__device__ __forceinline__ bool is_cut_edge(const uint64_t *edgeKeys, const int *edgeVals, uint32_t emask, uint32_t u,
                                            uint32_t v, uint32_t newBase)
{
    if (u < newBase || v < newBase)
        return false;
    uint32_t a = u - newBase, b = v - newBase;
    uint32_t lo = min(a, b), hi = max(a, b);
    return u64map_find(edgeKeys, edgeVals, emask, ((uint64_t)lo << 32) | hi) >= 0;
}

// The triangle the reference's flood reaches from arrangement triangle t across its edge i (v[i] -> v[i+1]),
// or -1: the half-edge is a cut-loop edge, t is not its table owner (a repeated half-edge is crossed by its
// first owner only), or the reverse half-edge has no owner (src/solidboolean.cpp:212-229). Through the input
// adjacency when both meshes hold every directed edge once (the tables then hold the re-triangulated
// triangles only), else through the full half-edge tables.
__device__ __forceinline__ int arr_twin(const AsmArgs &g, int t, int i)
{
    const int retriBase = g.uncutA + g.uncutB;
    const uint32_t *v = g.newT + 3 * (size_t)t;
    const int side = g.triMesh[t];
    const MeshDev &M = side == 0 ? g.A : g.B;
    const uint64_t *keys = side == 0 ? g.heKeysA : g.heKeysB;
    const int *vals = side == 0 ? g.heValsA : g.heValsB;
    const uint32_t a = v[i], b = v[(i + 1) % 3];
    const uint32_t newBase = (uint32_t)g.newBase;
    if (g.useAdj && t < retriBase) {
        const int *cut = side == 0 ? g.cutA : g.cutB;
        const int *urank = side == 0 ? g.uncutRankA : g.uncutRankB;
        const int outBase = side == 0 ? 0 : g.uncutA;
        const int j = M.adj[3 * (size_t)g.origUncut[t] + i];
        if (j < 0)
            return -1;
        return !cut[j] ? outBase + urank[j] : u64map_find(keys, vals, g.heMask, he_key(b, a));
    }
    const int owner = u64map_find(keys, vals, g.heMask, he_key(a, b));
    if (is_cut_edge(g.edgeKeys, g.edgeVals, g.edgeMask, a, b, newBase) || owner != t)
        return -1;
    int tw = u64map_find(keys, vals, g.heMask, he_key(b, a));
    if (g.useAdj && tw < 0 && a < newBase && b < newBase) {
        // an original edge of the cut face: the uncut neighbour across it
        const int *cut = side == 0 ? g.cutA : g.cutB;
        const int *urank = side == 0 ? g.uncutRankA : g.uncutRankB;
        const int outBase = side == 0 ? 0 : g.uncutA;
        const uint32_t vbase = side == 0 ? 0u : (uint32_t)g.A.nv;
        const int face = g.faceTri[g.retriFace[t - retriBase]];
        const uint32_t *c = M.t + 3 * (size_t)face;
        for (int kk = 0; kk < 3; ++kk)
            if (c[kk] + vbase == a && c[(kk + 1) % 3] + vbase == b) {
                const int j = M.adj[3 * (size_t)face + kk];
                if (j >= 0 && !cut[j])
                    tw = outBase + urank[j];
                break;
            }
    }
    return tw;
}
#endif

void launch_weld(const AsmArgs &g, cudaStream_t s);
void launch_weld_number(const AsmArgs &g, int nSeq, cudaStream_t s);
void launch_mark_cut(const AsmArgs &g, cudaStream_t s);
void launch_arrangement(const AsmArgs &g, cudaStream_t s);
void launch_loops(const AsmArgs &g, cudaStream_t s);
// the per-mesh half-edge tables (owners of directed edges)
void launch_halfedges(const AsmArgs &g, cudaStream_t s);
// union-find regions over the arrangement (after launch_halfedges), each region's seed and uncut minima
void launch_groups(const AsmArgs &g, cudaStream_t s);
void launch_sides(const AsmArgs &g, unsigned int nQueries, bool fp64, cudaStream_t s);
// layout of the side-ray buffers for nRays rays (base null: bytes only)
size_t side_layout(AsmArgs &g, int nRays, char *base);
// the three results at once: flags [op * (nTri + 1) + t], one exclusive scan over all 3 (nTri + 1), writes
void launch_fetch_flags(const AsmArgs &g, int *flag, cudaStream_t s);
void launch_fetch_write(const AsmArgs &g, const int *flag, const int *rank, uint32_t *const out[3], cudaStream_t s);

} // namespace sbg
