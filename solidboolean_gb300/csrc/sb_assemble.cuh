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
    kCntReps = 3,        // number of regions with a representative
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
    // groups
    uint64_t *heKeysA, *heKeysB;
    int *heValsA, *heValsB;
    uint32_t heMask;
    int *parent, *seedFlag, *seedMin, *remMin, *repOfRoot, *reps, *insideCount;
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

void launch_weld(const AsmArgs &g, cudaStream_t s);
void launch_weld_number(const AsmArgs &g, int nSeq, cudaStream_t s);
void launch_mark_cut(const AsmArgs &g, cudaStream_t s);
void launch_arrangement(const AsmArgs &g, cudaStream_t s);
void launch_loops(const AsmArgs &g, cudaStream_t s);
void launch_groups(const AsmArgs &g, cudaStream_t s);
void launch_sides(const AsmArgs &g, unsigned int nReps, bool fp64, cudaStream_t s);
// layout of the side-ray buffers for nRays rays (base null: bytes only)
size_t side_layout(AsmArgs &g, int nRays, char *base);
// the three results at once: flags [op * (nTri + 1) + t], one exclusive scan over all 3 (nTri + 1), writes
void launch_fetch_flags(const AsmArgs &g, int *flag, cudaStream_t s);
void launch_fetch_write(const AsmArgs &g, const int *flag, const int *rank, uint32_t *const out[3], cudaStream_t s);

} // namespace sbg
