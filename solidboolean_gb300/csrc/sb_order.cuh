// The reference's processing orders, reproduced on the GPU (launch interface).
//
// The reference's observable results depend on the iteration order of its standard hash containers:
//   * cut faces are re-triangulated in the order of unordered_map<size_t, IntersectedContext>
//     (src/solidboolean.cpp:352-358), which numbers the appended vertices (addNewPoint, :241-248) and the
//     re-triangulated triangles, and orders the cut edges that build the loop map (:397-404);
//   * the loops are listed in the order of unordered_map<size_t, unordered_set<size_t>> (:124-165), each
//     starting at its first vertex in that order and going towards its neighbour the set lists first;
//   * the face groups are seeded from the loops in that order and flooded first in, first out (:167-239);
//     each group's side is decided from its first triangle (:482-510).
// This file computes those orders with data-parallel kernels (see sb_order.cu).
#pragma once
#include "sb_assemble.cuh"
#include "sb_common.cuh"
#include "sb_internal.h"

namespace sbg {

// Scratch of one hash-order problem of n keys (hash_order_block) for the stages that do not fit in shared
// memory: 4 n + 2 n + 1 ints, plus 2 bucket arrays of hash_bucket_count(n) ints.
struct HashScratch {
    int *posA, *posB, *slotOf, *nxt, *runSize;
    int *bmin, *head;
};
size_t hash_scratch_ints(int n);
HashScratch hash_scratch_at(int *base, int n);

struct FaceOrderArgs {
    int nFaces, FA, FB;
    const int *faceTri, *faceBegin, *pairIdx;
    const uint32_t *pairAB;
    MeshDev A, B;
    int exact; // both meshes have the reference tree: order by its traversal, else by triangle index
    unsigned long long *key;   // [nFaces] traversal key of each face's first pair
    int *val;                  // [nFaces] face ids
    const int *sortedVal;      // [nFaces] faces sorted by key (mesh first)
    int *sortedOut;            // the same array, written by k_face_ctx when it sorts (blockSort)
    int blockSort;             // k_face_ctx sorts each mesh's faces by key itself (face_ctx_block_sort)
    int *faceRank;             // [nFaces] position in the reference's processing order (first mesh first)
    int *faceByRank;           // [nFaces]
    uint32_t *insKeys;         // [nFaces] scratch
    HashScratch hs[2];         // per mesh
    unsigned int *overflow;    // faces whose traversal path did not fit the key
};
// traversal key of each face's first intersecting pair (k_face_keys)
void launch_face_keys(const FaceOrderArgs &a, cudaStream_t s);
// faces sorted by key -> context-map iteration order per mesh (k_face_ctx)
void launch_face_ctx(const FaceOrderArgs &a, cudaStream_t s);
// whether k_face_ctx can sort each mesh's faces by key in its own block (up to 8,192 faces per mesh); else
// the caller sorts them device-wide into sortedVal first
bool face_ctx_block_sort(int FA, int FB);

// Exclusive scans of per-face values taken in the processing order: out[f] = sum of vals over the faces
// ranked before f; tot[0] = sum over the first mesh's faces, tot[1] = sum over all. Up to three arrays.
struct RankScanArgs {
    int n, FA, count;
    const int *faceByRank, *faceRank;
    const int *vals[3];
    int *out[3];   // [n + 1]
    int *tmp[3];   // [n + 1] scratch
    int *tot[3];   // [2]
    int *part;     // [3 * 1024] block partial sums (the multi-block form, past kRankScanBlockMax faces)
};
void launch_rank_scan(const RankScanArgs &a, cudaStream_t s);

// Loops, seeds and group representatives (k_loop_order, one block, then grid-wide seed kernels).
struct LoopOrderArgs {
    int nNew, nTri;
    uint32_t newBase;
    int slotDomain; // every first occurrence lies below it
    const int *degree, *nbr, *nbrSlot, *firstOcc;
    const unsigned int *loopBad;
    unsigned int *loopErr; // counts an iteration order that was not a permutation (nothing is seeded then)
    const uint64_t *heKeysA, *heKeysB;
    const int *heValsA, *heValsB;
    uint32_t heMask;
    // outputs
    int *seedTri;   // [2][2 nNew]: triangle of each seed entry (-1 none), mesh-major
    int *entryLoop; // [nNew] loop of each loop position
    int *firstQ;    // [nTri] first seed entry of each triangle (INT_MAX: none), filled in by the kernel
    int *group0;    // [2][2 nNew] first live entry of each group (INT_MAX: empty)
    int *gQuery;    // [2][2 nNew] side query of each group (-1: none)
    int *entryBase, *entryNext; // [nNew] per loop vertex: its loop position in the entry sequence, the next vertex
    int *qTri;      // side queries: their triangles
    unsigned int *qCount;
    int *info;      // [2] loop vertices, loops
    // scratch
    int *insRank, *hashOut;   // [nNew]
    uint32_t *insKeys;        // [nNew]
    int2 *vis;                // [2 nNew]
    HashScratch hs;           // for n = nNew
    int *scratch;             // loop_order_scratch_ints(): what does not fit in shared memory
    long long smemInts;       // set by launch_loop_order
    unsigned long long *stamps; // [8] device time at the phase boundaries (diagnostics; may be null)
};
size_t loop_order_scratch_ints(int slotDomain, int nNew);
// the loop order (one block); it needs the loop tables only
void launch_loop_order(LoopOrderArgs a, cudaStream_t s);
// the seed entries and each group's first entry (grid-wide); they need the loop order and the half-edge tables
void launch_seed_entries(const LoopOrderArgs &a, cudaStream_t s);
// side queries of the groups and of the regions without seeds (needs the union-find regions)
void launch_side_queries(const AsmArgs &g, const LoopOrderArgs &a, cudaStream_t s);

// Side of each region from its groups, then the exact first-in-first-out flood of the regions whose groups
// were decided differently, then the per-triangle labels.
struct FloodArgs {
    int nTri, nNew;
    const int *root, *seedMin;
    const int *seedTri, *firstQ, *entryLoop, *gQuery, *info;
    const int *insideCount, *regionQuery;
    int *rsMin, *rsMax;  // [nTri] per region: smallest / largest side among its live groups (2 / -1: none)
    int *bfsGroup;       // [nTri] group of each triangle reached by the flood (-1)
    int *best, *front0, *front1, *tgt, *flag; // scratch: nTri, nTri, nTri, 3 nTri, max(3 nTri, 4 nNew) + 1
    int *anyMixed;       // [1] set when some region's groups were decided differently (zeroed by the caller)
    unsigned int *errors;
};
void launch_flood_labels(const AsmArgs &g, const FloodArgs &f, cudaStream_t s);

} // namespace sbg
