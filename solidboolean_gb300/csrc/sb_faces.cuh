// Per-face re-triangulation launch interface.
#pragma once
#include "sb_common.cuh"
#include "sb_internal.h"

namespace sbg {

struct FaceJob {
    int side, tri, pairBegin, pairEnd;
};

struct FaceArgs {
    MeshDev A, B;
    int nFaces;
    const int *faceSide, *faceTri, *faceBegin; // faceBegin has nFaces + 1 entries
    const int *pairIdx;                        // per face, its pairs (indices into segs) in processing order
    const double *segs;                        // [K*6]
    double factor;
    char *scratch;
    const unsigned long long *scratchOff;
    const int *ptOff, *triOff, *edgeOff;       // exclusive prefix sums of the capacities (nFaces + 1)
    d3 *cutPts;
    Key *cutKeys;
    int *faceTris;                             // local ids, 3 per triangle
    int *faceEdges;                            // directed cut edges (local ids, 2 per edge) in the face's
                                               // neighbour-map iteration order, both directions
    int *faceStatus, *faceNpts, *faceNtris, *faceNedges;
    int *ptSrc = nullptr; // optional, per face point: 2 x (intersecting pair) + segment end it came from
    int robustEdges = 0;  // SB_ROBUST_EDGE_TOLERANCE: scale-relative point-on-edge test (0: the reference's)
    unsigned long long scratchCap = ~0ull; // bytes of scratch; a face whose slice ends past it reports capacity
    const double *frames = nullptr;        // optional: per face its projection axis and perpendicular (6 doubles)
    int filteredEarcut = 1;                // ear-clipping orientations FP32-filtered (0: plain FP64)
};

size_t face_scratch_bytes_host(int np);
// An upper bound of the summed scratch of nFaces faces whose pair counts sum to sumNp, each of at most 65,536
// pairs: alpha nFaces + beta (sumNp - nFaces) with alpha the scratch of one pair and beta the largest increment
// per further pair (computed once).
size_t face_scratch_bound(long long nFaces, long long sumNp);
void launch_face_sizes(int nFaces, const int *faceBegin, unsigned long long *scratchBytes, int *ptCap, int *triCap,
                       int *edgeCap, cudaStream_t s);
void launch_faces(const FaceArgs &a, cudaStream_t s);
// per face the projection axis and perpendicular, one thread per face (FaceArgs::frames)
void launch_face_frames(int nFaces, const int *faceSide, const int *faceTri, const MeshDev &A, const MeshDev &B,
                        double *frames, cudaStream_t s);
// The cut faces' table, first pairs and buffer offsets (exclusive scans with the totals in entry FA + FB) in
// one launch of one block, for up to kFaceLayoutBlockMax faces; past that the caller scans device-wide.
constexpr int kFaceLayoutBlockMax = 1 << 16;
void launch_face_layout(int FA, int FB, const int *uniqA, const int *cntA, const int *uniqB, const int *cntB,
                        int *faceSide, int *faceTri, int *faceCnt, int *faceBegin, unsigned long long *scratchOff,
                        int *ptCap, int *ptOff, int *triCap, int *triOff, int *edgeCap, int *edgeOff, cudaStream_t s);

} // namespace sbg
