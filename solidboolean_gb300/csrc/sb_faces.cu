// Re-triangulation of every cut face (the reTriangulate lambda of src/solidboolean.cpp:352-407 together
// with ReTriangulator, src/retriangulator.cpp:29-337), one thread per cut face, all faces of both meshes in
// one launch.
//
// Per face, in the reference's order of operations:
//   1. weld the segment end points of the face's pairs by PositionKey (first value of a key wins), giving
//      local ids 3+k (src/solidboolean.cpp:296-311, 315-341);
//   2. rebuild the face's neighbour sets and reproduce the iteration order of the reference's
//      unordered_map<size_t, unordered_set<size_t>> (it decides where polylines and closed inner loops start
//      and which neighbour is followed first);
//   3. project to 2-D on (normalised edge 0, normal x edge 0) (src/vector3.h:227-238);
//   4. extract polylines and inner loops (retriangulator.cpp:48-95), attach polyline ends to triangle edges
//      with |cross| <= DBL_EPSILON (:97-105, src/vector2.h:212-215), order them along each edge by squared
//      distance, walk the boundary ring into polygons (:133-236), nest inner loops by point-in-polygon
//      (:107-131, src/vector2.h:199-210);
//   5. ear-clip every polygon with its holes and every inner loop with its children (:238-325).
// The per-face scratch is carved from one device buffer at an offset given by a prefix sum of each face's
// bound, so all faces run independently.
#include <vector>

#include "sb_common.cuh"
#include "sb_earcut.cuh"
#include "sb_faces.cuh"
#include "sb_ktime.h"

namespace sbg {

struct FacePtrs {
    int *su, *sv, *rawDeg, *rawOff, *cursor, *raw, *nbrCnt, *touch, *touched;
    int *hnext, *hbucket, *horder;
    uint64_t *hkeys;
    int *outer, *visited, *linePts, *lineOff, *lineKind, *polyIdx, *innerIdx;
    int *epPoint, *epLink, *epLine, *epRev, *epEdge;
    double *epD2;
    int *ringPoint, *ringLink, *ringLine, *ringRev, *ringLinkTo, *ringVisited, *startQ;
    int *polyPts, *polyOff;
    int *relParent, *relChild, *hasParent, *holesPoly, *holesInner, *kids;
    int *ringIds, *ringOffs;
    int *ecOut, *hq;
    int2 *ecStack;
    EcNode *ecNodes;
    d2 *pts2;
};

struct FaceDims {
    int np, m, P, R, L, nodeCap, outCap, stkCap, qCap, polyCap, relCap, hashCap, bucketCap;
};

__host__ __device__ inline FaceDims face_dims(int np)
{
    FaceDims d;
    d.np = np;
    d.m = 2 * np;
    d.P = d.m + 3;
    d.R = 3 + d.m;
    d.L = 3 * d.m + 6;
    d.nodeCap = 6 * d.L + 16;
    d.outCap = 3 * d.nodeCap;
    d.stkCap = 2 * d.L + 8;
    d.qCap = 8 * d.R + 16;
    d.polyCap = 4 * d.P + 16;
    d.relCap = d.m + 8;
    d.hashCap = d.m + 1;
    d.bucketCap = (int)hash_bucket_count((uint32_t)d.hashCap);
    return d;
}

// carve the per-face scratch; with base == nullptr only the size is computed
__host__ __device__ inline size_t face_carve(int np, char *base, FacePtrs *p)
{
    FaceDims d = face_dims(np);
    size_t off = 0;
    auto take = [&](size_t bytes) -> char * {
        char *r = base ? base + off : nullptr;
        off += (bytes + 15) & ~size_t(15);
        return r;
    };
#define SB_TAKE(field, T, n) p->field = reinterpret_cast<T *>(take(sizeof(T) * (size_t)(n)))
    FacePtrs dummy;
    if (!p)
        p = &dummy;
    SB_TAKE(su, int, np);
    SB_TAKE(sv, int, np);
    SB_TAKE(rawDeg, int, d.m);
    SB_TAKE(rawOff, int, d.m + 1);
    SB_TAKE(cursor, int, d.m);
    SB_TAKE(raw, int, 2 * np);
    SB_TAKE(nbrCnt, int, d.m);
    SB_TAKE(touch, int, d.m);
    SB_TAKE(touched, int, d.m);
    SB_TAKE(hnext, int, d.hashCap);
    SB_TAKE(hbucket, int, d.bucketCap);
    SB_TAKE(horder, int, d.hashCap);
    SB_TAKE(hkeys, uint64_t, d.hashCap);
    SB_TAKE(outer, int, d.m);
    SB_TAKE(visited, int, d.m);
    SB_TAKE(linePts, int, d.m);
    SB_TAKE(lineOff, int, d.m + 1);
    SB_TAKE(lineKind, int, d.m);
    SB_TAKE(polyIdx, int, d.m);
    SB_TAKE(innerIdx, int, d.m);
    SB_TAKE(epPoint, int, d.m);
    SB_TAKE(epLink, int, d.m);
    SB_TAKE(epLine, int, d.m);
    SB_TAKE(epRev, int, d.m);
    SB_TAKE(epEdge, int, d.m);
    SB_TAKE(epD2, double, d.m);
    SB_TAKE(ringPoint, int, d.R);
    SB_TAKE(ringLink, int, d.R);
    SB_TAKE(ringLine, int, d.R);
    SB_TAKE(ringRev, int, d.R);
    SB_TAKE(ringLinkTo, int, d.R);
    SB_TAKE(ringVisited, int, d.R);
    SB_TAKE(startQ, int, d.qCap);
    SB_TAKE(polyPts, int, d.polyCap);
    SB_TAKE(polyOff, int, d.R + 1);
    SB_TAKE(relParent, int, d.relCap);
    SB_TAKE(relChild, int, d.relCap);
    SB_TAKE(hasParent, int, d.m);
    SB_TAKE(holesPoly, int, d.relCap);
    SB_TAKE(holesInner, int, d.relCap);
    SB_TAKE(kids, int, d.R + 8);
    SB_TAKE(ringIds, int, d.L);
    SB_TAKE(ringOffs, int, d.m + 2);
    SB_TAKE(ecOut, int, d.outCap);
    SB_TAKE(hq, int, d.m + 2);
    SB_TAKE(ecStack, int2, d.stkCap);
    SB_TAKE(ecNodes, EcNode, d.nodeCap);
    SB_TAKE(pts2, d2, d.P);
#undef SB_TAKE
    return (off + 255) & ~size_t(255);
}

size_t face_scratch_bytes_host(int np) { return face_carve(np, nullptr, nullptr); }

size_t face_scratch_bound(long long nFaces, long long sumNp)
{
    static const size_t alpha = face_scratch_bytes_host(1);
    static const size_t beta = [] {
        size_t b = 0;
        for (int np = 2; np <= 65536; ++np) {
            const size_t x = face_scratch_bytes_host(np), d = x > alpha ? x - alpha : 0;
            b = std::max(b, (d + (size_t)np - 2) / (size_t)(np - 1));
        }
        return b;
    }();
    if (nFaces <= 0)
        return 0;
    return alpha * (size_t)nFaces + beta * (size_t)std::max(0ll, sumNp - nFaces);
}
__device__ size_t face_scratch_bytes_dev(int np) { return face_carve(np, nullptr, nullptr); }

// Orders the distinct keys keys[0..n) like the library does (hash_iteration_order), writing the keys
// themselves (as ints) to dst in iteration order.
SB_HDF void ordered_keys(const int *src, int n, FacePtrs &s, int *dst)
{
    for (int i = 0; i < n; ++i)
        s.hkeys[i] = (uint64_t)src[i];
    hash_iteration_order(s.hkeys, n, s.hnext, s.hbucket, s.horder);
    for (int i = 0; i < n; ++i)
        dst[i] = src[s.horder[i]];
}

// Point-on-edge test of the polyline ends. The reference's bound is absolute: |cross| <= eps
// (src/vector2.h:212-215, src/double.h:30-33). With robust set, the bound scales with the edge and the face's
// coordinates: 256 eps L (L + S), L the edge's larger 2D extent, S the face's largest absolute 3D coordinate
// (a cut point on the edge carries rounding of order eps S from its construction and projection, and the
// cross product multiplies it by the edge's length). 256 eps is a power of two, so the bound is formed by
// the same roundings on every machine.
SB_HD bool on_line(d2 p, d2 a, d2 b, bool robust, double S)
{
    const double cr = fabs(fabs((p.y - a.y) * (b.x - a.x) - (p.x - a.x) * (b.y - a.y)));
    if (!robust)
        return cr <= kDblEps;
    const double L = fmax(fabs(b.x - a.x), fabs(b.y - a.y));
    return cr <= (256.0 * kDblEps) * (L * (L + S));
}

// pnpoly over a ring of local ids (src/vector2.h:199-210)
SB_HDF bool in_polygon(d2 p, const d2 *pts, const int *poly, int n)
{
    bool inside = false;
    int i, j;
    for (i = 0, j = n - 1; i < n; j = i++) {
        d2 a = pts[poly[i]];
        d2 b = pts[poly[j]];
        if (((a.y > p.y) != (b.y > p.y)) && (p.x < (b.x - a.x) * (p.y - a.y) / (b.y - a.y) + a.x))
            inside = !inside;
    }
    return inside;
}

struct FaceOut {
    int status, npts, ntris, nedges;
};

// The projection frame of a face (ReTriangulator's constructor, src/retriangulator.cpp:29-37): the axis along
// its first edge and the in-plane perpendicular cross(normal, axis).
SB_HDF void face_frame(const d3 *c, d3 &axis, d3 &perp)
{
    const d3 normal = unit_normal(c[0], c[1], c[2]);
    axis = normalized(c[1] - c[0]);
    perp = cross(normal, axis);
}

// One thread per face, so that the divisions and square roots of the frames run with the warps' lanes
// converged (inside the re-triangulation two faces share a warp and the FP64 pipe issues whole warps).
__global__ void k_face_frames(int nFaces, const int *__restrict__ faceSide, const int *__restrict__ faceTri,
                              MeshDev A, MeshDev B, double *frames)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces)
        return;
    const MeshDev &M = faceSide[f] == 0 ? A : B;
    const int tri = faceTri[f];
    d3 c[3];
    for (int k = 0; k < 3; ++k) {
        const double *p = M.v + 3 * (size_t)M.t[3 * (size_t)tri + k];
        c[k] = mk(p[0], p[1], p[2]);
    }
    d3 axis, perp;
    face_frame(c, axis, perp);
    double *fr = frames + 6 * (size_t)f;
    fr[0] = axis.x;
    fr[1] = axis.y;
    fr[2] = axis.z;
    fr[3] = perp.x;
    fr[4] = perp.y;
    fr[5] = perp.z;
}

void launch_face_frames(int nFaces, const int *faceSide, const int *faceTri, const MeshDev &A, const MeshDev &B,
                        double *frames, cudaStream_t s)
{
    if (nFaces <= 0)
        return;
    SB_COUNT(k_face_frames)<<<(nFaces + 31) / 32, 32, 0, s>>>(nFaces, faceSide, faceTri, A, B, frames);
}

SB_HDF FaceOut process_face(const FaceJob &job, const FaceArgs &a, int f, char *scratchBase)
{
    FaceOut res{0, 0, 0, 0};
    const int np = job.pairEnd - job.pairBegin;
    FaceDims D = face_dims(np);
    FacePtrs s;
    face_carve(np, scratchBase, &s);
    const MeshDev &M = job.side == 0 ? a.A : a.B;
    d3 *outPts = a.cutPts + a.ptOff[f];
    Key *outKeys = a.cutKeys + a.ptOff[f];
    int *outTris = a.faceTris + 3 * (size_t)a.triOff[f];
    int *outEdges = a.faceEdges + 2 * (size_t)a.edgeOff[f];
    const int triCap = a.triOff[f + 1] - a.triOff[f];

    // ---- 1. local weld: first inserted value of a key wins --------------------------------------------
    int m = 0;
    for (int k = 0; k < np; ++k) {
        const int pair = a.pairIdx[job.pairBegin + k];
        const double *sg = a.segs + 6 * (size_t)pair;
        int ids[2];
        for (int e = 0; e < 2; ++e) {
            d3 p = mk(sg[3 * e], sg[3 * e + 1], sg[3 * e + 2]);
            Key key = make_key(p, a.factor);
            int id = -1;
            for (int q = 0; q < m; ++q)
                if (key_eq(outKeys[q], key)) {
                    id = q;
                    break;
                }
            if (id < 0) {
                id = m++;
                outPts[id] = p;
                outKeys[id] = key;
                if (a.ptSrc)
                    a.ptSrc[a.ptOff[f] + id] = 2 * pair + e;
            }
            ids[e] = 3 + id;
        }
        s.su[k] = ids[0];
        s.sv[k] = ids[1];
    }
    res.npts = m;

    // ---- 2. neighbour sets in the library's iteration order -------------------------------------------
    for (int i = 0; i < m; ++i) {
        s.rawDeg[i] = 0;
        s.touched[i] = 0;
    }
    int nt = 0;
    for (int k = 0; k < np; ++k) {
        int u = s.su[k], v = s.sv[k];
        if (u == v)
            continue;
        s.rawDeg[u - 3]++;
        s.rawDeg[v - 3]++;
        if (!s.touched[u - 3]) {
            s.touched[u - 3] = 1;
            s.touch[nt++] = u;
        }
        if (!s.touched[v - 3]) {
            s.touched[v - 3] = 1;
            s.touch[nt++] = v;
        }
    }
    s.rawOff[0] = 0;
    for (int i = 0; i < m; ++i) {
        s.rawOff[i + 1] = s.rawOff[i] + s.rawDeg[i];
        s.cursor[i] = s.rawOff[i];
    }
    for (int k = 0; k < np; ++k) {
        int u = s.su[k], v = s.sv[k];
        if (u == v)
            continue;
        s.raw[s.cursor[u - 3]++] = v;
        s.raw[s.cursor[v - 3]++] = u;
    }
    for (int i = 0; i < m; ++i) {
        // distinct neighbours in insertion order, then library order, in place
        int *lst = s.raw + s.rawOff[i];
        int n = 0;
        for (int q = 0; q < s.rawDeg[i]; ++q) {
            int x = lst[q];
            bool dup = false;
            for (int r = 0; r < n; ++r)
                dup |= (lst[r] == x);
            if (!dup)
                lst[n++] = x;
        }
        s.nbrCnt[i] = n;
        if (n > 1) {
            for (int q = 0; q < n; ++q)
                s.kids[q] = lst[q];
            ordered_keys(s.kids, n, s, lst);
        }
    }
    ordered_keys(s.touch, nt, s, s.outer);

    // ---- 3. projection --------------------------------------------------------------------------------
    d3 c[3];
    for (int k = 0; k < 3; ++k) {
        const double *p = M.v + 3 * (size_t)M.t[3 * (size_t)job.tri + k];
        c[k] = mk(p[0], p[1], p[2]);
    }
    double faceScale = 0.0; // largest absolute corner coordinate (the robust point-on-edge bound)
    for (int k = 0; k < 3; ++k)
        faceScale = fmax(faceScale, fmax(fabs(c[k].x), fmax(fabs(c[k].y), fabs(c[k].z))));
    d3 axis, perp;
    if (a.frames) { // computed beforehand by k_face_frames, with the same operations
        const double *fr = a.frames + 6 * (size_t)f;
        axis = mk(fr[0], fr[1], fr[2]);
        perp = mk(fr[3], fr[4], fr[5]);
    } else {
        face_frame(c, axis, perp);
    }
    for (int k = 0; k < 3; ++k) {
        d3 dir = c[k] - c[0];
        s.pts2[k] = d2{dot(dir, axis), dot(dir, perp)};
    }
    for (int i = 0; i < m; ++i) {
        d3 dir = outPts[i] - c[0];
        s.pts2[3 + i] = d2{dot(dir, axis), dot(dir, perp)};
    }

    // ---- 4a. polylines and inner loops ----------------------------------------------------------------
    int nEnds = 0;
    for (int q = 0; q < nt; ++q)
        if (s.nbrCnt[s.outer[q] - 3] == 1)
            s.kids[nEnds++] = s.outer[q];
    for (int q = 0; q < nt; ++q)
        if (s.nbrCnt[s.outer[q] - 3] > 1)
            s.kids[nEnds++] = s.outer[q];
    for (int i = 0; i < m; ++i)
        s.visited[i] = 0;
    int nLines = 0, nLinePts = 0, nPoly = 0, nInner = 0;
    s.lineOff[0] = 0;
    for (int q = 0; q < nEnds; ++q) {
        int start = s.kids[q];
        if (s.visited[start - 3])
            continue;
        int begin = nLinePts;
        int cur = start;
        for (int guard = 0; guard <= m; ++guard) {
            s.visited[cur - 3] = 1;
            s.linePts[nLinePts++] = cur;
            const int *nb = s.raw + s.rawOff[cur - 3];
            int nxt = -1;
            for (int r = 0; r < s.nbrCnt[cur - 3]; ++r)
                if (!s.visited[nb[r] - 3]) {
                    nxt = nb[r];
                    break;
                }
            if (nxt < 0)
                break;
            cur = nxt;
        }
        int len = nLinePts - begin;
        int kind = -1;
        if (len >= 3) {
            int last = s.linePts[nLinePts - 1];
            const int *nb = s.raw + s.rawOff[last - 3];
            for (int r = 0; r < s.nbrCnt[last - 3]; ++r)
                if (nb[r] == start)
                    kind = 1;
        }
        if (kind != 1 && len >= 2)
            kind = 0;
        if (kind < 0) {
            nLinePts = begin;
            continue;
        }
        s.lineKind[nLines] = kind;
        if (kind == 1)
            s.innerIdx[nInner++] = nLines;
        else
            s.polyIdx[nPoly++] = nLines;
        s.lineOff[++nLines] = nLinePts;
    }

    // ---- 4b. attach polyline ends, order along edges, build the ring ---------------------------------
    int nEp = 0;
    for (int li = 0; li < nPoly; ++li) {
        int L0 = s.lineOff[s.polyIdx[li]], L1 = s.lineOff[s.polyIdx[li] + 1];
        int front = s.linePts[L0], back = s.linePts[L1 - 1];
        int fe = -1, be = -1;
        for (int e = 0; e < 3 && fe < 0; ++e)
            if (on_line(s.pts2[front], s.pts2[e], s.pts2[(e + 1) % 3], a.robustEdges != 0, faceScale))
                fe = e;
        for (int e = 0; e < 3 && be < 0; ++e)
            if (on_line(s.pts2[back], s.pts2[e], s.pts2[(e + 1) % 3], a.robustEdges != 0, faceScale))
                be = e;
        if (fe < 0 || be < 0) {
            res.status = 1;
            return res;
        }
        d2 df{s.pts2[front].x - s.pts2[fe].x, s.pts2[front].y - s.pts2[fe].y};
        d2 db{s.pts2[back].x - s.pts2[be].x, s.pts2[back].y - s.pts2[be].y};
        s.epPoint[nEp] = front;
        s.epLink[nEp] = back;
        s.epLine[nEp] = li;
        s.epRev[nEp] = 0;
        s.epD2[nEp] = df.x * df.x + df.y * df.y;
        s.epEdge[nEp] = fe;
        ++nEp;
        s.epPoint[nEp] = back;
        s.epLink[nEp] = front;
        s.epLine[nEp] = li;
        s.epRev[nEp] = 1;
        s.epD2[nEp] = db.x * db.x + db.y * db.y;
        s.epEdge[nEp] = be;
        ++nEp;
    }
    int R = 0;
    for (int e = 0; e < 3; ++e) {
        s.ringPoint[R] = e;
        s.ringLink[R] = 0;
        s.ringLine[R] = -1;
        s.ringRev[R] = 0;
        s.ringLinkTo[R] = -1;
        ++R;
        int first = R;
        for (int q = 0; q < nEp; ++q) {
            if (s.epEdge[q] != e)
                continue;
            // stable insertion by squared distance (the library sort for up to 16 entries)
            int pos = R;
            while (pos > first && s.epD2[s.kids[pos - 1]] > s.epD2[q]) {
                s.kids[pos] = s.kids[pos - 1];
                --pos;
            }
            s.kids[pos] = q;
            ++R;
        }
        for (int r = first; r < R; ++r) {
            int q = s.kids[r];
            s.ringPoint[r] = s.epPoint[q];
            s.ringLink[r] = s.epLink[q];
            s.ringLine[r] = s.epLine[q];
            s.ringRev[r] = s.epRev[q];
            s.ringLinkTo[r] = -1;
        }
    }
    for (int r = 0; r < R; ++r) {
        if (s.ringLine[r] == -1)
            continue;
        for (int q = 0; q < R; ++q)
            if (s.ringLine[q] != -1 && s.ringPoint[q] == s.ringLink[r]) {
                s.ringLinkTo[r] = q;
                break;
            }
    }

    // ---- 4c. walk the ring into polygons ---------------------------------------------------------------
    for (int r = 0; r < R; ++r)
        s.ringVisited[r] = 0;
    int qh = 0, qt = 0, nPolys = 0, nPolyPts = 0;
    s.startQ[qt++] = 0;
    s.polyOff[0] = 0;
    int steps = 0;
    const int stepCap = 4 * D.polyCap + 64;
    while (qh < qt) {
        int st = s.startQ[qh++];
        if (s.ringVisited[st])
            continue;
        int k = st;
        do {
            if (++steps > stepCap || nPolys >= D.R) {
                res.status = 3;
                return res;
            }
            s.ringVisited[k] = 1;
            if (s.ringLine[k] == -1) {
                if (nPolyPts >= D.polyCap) {
                    res.status = 3;
                    return res;
                }
                s.polyPts[nPolyPts++] = s.ringPoint[k];
                k = (k + 1) % R;
            } else if (s.ringLinkTo[k] != -1) {
                int line = s.polyIdx[s.ringLine[k]];
                int L0 = s.lineOff[line], L1 = s.lineOff[line + 1];
                if (nPolyPts + (L1 - L0) > D.polyCap || qt >= D.qCap) {
                    res.status = 3;
                    return res;
                }
                if (s.ringRev[k])
                    for (int i = L1 - 1; i >= L0; --i)
                        s.polyPts[nPolyPts++] = s.linePts[i];
                else
                    for (int i = L0; i < L1; ++i)
                        s.polyPts[nPolyPts++] = s.linePts[i];
                s.startQ[qt++] = (k + 1) % R;
                k = (s.ringLinkTo[k] + 1) % R;
            } else {
                res.status = 2;
                return res;
            }
        } while (k != st);
        s.polyOff[++nPolys] = nPolyPts;
    }

    // ---- 4d. inner-loop hierarchy ----------------------------------------------------------------------
    int nRel = 0;
    for (int i = 0; i < nInner; ++i)
        s.hasParent[i] = 0;
    for (int i = 0; i < nInner; ++i)
        for (int j = i + 1; j < nInner; ++j) {
            const int *Ii = s.linePts + s.lineOff[s.innerIdx[i]];
            const int *Ij = s.linePts + s.lineOff[s.innerIdx[j]];
            int ni = s.lineOff[s.innerIdx[i] + 1] - s.lineOff[s.innerIdx[i]];
            int nj = s.lineOff[s.innerIdx[j] + 1] - s.lineOff[s.innerIdx[j]];
            int par = -1, chi = -1;
            if (in_polygon(s.pts2[Ii[0]], s.pts2, Ij, nj)) {
                par = j;
                chi = i;
            } else if (in_polygon(s.pts2[Ij[0]], s.pts2, Ii, ni)) {
                par = i;
                chi = j;
            }
            if (par >= 0) {
                if (nRel >= D.relCap) {
                    res.status = 3;
                    return res;
                }
                s.relParent[nRel] = par;
                s.relChild[nRel] = chi;
                ++nRel;
                s.hasParent[chi] = 1;
            }
        }
    int nHoles = 0;
    for (int i = 0; i < nInner; ++i) {
        if (s.hasParent[i])
            continue;
        const int *Ii = s.linePts + s.lineOff[s.innerIdx[i]];
        for (int j = 0; j < nPolys; ++j)
            if (in_polygon(s.pts2[Ii[0]], s.pts2, s.polyPts + s.polyOff[j], s.polyOff[j + 1] - s.polyOff[j])) {
                if (nHoles >= D.relCap) {
                    res.status = 3;
                    return res;
                }
                s.holesPoly[nHoles] = j;
                s.holesInner[nHoles] = i;
                ++nHoles;
            }
    }

    // ---- 5. ear clipping -------------------------------------------------------------------------------
    DevEarcut ec;
    ec.filtered = a.filteredEarcut != 0;
    ec.N = s.ecNodes;
    ec.cap = D.nodeCap;
    ec.out = s.ecOut;
    ec.outCap = D.outCap;
    ec.stk = s.ecStack;
    ec.stkCap = D.stkCap;
    ec.hq = s.hq;
    int nTris = 0;
    auto triangulate_rings = [&](int nr) -> bool {
        ec.error = 0;
        long long L = s.ringOffs[nr];
        ec.budget = 64 * L * L + 100000;
        ec.run(s.pts2, s.ringIds, s.ringOffs, nr);
        if (ec.error)
            return false;
        int nOut = ec.outCnt / 3;
        if (nTris + nOut > triCap)
            return false;
        for (int k = 0; k < 3 * nOut; ++k)
            outTris[3 * nTris + k] = s.ringIds[ec.out[k]];
        nTris += nOut;
        return true;
    };
    auto add_ring = [&](int &nr, const int *ids, int n) -> bool {
        int base = s.ringOffs[nr];
        if (base + n > D.L || nr + 1 > D.m + 1)
            return false;
        for (int k = 0; k < n; ++k)
            s.ringIds[base + k] = ids[k];
        s.ringOffs[++nr] = base + n;
        return true;
    };
    for (int pi = 0; pi < nPolys; ++pi) {
        int nr = 0;
        s.ringOffs[0] = 0;
        bool ok = add_ring(nr, s.polyPts + s.polyOff[pi], s.polyOff[pi + 1] - s.polyOff[pi]);
        for (int h = 0; h < nHoles && ok; ++h)
            if (s.holesPoly[h] == pi) {
                int li = s.innerIdx[s.holesInner[h]];
                ok = add_ring(nr, s.linePts + s.lineOff[li], s.lineOff[li + 1] - s.lineOff[li]);
            }
        if (!ok || !triangulate_rings(nr)) {
            res.status = 3;
            return res;
        }
    }
    for (int qi = 0; qi < nInner; ++qi) {
        int nr = 0;
        s.ringOffs[0] = 0;
        int li = s.innerIdx[qi];
        bool ok = add_ring(nr, s.linePts + s.lineOff[li], s.lineOff[li + 1] - s.lineOff[li]);
        // children of qi in the library's set order, minus grandchildren (retriangulator.cpp:271-291)
        int nk = 0;
        for (int r = 0; r < nRel; ++r)
            if (s.relParent[r] == qi)
                s.kids[nk++] = s.relChild[r];
        if (nk > 1) {
            for (int q = 0; q < nk; ++q)
                s.touch[q] = s.kids[q];
            ordered_keys(s.touch, nk, s, s.kids);
        }
        for (int q = 0; q < nk && ok; ++q) {
            int child = s.kids[q];
            bool grand = false;
            for (int r = 0; r < nRel && !grand; ++r) {
                if (s.relChild[r] != child)
                    continue;
                int mid = s.relParent[r];
                for (int r2 = 0; r2 < nRel; ++r2)
                    if (s.relParent[r2] == qi && s.relChild[r2] == mid)
                        grand = true;
            }
            if (grand)
                continue;
            int lc = s.innerIdx[child];
            ok = add_ring(nr, s.linePts + s.lineOff[lc], s.lineOff[lc + 1] - s.lineOff[lc]);
        }
        if (!ok || !triangulate_rings(nr)) {
            res.status = 3;
            return res;
        }
    }
    res.ntris = nTris;

    // ---- cut edges: the neighbour map walked as the reference's reTriangulate lambda walks it
    // (src/solidboolean.cpp:397-404): keys in the library's iteration order, each key's set in its order, as
    // directed (from, to) pairs of local ids; every undirected edge appears once from each end. The global
    // cut-loop map is built from this sequence, so its order decides where each loop starts.
    int ne = 0;
    for (int q = 0; q < nt; ++q) {
        const int from = s.outer[q];
        const int *nb = s.raw + s.rawOff[from - 3];
        for (int r = 0; r < s.nbrCnt[from - 3]; ++r)
            if (ne < 2 * np) {
                outEdges[2 * ne] = from;
                outEdges[2 * ne + 1] = nb[r];
                ++ne;
            }
    }
    res.nedges = ne;
    return res;
}

// Faces per warp. A face is a long serial chain of FP64 operations and FP64 issue is the limit (a warp
// instruction occupies the FP64 pipe however few of its lanes are active), so lanes should share
// instructions; but faces differ in control flow, and beyond two per warp their divergent paths cost more
// than the shared issue saves (measured: 1, 2, 4, 8 faces per warp).
constexpr int kFacesPerWarp = 2;

__global__ void __launch_bounds__(32) k_faces(FaceArgs a)
{
    const int f = blockIdx.x * kFacesPerWarp + threadIdx.x;
    if (threadIdx.x >= kFacesPerWarp || f >= a.nFaces)
        return;
    FaceJob job;
    job.side = a.faceSide[f];
    job.tri = a.faceTri[f];
    job.pairBegin = a.faceBegin[f];
    job.pairEnd = a.faceBegin[f + 1];
    if (a.scratchOff[f + 1] > a.scratchCap) { // past the allocation's bound (never expected): capacity
        a.faceStatus[f] = 3;
        a.faceNpts[f] = a.faceNtris[f] = a.faceNedges[f] = 0;
        return;
    }
    FaceOut r = process_face(job, a, f, a.scratch + a.scratchOff[f]);
    a.faceStatus[f] = r.status;
    a.faceNpts[f] = r.npts;
    a.faceNtris[f] = r.status == 0 ? r.ntris : 0;
    a.faceNedges[f] = r.status == 0 ? r.nedges : 0;
}

// Exclusive scan of n + 1 values in place by one block (a[n] receives the total); every thread must call it.
template <class T> __device__ T block_scan_inplace(T *a, int n)
{
    __shared__ T part[32];
    __shared__ T carry;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, W = blockDim.x >> 5;
    if (tid == 0)
        carry = 0;
    __syncthreads();
    for (int base = 0; base <= n; base += blockDim.x) {
        const int i = base + tid;
        const T x = i < n ? a[i] : T(0);
        T y = x;
        for (int o = 1; o < 32; o <<= 1) {
            const T v = __shfl_up_sync(0xFFFFFFFFu, y, o);
            if (lane >= o)
                y += v;
        }
        if (lane == 31)
            part[w] = y;
        __syncthreads();
        if (w == 0) {
            T z = lane < W ? part[lane] : T(0);
            for (int o = 1; o < 32; o <<= 1) {
                const T v = __shfl_up_sync(0xFFFFFFFFu, z, o);
                if (lane >= o)
                    z += v;
            }
            part[lane] = z; // inclusive over warps
        }
        __syncthreads();
        const T before = carry + (w > 0 ? part[w - 1] : T(0)) + (y - x);
        if (i <= n)
            a[i] = before;
        __syncthreads();
        if (tid == 0)
            carry += part[W - 1];
        __syncthreads();
    }
    return carry;
}

// The cut faces' table and buffer layout in one launch (one block; for up to kFaceLayoutBlockMax faces): side,
// triangle and pair count of each face, its first pair (exclusive scan of the counts) and the exclusive scans
// of its scratch bytes and point, triangle and edge capacities, each with its total in entry nFaces.
__global__ void __launch_bounds__(1024) k_face_layout(int FA, int FB, const int *__restrict__ uniqA,
                                                      const int *__restrict__ cntA, const int *__restrict__ uniqB,
                                                      const int *__restrict__ cntB, int *faceSide, int *faceTri,
                                                      int *faceCnt, int *faceBegin, unsigned long long *scratchOff,
                                                      int *ptCap, int *ptOff, int *triCap, int *triOff,
                                                      int *edgeCap, int *edgeOff)
{
    const int n = FA + FB;
    for (int f = threadIdx.x; f < n; f += blockDim.x) {
        const bool a = f < FA;
        const int np = a ? cntA[f] : cntB[f - FA];
        faceSide[f] = a ? 0 : 1;
        faceTri[f] = a ? uniqA[f] : uniqB[f - FA];
        faceCnt[f] = np;
        faceBegin[f] = np;
        scratchOff[f] = (unsigned long long)face_scratch_bytes_dev(np);
        ptCap[f] = ptOff[f] = 2 * np;
        triCap[f] = triOff[f] = 32 * np + 16;
        edgeCap[f] = edgeOff[f] = 2 * np; // directed: each undirected edge from both ends
    }
    __syncthreads();
    block_scan_inplace(faceBegin, n);
    block_scan_inplace(scratchOff, n);
    block_scan_inplace(ptOff, n);
    block_scan_inplace(triOff, n);
    block_scan_inplace(edgeOff, n);
}

void launch_face_layout(int FA, int FB, const int *uniqA, const int *cntA, const int *uniqB, const int *cntB,
                        int *faceSide, int *faceTri, int *faceCnt, int *faceBegin, unsigned long long *scratchOff,
                        int *ptCap, int *ptOff, int *triCap, int *triOff, int *edgeCap, int *edgeOff, cudaStream_t s)
{
    if (FA + FB <= 0)
        return;
    SB_COUNT(k_face_layout)<<<1, 1024, 0, s>>>(FA, FB, uniqA, cntA, uniqB, cntB, faceSide, faceTri, faceCnt, faceBegin,
                                               scratchOff, ptCap, ptOff, triCap, triOff, edgeCap, edgeOff);
}

// per-face capacities: scratch bytes, points, triangles, edges (written as counts; scanned by the caller)
__global__ void k_face_sizes(int nFaces, const int *__restrict__ faceBegin, unsigned long long *scratchBytes,
                             int *ptCap, int *triCap, int *edgeCap)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces)
        return;
    int np = faceBegin[f + 1] - faceBegin[f];
    scratchBytes[f] = (unsigned long long)face_scratch_bytes_dev(np);
    ptCap[f] = 2 * np;
    triCap[f] = 32 * np + 16;
    edgeCap[f] = 2 * np; // directed: each undirected edge from both ends
}

void launch_face_sizes(int nFaces, const int *faceBegin, unsigned long long *scratchBytes, int *ptCap, int *triCap,
                       int *edgeCap, cudaStream_t s)
{
    if (nFaces <= 0)
        return;
    SB_COUNT(k_face_sizes)<<<(nFaces + 255) / 256, 256, 0, s>>>(nFaces, faceBegin, scratchBytes, ptCap, triCap, edgeCap);
}


void launch_faces(const FaceArgs &a, cudaStream_t s)
{
    if (a.nFaces <= 0)
        return;
    KTime kt("k_faces", s);
    SB_COUNT(k_faces)<<<(a.nFaces + kFacesPerWarp - 1) / kFacesPerWarp, 32, 0, s>>>(a);
}

// ---------------------------------------------------------------------------------------------------
// The device ear-clipper on its own (sb_debug_earcut): one polygon with holes, one thread, with the same
// scratch sizing rule as a cut face (nodes 6 L + 16, output 3 x nodes, stack 2 L + 8 for L ring points).
// ---------------------------------------------------------------------------------------------------
__global__ void k_earcut_one(const double *__restrict__ xy, const int *__restrict__ off, int nrings, int L,
                             EcNode *nodes, int nodeCap, int *out, int outCap, int2 *stk, int stkCap, int *hq,
                             int *ids, d2 *pts, int *result)
{
    if (blockIdx.x != 0 || threadIdx.x != 0)
        return;
    for (int i = 0; i < L; ++i) {
        pts[i] = d2{xy[2 * i], xy[2 * i + 1]};
        ids[i] = i;
    }
    DevEarcut ec;
    ec.N = nodes;
    ec.cap = nodeCap;
    ec.out = out;
    ec.outCap = outCap;
    ec.stk = stk;
    ec.stkCap = stkCap;
    ec.hq = hq;
    ec.error = 0;
    ec.budget = 64ll * L * L + 100000;
    ec.run(pts, ids, off, nrings);
    result[0] = ec.outCnt;
    result[1] = ec.error;
}

} // namespace sbg

using namespace sbg;

extern "C" sb_status sb_debug_earcut(const double *xy, const int64_t *ring_off, size_t n_rings, int64_t *indices,
                                     size_t cap, size_t *count)
{
    if (!xy || !ring_off || !count || n_rings == 0 || n_rings > (1u << 20))
        return SB_ERR_INVALID;
    const int64_t L64 = ring_off[n_rings];
    if (ring_off[0] != 0 || L64 <= 0 || L64 > (1 << 20))
        return SB_ERR_INVALID;
    for (size_t r = 0; r < n_rings; ++r)
        if (ring_off[r + 1] < ring_off[r])
            return SB_ERR_INVALID;
    const int L = (int)L64;
    const int nodeCap = 6 * L + 16, outCap = 3 * nodeCap, stkCap = 2 * L + 8;
    std::vector<int> off(n_rings + 1);
    for (size_t r = 0; r <= n_rings; ++r)
        off[r] = (int)ring_off[r];
    DevBuf buf;
    Carve c;
    const size_t o_xy = c.take<double>(2 * (size_t)L), o_off = c.take<int>(n_rings + 1);
    const size_t o_nodes = c.take<EcNode>(nodeCap), o_out = c.take<int>(outCap), o_stk = c.take<int2>(stkCap);
    const size_t o_hq = c.take<int>(n_rings + 1), o_ids = c.take<int>(L), o_pts = c.take<d2>(L);
    const size_t o_res = c.take<int>(2);
    SB_CUDA_CHECK(buf.ensure(c.off));
    char *b = buf.as<char>();
    sb_status st = SB_OK;
    int res[2] = {0, 0};
    std::vector<int> out;
    cudaError_t e = cudaMemcpy(b + o_xy, xy, sizeof(double) * 2 * (size_t)L, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b + o_off, off.data(), sizeof(int) * (n_rings + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        count_launch();
        k_earcut_one<<<1, 32>>>((const double *)(b + o_xy), (const int *)(b + o_off), (int)n_rings, L,
                                (EcNode *)(b + o_nodes), nodeCap, (int *)(b + o_out), outCap, (int2 *)(b + o_stk),
                                stkCap, (int *)(b + o_hq), (int *)(b + o_ids), (d2 *)(b + o_pts),
                                (int *)(b + o_res));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(res, b + o_res, sizeof res, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && res[1] == 0 && res[0] > 0) {
        out.resize((size_t)res[0]);
        e = cudaMemcpy(out.data(), b + o_out, sizeof(int) * out.size(), cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) {
        st = cuda_fail(e, "sb_debug_earcut", __FILE__, __LINE__);
    } else if (res[1] != 0) {
        set_last_error(res[1] == 1 ? "earcut: node capacity exceeded" : "earcut: iteration budget exceeded");
        st = SB_ERR_CAPACITY;
    } else {
        *count = out.size();
        if (indices) {
            if (cap < out.size()) {
                st = SB_ERR_INVALID;
            } else {
                for (size_t k = 0; k < out.size(); ++k)
                    indices[k] = out[k];
            }
        }
    }
    buf.release();
    return st;
}
