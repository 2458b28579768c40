/*
 * CPU ORACLE (test infrastructure only): a restatement, in our own code, of the reference's mesh-boolean
 * path, used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the checker. The product
 * never links, imports or calls this file.
 *
 * It follows huxingyi/solidboolean step by step:
 *   prepare           src/solidmesh.cpp:42-76 (normals, per-triangle boxes and centres, tree)
 *   tree build        src/axisalignedboundingboxtree.cpp:27-45, 71-141 (mean-centre split on the longest
 *                     float span, leaf size 20, halving when one side is empty)
 *   tree traversal    src/axisalignedboundingboxtree.h:54-95
 *   tri-tri           thirdparty/GuigueDevillers03/tri_tri_intersect.c:285-472 (orientation signs,
 *                     canonical permutations, segment construction; coplanar pairs are rejected by the
 *                     caller, src/solidboolean.cpp:103-122)
 *   per-face contexts src/solidboolean.cpp:296-341 (PositionKey weld, local ids 3+k, neighbour sets)
 *   PositionKey       src/positionkey.cpp:25-61 ((long)(c * factor) truncation, lexicographic order)
 *   addUnintersected  src/solidboolean.cpp:250-286
 *   reTriangulate     src/solidboolean.cpp:352-407 and src/retriangulator.cpp:29-337
 *   earcut            sb_oracle_earcut.hpp
 *   loops             src/solidboolean.cpp:124-165
 *   face groups       src/solidboolean.cpp:167-239
 *   sides             src/solidboolean.cpp:48-92, 482-510
 *   fetch             src/solidboolean.cpp:512-570
 *
 * The reference's output depends on the iteration order of libstdc++'s unordered containers (which cut
 * point starts a closed loop, which loop vertex seeds a group, ...). That order is part of its observable
 * behaviour, so this restatement keeps the same standard containers and the same insertion sequences.
 * Every floating-point expression keeps the reference's operation order; the file is compiled with
 * -ffp-contract=off so no multiply-add is fused.
 */
#include "sb_oracle.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <queue>
#include <set>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "sb_oracle_dump.hpp"
#include "sb_oracle_earcut.hpp"

namespace port {

static const double kEps = std::numeric_limits<double>::epsilon();
static long g_factor = 100000;
// sb_robust flags of the run (include/solidboolean_gb300.h): bit 0 = scale-relative point-on-edge test.
// Not part of the reference: the robust mode's own checker. 0 = the reference's behaviour.
static int g_robust = 0;

struct V3 {
    double x = 0, y = 0, z = 0;
    V3() {}
    V3(double a, double b, double c) : x(a), y(b), z(c) {}
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline V3 operator+(const V3 &a, const V3 &b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(const V3 &a, const V3 &b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator-(const V3 &a) { return V3(-a.x, -a.y, -a.z); }
static inline V3 operator/(const V3 &a, double d) { return V3(a.x / d, a.y / d, a.z / d); }
static inline V3 operator*(double s, const V3 &a) { return V3(s * a.x, s * a.y, s * a.z); }
static inline double dot3(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross3(const V3 &a, const V3 &b)
{
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// unit normal of (a, b, c), zero when the cross product is within DBL_EPSILON of zero (vector3.h:155-176)
static inline V3 unitNormal(const V3 &a, const V3 &b, const V3 &c)
{
    double bax = b.x - a.x, bay = b.y - a.y, baz = b.z - a.z;
    double cax = c.x - a.x, cay = c.y - a.y, caz = c.z - a.z;
    double nx = bay * caz - baz * cay;
    double ny = baz * cax - bax * caz;
    double nz = bax * cay - bay * cax;
    double len = std::sqrt(nx * nx + ny * ny + nz * nz);
    if (std::abs(len) <= kEps)
        return V3();
    return V3(nx / len, ny / len, nz / len);
}
static inline V3 normalized(const V3 &v)
{
    double len = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    if (std::abs(len) <= kEps)
        return V3();
    return V3(v.x / len, v.y / len, v.z / len);
}

struct V2 {
    double x = 0, y = 0;
};

// quantised weld key (positionkey.cpp:32-54)
struct Key {
    long x, y, z;
    explicit Key(const V3 &v)
        : x((long)(v.x * (double)g_factor)), y((long)(v.y * (double)g_factor)), z((long)(v.z * (double)g_factor))
    {
    }
    bool operator<(const Key &o) const
    {
        if (x != o.x)
            return x < o.x;
        if (y != o.y)
            return y < o.y;
        return z < o.z;
    }
};

struct Box {
    V3 lo{std::numeric_limits<double>::max(), std::numeric_limits<double>::max(),
          std::numeric_limits<double>::max()};
    V3 hi{std::numeric_limits<double>::lowest(), std::numeric_limits<double>::lowest(),
          std::numeric_limits<double>::lowest()};
    V3 sum;
    size_t num = 0;
    V3 center;
    void add(const V3 &v)
    {
        if (v.x > hi.x) hi.x = v.x;
        if (v.x < lo.x) lo.x = v.x;
        sum.x += v.x;
        if (v.y > hi.y) hi.y = v.y;
        if (v.y < lo.y) lo.y = v.y;
        sum.y += v.y;
        if (v.z > hi.z) hi.z = v.z;
        if (v.z < lo.z) lo.z = v.z;
        sum.z += v.z;
        ++num;
    }
    void finish()
    {
        if (!num)
            return;
        double c = (double)(float)num;
        sum = V3(sum.x / c, sum.y / c, sum.z / c);
        center = sum;
    }
    bool overlaps(const Box &o) const
    {
        return lo.x <= o.hi.x && hi.x >= o.lo.x && lo.y <= o.hi.y && hi.y >= o.lo.y && lo.z <= o.hi.z &&
               hi.z >= o.lo.z;
    }
};

// Top-down tree with the reference's split rule.
struct Tree {
    struct Node {
        Box box;
        V3 center;
        std::vector<size_t> idx;
        int left = -1, right = -1;
    };
    const std::vector<Box> *boxes = nullptr;
    std::vector<Node> nodes;
    std::vector<size_t> scratch;

    void build(const std::vector<Box> *bx, const Box &outer)
    {
        boxes = bx;
        nodes.clear();
        nodes.emplace_back();
        nodes[0].box = outer;
        for (size_t i = 0; i < bx->size(); ++i)
            nodes[0].idx.push_back(i);
        if (!bx->empty()) {
            V3 c;
            for (size_t i : nodes[0].idx) {
                const V3 &bc = (*bx)[i].center;
                c = V3(c.x + bc.x, c.y + bc.y, c.z + bc.z);
            }
            double n = (double)(float)nodes[0].idx.size();
            nodes[0].center = V3(c.x / n, c.y / n, c.z / n);
        }
        split(0);
    }

    void split(int ni)
    {
        const size_t n = nodes[ni].idx.size();
        if (n <= 20)
            return;
        const V3 lo = nodes[ni].box.lo, hi = nodes[ni].box.hi;
        float span[3] = {(float)(hi.x - lo.x), (float)(hi.y - lo.y), (float)(hi.z - lo.z)};
        int axis = 0;
        for (int k = 1; k < 3; ++k)
            if (span[axis] < span[k])
                axis = k;
        const double splitAt = nodes[ni].center[axis];
        scratch.assign(n + n + 2, 0);
        size_t leftOff = n, rightOff = n - 1, leftCount = 0, rightCount = 0;
        for (size_t i = 0; i < n; ++i) {
            size_t bi = nodes[ni].idx[i];
            if ((*boxes)[bi].center[axis] < splitAt) {
                scratch[--leftOff] = bi;
                ++leftCount;
            } else {
                scratch[++rightOff] = bi;
                ++rightCount;
            }
        }
        if (leftCount == 0) {
            leftCount = rightCount / 2;
            rightCount -= leftCount;
            leftOff = rightOff - n + 1;
        } else if (rightCount == 0) {
            rightCount = leftCount / 2;
            leftCount -= rightCount;
            rightOff = leftOff + n - 1;
        }
        size_t mid = leftOff + leftCount - 1;
        int L = (int)nodes.size();
        nodes.emplace_back();
        int R = (int)nodes.size();
        nodes.emplace_back();
        nodes[ni].left = L;
        nodes[ni].right = R;
        auto fill = [&](int child, size_t from, size_t to) {
            V3 c;
            for (size_t i = from; i <= to; ++i) {
                size_t bi = scratch[i];
                const Box &b = (*boxes)[bi];
                nodes[child].box.add(b.lo);
                nodes[child].box.add(b.hi);
                nodes[child].idx.push_back(bi);
                c = V3(c.x + b.center.x, c.y + b.center.y, c.z + b.center.z);
            }
            double cnt = (double)(float)nodes[child].idx.size();
            nodes[child].center = V3(c.x / cnt, c.y / cnt, c.z / cnt);
        };
        fill(L, leftOff, mid);
        fill(R, mid + 1, rightOff);
        split(L);
        split(R);
    }

    bool leaf(int n) const { return nodes[n].left < 0 && nodes[n].right < 0; }

    // dual traversal emitting (this tree's box, other tree's box) pairs in the reference's DFS order
    void test(int a, const Tree &o, int b, std::vector<std::pair<size_t, size_t>> &out) const
    {
        const Node &A = nodes[a];
        const Node &B = o.nodes[b];
        if (!A.box.overlaps(B.box))
            return;
        if (leaf(a)) {
            if (o.leaf(b)) {
                for (size_t x : A.idx)
                    for (size_t y : B.idx)
                        if ((*boxes)[x].overlaps((*o.boxes)[y]))
                            out.emplace_back(x, y);
            } else {
                test(a, o, B.left, out);
                test(a, o, B.right, out);
            }
        } else if (o.leaf(b) || !(A.idx.size() < B.idx.size())) {
            test(A.left, o, b, out);
            test(A.right, o, b, out);
        } else {
            test(a, o, B.left, out);
            test(a, o, B.right, out);
        }
    }

    void boxQuery(int a, const Box &q, std::vector<size_t> &out) const
    {
        const Node &A = nodes[a];
        if (!A.box.overlaps(q))
            return;
        if (leaf(a)) {
            for (size_t x : A.idx)
                if ((*boxes)[x].overlaps(q))
                    out.push_back(x);
            return;
        }
        boxQuery(A.left, q, out);
        boxQuery(A.right, q, out);
    }

    void leafOrder(int a, std::vector<int64_t> &out) const
    {
        if (leaf(a)) {
            for (size_t x : nodes[a].idx)
                out.push_back((int64_t)x);
            return;
        }
        leafOrder(nodes[a].left, out);
        leafOrder(nodes[a].right, out);
    }
};

struct Mesh {
    std::vector<V3> v;
    std::vector<std::array<size_t, 3>> t;
    std::vector<V3> normals;
    std::vector<Box> boxes;
    Tree tree;
    void prepare()
    {
        normals.clear();
        normals.reserve(t.size());
        for (const auto &f : t)
            normals.push_back(unitNormal(v[f[0]], v[f[1]], v[f[2]]));
        boxes.assign(t.size(), Box());
        for (size_t i = 0; i < t.size(); ++i) {
            for (int k = 0; k < 3; ++k)
                boxes[i].add(v[t[i][k]]);
            boxes[i].finish();
        }
        Box outer;
        for (size_t i = 0; i < t.size(); ++i)
            for (int k = 0; k < 3; ++k)
                outer.add(v[t[i][k]]);
        outer.finish();
        tree.build(&boxes, outer);
    }
};

// ---------------------------------------------------------------------------------------------------
// Guigue-Devillers triangle-triangle intersection with segment construction.
// Returns 1 when a non-coplanar intersection segment was produced.
// ---------------------------------------------------------------------------------------------------
namespace gd {
typedef double P[3];
static inline void sub(double *d, const double *a, const double *b)
{
    d[0] = a[0] - b[0];
    d[1] = a[1] - b[1];
    d[2] = a[2] - b[2];
}
static inline void crs(double *d, const double *a, const double *b)
{
    d[0] = a[1] * b[2] - a[2] * b[1];
    d[1] = a[2] * b[0] - a[0] * b[2];
    d[2] = a[0] * b[1] - a[1] * b[0];
}
static inline double dt(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// point on the segment from `a` towards `b`, where the plane (normal n) is met: a - (d(a-c? ) ...)
// out = base - alpha * (base - other), alpha = dot(base - ref, n) / dot(base - other, n)
static inline void along(double *out, const double *base, const double *ref, const double *other, const double *n)
{
    double v1[3], v2[3];
    sub(v1, base, ref);
    sub(v2, base, other);
    double alpha = dt(v1, n) / dt(v2, n);
    v1[0] = alpha * v2[0];
    v1[1] = alpha * v2[1];
    v1[2] = alpha * v2[2];
    sub(out, base, v1);
}

// tri_tri_intersect.c:285-356, with (p1,q1,r1) and (p2,q2,r2) already in canonical order
static int construct(const double *p1, const double *q1, const double *r1, const double *p2, const double *q2,
                     const double *r2, const double *N1, const double *N2, double *src, double *tgt)
{
    double v1[3], v2[3], v[3], N[3];
    sub(v1, q1, p1);
    sub(v2, r2, p1);
    crs(N, v1, v2);
    sub(v, p2, p1);
    if (dt(v, N) > 0.0) {
        sub(v1, r1, p1);
        crs(N, v1, v2);
        if (dt(v, N) <= 0.0) {
            sub(v2, q2, p1);
            crs(N, v1, v2);
            if (dt(v, N) > 0.0) {
                along(src, p1, p2, r1, N2);
                along(tgt, p2, p1, r2, N1);
            } else {
                along(src, p2, p1, q2, N1);
                along(tgt, p2, p1, r2, N1);
            }
            return 1;
        }
        return 0;
    }
    sub(v2, q2, p1);
    crs(N, v1, v2);
    if (dt(v, N) < 0.0)
        return 0;
    sub(v1, r1, p1);
    crs(N, v1, v2);
    if (dt(v, N) >= 0.0) {
        along(src, p1, p2, r1, N2);
        along(tgt, p1, p2, q1, N2);
    } else {
        along(src, p2, p1, q2, N1);
        along(tgt, p1, p2, q1, N2);
    }
    return 1;
}

// second-level permutation of T2 (tri_tri_intersect.c:360-385); returns -1 for coplanar
static int stage2(const double *p1, const double *q1, const double *r1, const double *p2, const double *q2,
                  const double *r2, double dp2, double dq2, double dr2, const double *N1, const double *N2,
                  double *s, double *t)
{
    if (dp2 > 0.0) {
        if (dq2 > 0.0)
            return construct(p1, r1, q1, r2, p2, q2, N1, N2, s, t);
        if (dr2 > 0.0)
            return construct(p1, r1, q1, q2, r2, p2, N1, N2, s, t);
        return construct(p1, q1, r1, p2, q2, r2, N1, N2, s, t);
    }
    if (dp2 < 0.0) {
        if (dq2 < 0.0)
            return construct(p1, q1, r1, r2, p2, q2, N1, N2, s, t);
        if (dr2 < 0.0)
            return construct(p1, q1, r1, q2, r2, p2, N1, N2, s, t);
        return construct(p1, r1, q1, p2, q2, r2, N1, N2, s, t);
    }
    if (dq2 < 0.0) {
        if (dr2 >= 0.0)
            return construct(p1, r1, q1, q2, r2, p2, N1, N2, s, t);
        return construct(p1, q1, r1, p2, q2, r2, N1, N2, s, t);
    }
    if (dq2 > 0.0) {
        if (dr2 > 0.0)
            return construct(p1, r1, q1, p2, q2, r2, N1, N2, s, t);
        return construct(p1, q1, r1, q2, r2, p2, N1, N2, s, t);
    }
    if (dr2 > 0.0)
        return construct(p1, q1, r1, r2, p2, q2, N1, N2, s, t);
    if (dr2 < 0.0)
        return construct(p1, r1, q1, r2, p2, q2, N1, N2, s, t);
    return -1;
}

// tri_tri_intersect.c:395-472. Returns 1 for a segment, 0 for none, -1 for coplanar.
static int intersect(const double *p1, const double *q1, const double *r1, const double *p2, const double *q2,
                     const double *r2, double *s, double *t)
{
    double v1[3], v2[3], N1[3], N2[3];
    sub(v1, p2, r2);
    sub(v2, q2, r2);
    crs(N2, v1, v2);
    sub(v1, p1, r2);
    double dp1 = dt(v1, N2);
    sub(v1, q1, r2);
    double dq1 = dt(v1, N2);
    sub(v1, r1, r2);
    double dr1 = dt(v1, N2);
    if (((dp1 * dq1) > 0.0) && ((dp1 * dr1) > 0.0))
        return 0;
    sub(v1, q1, p1);
    sub(v2, r1, p1);
    crs(N1, v1, v2);
    sub(v1, p2, r1);
    double dp2 = dt(v1, N1);
    sub(v1, q2, r1);
    double dq2 = dt(v1, N1);
    sub(v1, r2, r1);
    double dr2 = dt(v1, N1);
    if (((dp2 * dq2) > 0.0) && ((dp2 * dr2) > 0.0))
        return 0;
    if (dp1 > 0.0) {
        if (dq1 > 0.0)
            return stage2(r1, p1, q1, p2, r2, q2, dp2, dr2, dq2, N1, N2, s, t);
        if (dr1 > 0.0)
            return stage2(q1, r1, p1, p2, r2, q2, dp2, dr2, dq2, N1, N2, s, t);
        return stage2(p1, q1, r1, p2, q2, r2, dp2, dq2, dr2, N1, N2, s, t);
    }
    if (dp1 < 0.0) {
        if (dq1 < 0.0)
            return stage2(r1, p1, q1, p2, q2, r2, dp2, dq2, dr2, N1, N2, s, t);
        if (dr1 < 0.0)
            return stage2(q1, r1, p1, p2, q2, r2, dp2, dq2, dr2, N1, N2, s, t);
        return stage2(p1, q1, r1, p2, r2, q2, dp2, dr2, dq2, N1, N2, s, t);
    }
    if (dq1 < 0.0) {
        if (dr1 >= 0.0)
            return stage2(q1, r1, p1, p2, r2, q2, dp2, dr2, dq2, N1, N2, s, t);
        return stage2(p1, q1, r1, p2, q2, r2, dp2, dq2, dr2, N1, N2, s, t);
    }
    if (dq1 > 0.0) {
        if (dr1 > 0.0)
            return stage2(p1, q1, r1, p2, r2, q2, dp2, dr2, dq2, N1, N2, s, t);
        return stage2(q1, r1, p1, p2, q2, r2, dp2, dq2, dr2, N1, N2, s, t);
    }
    if (dr1 > 0.0)
        return stage2(r1, p1, q1, p2, q2, r2, dp2, dq2, dr2, N1, N2, s, t);
    if (dr1 < 0.0)
        return stage2(r1, p1, q1, p2, r2, q2, dp2, dr2, dq2, N1, N2, s, t);
    return -1;
}
} // namespace gd

// ---------------------------------------------------------------------------------------------------
// Per-face re-triangulation (retriangulator.cpp:29-337)
// ---------------------------------------------------------------------------------------------------
typedef std::unordered_map<size_t, std::unordered_set<size_t>> NeighborMap;

static inline bool onLine(const V2 &p, const V2 &a, const V2 &b, double faceScale)
{
    const double cr = std::abs(std::abs((p.y - a.y) * (b.x - a.x) - (p.x - a.x) * (b.y - a.y)));
    if (!(g_robust & 1))
        return cr <= kEps; // src/vector2.h:212-215, src/double.h:30-33
    // robust mode (not the reference): 256 eps L (L + S), L the edge's larger 2D extent, S the face's largest
    // absolute corner coordinate
    const double L = std::max(std::abs(b.x - a.x), std::abs(b.y - a.y));
    return cr <= (256.0 * kEps) * (L * (L + faceScale));
}
static inline bool inPolygon(const V2 &p, const std::vector<V2> &pts, const std::vector<size_t> &poly)
{
    bool inside = false;
    int i, j;
    for (i = 0, j = (int)poly.size() - 1; i < (int)poly.size(); j = i++) {
        const V2 &a = pts[poly[i]];
        const V2 &b = pts[poly[j]];
        if (((a.y > p.y) != (b.y > p.y)) && (p.x < (b.x - a.x) * (p.y - a.y) / (b.y - a.y) + a.x))
            inside = !inside;
    }
    return inside;
}

struct ReTri {
    V3 axis, origin, normal;
    double faceScale = 0.0; // largest absolute corner coordinate (robust mode only)
    std::vector<V2> pts;
    const NeighborMap *nbr = nullptr;
    std::vector<std::vector<size_t>> polylines, inner, polygons, tris;
    std::unordered_map<size_t, std::unordered_set<size_t>> innerParents, innerChildren;
    std::unordered_map<size_t, std::vector<size_t>> holes;
    int failure = 0; // 1 attach, 2 link

    void project(const std::vector<V3> &in)
    {
        V3 perp = cross3(normal, axis);
        for (const auto &p : in) {
            V3 d = p - origin;
            pts.push_back(V2{dot3(d, axis), dot3(d, perp)});
        }
    }
    ReTri(const std::vector<V3> &corners, const V3 &n) : normal(n)
    {
        axis = normalized(corners[1] - corners[0]);
        origin = corners[0];
        for (const auto &c : corners)
            faceScale = std::max(faceScale, std::max(std::abs(c.x), std::max(std::abs(c.y), std::abs(c.z))));
        project(corners);
    }
    void setEdges(const std::vector<V3> &p, const NeighborMap *m)
    {
        project(p);
        nbr = m;
    }

    void lookupPolylines()
    {
        std::vector<size_t> ends;
        for (const auto &it : *nbr)
            if (it.second.size() == 1)
                ends.push_back(it.first);
        for (const auto &it : *nbr)
            if (it.second.size() > 1)
                ends.push_back(it.first);
        std::unordered_set<size_t> visited;
        for (size_t start : ends) {
            if (visited.count(start))
                continue;
            std::queue<size_t> q;
            q.push(start);
            std::vector<size_t> line;
            while (!q.empty()) {
                size_t cur = q.front();
                visited.insert(cur);
                line.push_back(cur);
                q.pop();
                auto f = nbr->find(cur);
                if (f == nbr->end())
                    break;
                for (size_t nb : f->second)
                    if (!visited.count(nb)) {
                        q.push(nb);
                        break;
                    }
            }
            if (line.size() >= 3) {
                auto last = nbr->find(line.back());
                if (last->second.count(start)) {
                    inner.push_back(line);
                    continue;
                }
            }
            if (line.size() >= 2)
                polylines.push_back(line);
        }
    }

    int attach(const V2 &p)
    {
        for (int i = 0; i < 3; ++i)
            if (onLine(p, pts[i], pts[(i + 1) % 3], faceScale))
                return i;
        return -1;
    }

    bool buildPolygons()
    {
        struct EP {
            size_t point = 0, linkPoint = 0;
            int line = -1;
            bool reversed = false;
            double d2 = 0.0;
            int linkTo = -1;
        };
        std::vector<std::vector<EP>> onEdge(3);
        for (int li = 0; li < (int)polylines.size(); ++li) {
            const auto &line = polylines[li];
            int fe = attach(pts[line.front()]);
            int be = attach(pts[line.back()]);
            if (fe < 0 || be < 0) {
                failure = 1;
                return false;
            }
            V2 df{pts[line.front()].x - pts[fe].x, pts[line.front()].y - pts[fe].y};
            V2 db{pts[line.back()].x - pts[be].x, pts[line.back()].y - pts[be].y};
            EP a;
            a.point = line.front();
            a.linkPoint = line.back();
            a.line = li;
            a.reversed = false;
            a.d2 = df.x * df.x + df.y * df.y;
            onEdge[fe].push_back(a);
            EP b;
            b.point = line.back();
            b.linkPoint = line.front();
            b.line = li;
            b.reversed = true;
            b.d2 = db.x * db.x + db.y * db.y;
            onEdge[be].push_back(b);
        }
        for (auto &e : onEdge)
            std::sort(e.begin(), e.end(), [](const EP &x, const EP &y) { return x.d2 < y.d2; });
        std::vector<EP> ring;
        for (size_t i = 0; i < 3; ++i) {
            EP c;
            c.point = i;
            ring.push_back(c);
            for (const auto &e : onEdge[i])
                ring.push_back(e);
        }
        std::unordered_map<size_t, size_t> ringPos;
        for (size_t i = 0; i < ring.size(); ++i)
            if (ring[i].line != -1)
                ringPos.insert({ring[i].point, i});
        for (auto &e : ring) {
            if (e.line == -1)
                continue;
            auto f = ringPos.find(e.linkPoint);
            if (f == ringPos.end())
                continue;
            e.linkTo = (int)f->second;
        }
        std::unordered_set<size_t> visited;
        std::queue<size_t> starts;
        starts.push(0);
        while (!starts.empty()) {
            size_t s = starts.front();
            starts.pop();
            if (visited.count(s))
                continue;
            std::vector<size_t> poly;
            size_t k = s;
            do {
                const EP &e = ring[k];
                visited.insert(k);
                if (e.line == -1) {
                    poly.push_back(e.point);
                    k = (k + 1) % ring.size();
                } else if (e.linkTo != -1) {
                    const auto &line = polylines[e.line];
                    if (e.reversed)
                        for (int i = (int)line.size() - 1; i >= 0; --i)
                            poly.push_back(line[i]);
                    else
                        for (size_t p : line)
                            poly.push_back(p);
                    starts.push((k + 1) % ring.size());
                    k = (e.linkTo + 1) % ring.size();
                } else {
                    failure = 2;
                    return false;
                }
            } while (k != s);
            polygons.push_back(poly);
        }
        return true;
    }

    void hierarchy()
    {
        for (size_t i = 0; i < inner.size(); ++i)
            for (size_t j = i + 1; j < inner.size(); ++j) {
                if (inPolygon(pts[inner[i][0]], pts, inner[j])) {
                    innerChildren[j].insert(i);
                    innerParents[i].insert(j);
                } else if (inPolygon(pts[inner[j][0]], pts, inner[i])) {
                    innerChildren[i].insert(j);
                    innerParents[j].insert(i);
                }
            }
        for (size_t i = 0; i < inner.size(); ++i) {
            if (innerParents.count(i))
                continue;
            for (size_t j = 0; j < polygons.size(); ++j)
                if (inPolygon(pts[inner[i][0]], pts, polygons[j]))
                    holes[j].push_back(i);
        }
    }

    void earcutInto(const std::vector<size_t> &outerRing, const std::vector<const std::vector<size_t> *> &holeRings)
    {
        std::vector<std::vector<std::array<double, 2>>> rings;
        std::vector<size_t> ids;
        rings.emplace_back();
        for (size_t p : outerRing) {
            ids.push_back(p);
            rings.back().push_back({pts[p].x, pts[p].y});
        }
        for (const auto *h : holeRings) {
            rings.emplace_back();
            for (size_t p : *h) {
                ids.push_back(p);
                rings.back().push_back({pts[p].x, pts[p].y});
            }
        }
        Earcut ec;
        ec.run(rings);
        for (size_t i = 0; i + 2 < ec.indices.size(); i += 3)
            tris.push_back({ids[(size_t)ec.indices[i]], ids[(size_t)ec.indices[i + 1]], ids[(size_t)ec.indices[i + 2]]});
    }

    void triangulate()
    {
        for (size_t pi = 0; pi < polygons.size(); ++pi) {
            std::vector<const std::vector<size_t> *> hr;
            auto f = holes.find(pi);
            if (f != holes.end())
                for (size_t h : f->second)
                    hr.push_back(&inner[h]);
            earcutInto(polygons[pi], hr);
        }
        for (size_t pi = 0; pi < inner.size(); ++pi) {
            std::vector<const std::vector<size_t> *> hr;
            auto f = innerChildren.find(pi);
            if (f != innerChildren.end()) {
                std::unordered_set<size_t> kids = f->second;
                for (size_t c : f->second) {
                    auto g = innerChildren.find(c);
                    if (g != innerChildren.end())
                        for (size_t gc : g->second)
                            kids.erase(gc);
                }
                for (size_t c : kids)
                    hr.push_back(&inner[c]);
            }
            earcutInto(inner[pi], hr);
        }
    }

    bool run()
    {
        lookupPolylines();
        if (!buildPolygons())
            return false;
        hierarchy();
        triangulate();
        return true;
    }
};

// ---------------------------------------------------------------------------------------------------
// The boolean (solidboolean.cpp)
// ---------------------------------------------------------------------------------------------------
static inline uint64_t heKey(size_t a, size_t b) { return ((uint64_t)a << 32) | (uint64_t)b; }

struct Boolean {
    const Mesh *A, *B;
    std::vector<std::pair<size_t, size_t>> cand;
    std::vector<V3> newV;
    std::vector<std::array<size_t, 3>> newT;
    std::map<Key, size_t> newPos;
    std::vector<std::vector<size_t>> groupsA, groupsB;
    std::vector<bool> sidesA, sidesB;
    std::unordered_set<size_t> cutA, cutB;
    double tm[7] = {0, 0, 0, 0, 0, 0, 0};
    // debug views of intermediate orders: cut faces in the contexts' iteration order, the first mesh's loops
    std::vector<size_t> ctxOrderA, ctxOrderB;
    std::vector<std::vector<size_t>> loopsFirst;
    int64_t triRanges[4] = {0, 0, 0, 0}; // uncut first, uncut second, re-triangulated first, second

    size_t addNewPoint(const V3 &p)
    {
        auto r = newPos.insert({Key(p), newV.size()});
        if (r.second)
            newV.push_back(p);
        return r.first->second;
    }

    bool addUncut(const Mesh *m, const std::unordered_set<size_t> &used, std::unordered_map<uint64_t, size_t> &he)
    {
        size_t base = newV.size();
        newV.insert(newV.end(), m->v.begin(), m->v.end());
        for (size_t i = 0; i < m->t.size(); ++i) {
            if (used.count(i))
                continue;
            const auto &o = m->t[i];
            size_t idx = newT.size();
            newT.push_back({o[0] + base, o[1] + base, o[2] + base});
            const auto &n = newT.back();
            if (!he.insert({heKey(n[0], n[1]), idx}).second)
                return false;
            if (!he.insert({heKey(n[1], n[2]), idx}).second)
                return false;
            if (!he.insert({heKey(n[2], n[0]), idx}).second)
                return false;
        }
        return true;
    }

    struct Ctx {
        std::vector<V3> points;
        std::map<Key, size_t> pos;
        NeighborMap nbr;
        size_t add(const V3 &p)
        {
            auto r = pos.insert({Key(p), points.size()});
            if (r.second)
                points.push_back(p);
            return r.first->second;
        }
        void segment(const V3 &s, const V3 &t)
        {
            size_t a = 3 + add(s);
            size_t b = 3 + add(t);
            if (a != b) {
                nbr[a].insert(b);
                nbr[b].insert(a);
            }
        }
    };

    bool retri(const std::unordered_map<size_t, Ctx> &ctxs, const Mesh *m, size_t vbase,
               std::unordered_map<size_t, std::unordered_set<size_t>> &edges,
               std::unordered_map<uint64_t, size_t> &he)
    {
        for (const auto &it : ctxs) {
            const auto &tri = m->t[it.first];
            ReTri rt({m->v[tri[0]], m->v[tri[1]], m->v[tri[2]]}, m->normals[it.first]);
            rt.setEdges(it.second.points, &it.second.nbr);
            if (!rt.run())
                return false;
            std::vector<size_t> ids;
            ids.reserve(3 + it.second.points.size());
            ids.push_back(vbase + tri[0]);
            ids.push_back(vbase + tri[1]);
            ids.push_back(vbase + tri[2]);
            for (const auto &p : it.second.points)
                ids.push_back(addNewPoint(p));
            for (const auto &t : rt.tris) {
                size_t idx = newT.size();
                newT.push_back({ids[t[0]], ids[t[1]], ids[t[2]]});
                const auto &n = newT.back();
                he.insert({heKey(n[0], n[1]), idx});
                he.insert({heKey(n[1], n[2]), idx});
                he.insert({heKey(n[2], n[0]), idx});
            }
            for (const auto &e : it.second.nbr) {
                size_t from = ids[e.first];
                for (size_t to0 : e.second) {
                    size_t to = ids[to0];
                    edges[from].insert(to);
                    edges[to].insert(from);
                }
            }
        }
        return true;
    }

    static bool loops(const std::unordered_map<size_t, std::unordered_set<size_t>> &edges,
                      std::vector<std::vector<size_t>> &out)
    {
        std::unordered_set<size_t> visited;
        for (const auto &e : edges) {
            size_t start = e.first;
            if (visited.count(start))
                continue;
            std::queue<size_t> q;
            q.push(start);
            std::vector<size_t> line;
            while (!q.empty()) {
                size_t cur = q.front();
                visited.insert(cur);
                line.push_back(cur);
                q.pop();
                auto f = edges.find(cur);
                if (f == edges.end())
                    break;
                for (size_t nb : f->second)
                    if (!visited.count(nb)) {
                        q.push(nb);
                        break;
                    }
            }
            if (line.size() <= 2)
                return false;
            auto last = edges.find(line.back());
            if (!last->second.count(start))
                return false;
            out.push_back(line);
        }
        return true;
    }

    void faceGroups(const std::vector<std::vector<size_t>> &loopsIn, const std::unordered_map<uint64_t, size_t> &he,
                    size_t remStart, size_t remCount, std::vector<std::vector<size_t>> &groups)
    {
        std::unordered_map<uint64_t, size_t> heGroup;
        size_t g = 0;
        std::queue<std::pair<size_t, size_t>> q;
        for (const auto &loop : loopsIn) {
            for (size_t i = 0; i < loop.size(); ++i) {
                size_t j = (i + 1) % loop.size();
                uint64_t k1 = heKey(loop[i], loop[j]);
                heGroup.insert({k1, g});
                auto f1 = he.find(k1);
                if (f1 != he.end())
                    q.push({f1->second, g});
                uint64_t k2 = heKey(loop[j], loop[i]);
                heGroup.insert({k2, g + 1});
                auto f2 = he.find(k2);
                if (f2 != he.end())
                    q.push({f2->second, g + 1});
            }
            g += 2;
        }
        groups.resize(g);
        std::unordered_set<size_t> seen;
        auto drain = [&]() {
            while (!q.empty()) {
                auto tg = q.front();
                q.pop();
                if (seen.count(tg.first))
                    continue;
                seen.insert(tg.first);
                groups[tg.second].push_back(tg.first);
                const auto &t = newT[tg.first];
                for (int i = 0; i < 3; ++i) {
                    int j = (i + 1) % 3;
                    uint64_t k = heKey(t[i], t[j]);
                    if (heGroup.count(k))
                        continue;
                    heGroup.insert({k, tg.second});
                    auto f = he.find(heKey(t[j], t[i]));
                    if (f != he.end())
                        q.push({f->second, tg.second});
                }
            }
        };
        drain();
        for (size_t t = remStart; t < remStart + remCount; ++t) {
            if (seen.count(t))
                continue;
            groups.emplace_back();
            q.push({t, g});
            ++g;
            drain();
        }
    }

    bool pointInMesh(const V3 &p, const Mesh *m, const V3 &axis)
    {
        V3 end = p + axis;
        Box rb;
        rb.add(p);
        rb.add(end);
        std::vector<size_t> hitsTri;
        m->tree.boxQuery(0, rb, hitsTri);
        std::set<Key> hits;
        for (size_t ti : hitsTri) {
            const auto &t = m->t[ti];
            const V3 &a = m->v[t[0]];
            const V3 &n = m->normals[ti];
            V3 u = end - p;
            V3 w = p - a;
            double d = dot3(n, u);
            double nn = dot3(-n, w);
            if (std::abs(d) <= kEps)
                continue;
            double s = nn / d;
            if (s < 0 || s > 1 || std::isnan(s) || std::isinf(s))
                continue;
            V3 x = p + s * u;
            V3 tp[3] = {m->v[t[0]], m->v[t[1]], m->v[t[2]]};
            V3 n0 = unitNormal(x, tp[0], tp[1]);
            V3 n1 = unitNormal(x, tp[1], tp[2]);
            V3 n2 = unitNormal(x, tp[2], tp[0]);
            if (dot3(n0, n1) > 0 && dot3(n0, n2) > 0)
                hits.insert(Key(x));
        }
        return hits.size() % 2 != 0;
    }

    void sides(const std::vector<std::vector<size_t>> &groups, const Mesh *m, std::vector<bool> &out)
    {
        static const double mx = std::numeric_limits<double>::max();
        const V3 axes[3] = {V3(mx, kEps, kEps), V3(kEps, mx, kEps), V3(kEps, kEps, mx)};
        out.assign(groups.size(), false);
        for (size_t i = 0; i < groups.size(); ++i) {
            if (groups[i].empty())
                continue;
            const auto &t = newT[groups[i][0]];
            V3 c = (newV[t[0]] + newV[t[1]] + newV[t[2]]) / 3.0;
            size_t inside = 0, total = 0;
            for (int k = 0; k < 3; ++k) {
                if (pointInMesh(c, m, axes[k]))
                    ++inside;
                ++total;
            }
            out[i] = (float)inside / total > 0.5;
        }
    }

    bool combine()
    {
        using C = std::chrono::steady_clock;
        auto ms = [](C::time_point a, C::time_point b) {
            return std::chrono::duration<double, std::milli>(b - a).count();
        };
        auto t0 = C::now();
        A->tree.test(0, B->tree, 0, cand);
        auto t1 = C::now();
        std::unordered_map<size_t, Ctx> ctxA, ctxB;
        for (const auto &pr : cand) {
            const auto &fa = A->t[pr.first];
            const auto &fb = B->t[pr.second];
            double pa[3][3], pb[3][3];
            for (int k = 0; k < 3; ++k) {
                pa[k][0] = A->v[fa[k]].x;
                pa[k][1] = A->v[fa[k]].y;
                pa[k][2] = A->v[fa[k]].z;
                pb[k][0] = B->v[fb[k]].x;
                pb[k][1] = B->v[fb[k]].y;
                pb[k][2] = B->v[fb[k]].z;
            }
            double s[3], t[3];
            if (gd::intersect(pa[0], pa[1], pa[2], pb[0], pb[1], pb[2], s, t) != 1)
                continue;
            cutA.insert(pr.first);
            cutB.insert(pr.second);
            V3 S(s[0], s[1], s[2]), T(t[0], t[1], t[2]);
            ctxA[pr.first].segment(S, T);
            ctxB[pr.second].segment(S, T);
        }
        auto t2 = C::now();
        for (const auto &it : ctxA)
            ctxOrderA.push_back(it.first);
        for (const auto &it : ctxB)
            ctxOrderB.push_back(it.first);
        std::unordered_map<size_t, std::unordered_set<size_t>> edgesA, edgesB;
        std::vector<std::vector<size_t>> loopsA;
        std::unordered_map<uint64_t, size_t> heA, heB;
        size_t remA0 = newT.size();
        addUncut(A, cutA, heA);
        size_t remA = newT.size() - remA0;
        size_t remB0 = newT.size();
        addUncut(B, cutB, heB);
        size_t remB = newT.size() - remB0;
        auto t3 = C::now();
        tm[0] = ms(t0, t1);
        tm[1] = ms(t1, t2);
        tm[2] = ms(t2, t3);
        triRanges[0] = (int64_t)remA;
        triRanges[1] = (int64_t)remB;
        const size_t retri0 = newT.size();
        if (!retri(ctxA, A, 0, edgesA, heA))
            return false;
        triRanges[2] = (int64_t)(newT.size() - retri0);
        if (!retri(ctxB, B, A->v.size(), edgesB, heB))
            return false;
        triRanges[3] = (int64_t)(newT.size() - retri0) - triRanges[2];
        auto t4 = C::now();
        tm[3] = ms(t3, t4);
        const bool loopsOk = loops(edgesA, loopsA);
        loopsFirst = loopsA;
        if (!loopsOk)
            return false;
        auto t5 = C::now();
        tm[4] = ms(t4, t5);
        faceGroups(loopsA, heA, remA0, remA, groupsA);
        faceGroups(loopsA, heB, remB0, remB, groupsB);
        auto t6 = C::now();
        tm[5] = ms(t5, t6);
        sides(groupsA, B, sidesA);
        sides(groupsB, A, sidesB);
        tm[6] = ms(t6, C::now());
        return true;
    }

    void fetch(int op, std::vector<std::array<size_t, 3>> &out)
    {
        for (size_t i = 0; i < sidesA.size(); ++i) {
            if (sidesA[i] != (op == 2))
                continue;
            for (size_t t : groupsA[i])
                out.push_back(newT[t]);
        }
        for (size_t i = 0; i < sidesB.size(); ++i) {
            bool want = (op != 0);
            if (sidesB[i] != want)
                continue;
            for (size_t t : groupsB[i]) {
                const auto &x = newT[t];
                if (op == 1)
                    out.push_back({x[2], x[1], x[0]});
                else
                    out.push_back(x);
            }
        }
    }
};

} // namespace port

using namespace port;

static sbo::Dump *run_once(const double *va, size_t nva, const uint32_t *ta, size_t nta, const double *vb,
                           size_t nvb, const uint32_t *tb, size_t ntb, long quantum)
{
    using C = std::chrono::steady_clock;
    g_factor = quantum;
    auto *d = new sbo::Dump;
    Mesh a, b;
    for (size_t i = 0; i < nva; ++i)
        a.v.emplace_back(va[3 * i], va[3 * i + 1], va[3 * i + 2]);
    for (size_t i = 0; i < nvb; ++i)
        b.v.emplace_back(vb[3 * i], vb[3 * i + 1], vb[3 * i + 2]);
    for (size_t i = 0; i < nta; ++i)
        a.t.push_back({ta[3 * i], ta[3 * i + 1], ta[3 * i + 2]});
    for (size_t i = 0; i < ntb; ++i)
        b.t.push_back({tb[3 * i], tb[3 * i + 1], tb[3 * i + 2]});
    auto t0 = C::now();
    a.prepare();
    auto t1 = C::now();
    b.prepare();
    auto t2 = C::now();
    Boolean sb;
    sb.A = &a;
    sb.B = &b;
    bool ok = sb.combine();
    d->i64["status"] = {ok ? 1 : 0};
    auto &cand = d->i64["cand"];
    auto &isect = d->i64["isect"];
    auto &seg = d->f64["seg"];
    for (const auto &pr : sb.cand) {
        cand.push_back((int64_t)pr.first);
        cand.push_back((int64_t)pr.second);
        const auto &fa = a.t[pr.first];
        const auto &fb = b.t[pr.second];
        double pa[3][3], pb[3][3];
        for (int k = 0; k < 3; ++k) {
            pa[k][0] = a.v[fa[k]].x;
            pa[k][1] = a.v[fa[k]].y;
            pa[k][2] = a.v[fa[k]].z;
            pb[k][0] = b.v[fb[k]].x;
            pb[k][1] = b.v[fb[k]].y;
            pb[k][2] = b.v[fb[k]].z;
        }
        double s[3] = {0, 0, 0}, t[3] = {0, 0, 0};
        bool hit = gd::intersect(pa[0], pa[1], pa[2], pb[0], pb[1], pb[2], s, t) == 1;
        isect.push_back(hit ? 1 : 0);
        for (int k = 0; k < 3; ++k)
            seg.push_back(hit ? s[k] : 0.0);
        for (int k = 0; k < 3; ++k)
            seg.push_back(hit ? t[k] : 0.0);
    }
    auto &nv = d->f64["newv"];
    for (const auto &v : sb.newV) {
        nv.push_back(v.x);
        nv.push_back(v.y);
        nv.push_back(v.z);
    }
    auto &nt = d->i64["newt"];
    for (const auto &t : sb.newT)
        for (int k = 0; k < 3; ++k)
            nt.push_back((int64_t)t[k]);
    auto groups = [&](const std::vector<std::vector<size_t>> &g, const char *off, const char *idx) {
        auto &o = d->i64[off];
        auto &x = d->i64[idx];
        o.push_back(0);
        for (const auto &grp : g) {
            for (auto t : grp)
                x.push_back((int64_t)t);
            o.push_back((int64_t)x.size());
        }
    };
    groups(sb.groupsA, "groups_a_off", "groups_a");
    groups(sb.groupsB, "groups_b_off", "groups_b");
    groups(sb.loopsFirst, "loops_a_off", "loops_a");
    d->i64["tri_ranges"] = {sb.triRanges[0], sb.triRanges[1], sb.triRanges[2], sb.triRanges[3]};
    for (size_t f : sb.ctxOrderA)
        d->i64["ctx_a"].push_back((int64_t)f);
    for (size_t f : sb.ctxOrderB)
        d->i64["ctx_b"].push_back((int64_t)f);
    d->i64["sides_a"];
    d->i64["sides_b"];
    for (bool s : sb.sidesA)
        d->i64["sides_a"].push_back(s ? 1 : 0);
    for (bool s : sb.sidesB)
        d->i64["sides_b"].push_back(s ? 1 : 0);
    const char *names[3] = {"union", "diff", "intersect"};
    for (int op = 0; op < 3; ++op) {
        std::vector<std::array<size_t, 3>> r;
        sb.fetch(op, r);
        auto &o = d->i64[names[op]];
        for (const auto &t : r)
            for (int k = 0; k < 3; ++k)
                o.push_back((int64_t)t[k]);
    }
    a.tree.leafOrder(0, d->i64["leaforder_a"]);
    b.tree.leafOrder(0, d->i64["leaforder_b"]);
    auto ms = [](C::time_point x, C::time_point y) { return std::chrono::duration<double, std::milli>(y - x).count(); };
    d->f64["time_ms"] = {ms(t0, t1), ms(t1, t2), sb.tm[0], sb.tm[1], sb.tm[2], sb.tm[3], sb.tm[4], sb.tm[5], sb.tm[6]};
    g_factor = 100000;
    return d;
}

extern "C" void *sbo_run(const double *va, size_t nva, const uint32_t *ta, size_t nta, const double *vb, size_t nvb,
                         const uint32_t *tb, size_t ntb, long quantum)
{
    g_robust = 0;
    return run_once(va, nva, ta, nta, vb, nvb, tb, ntb, quantum);
}

// The robust mode's checker (not the reference): flags bit 0 = scale-relative point-on-edge test, bit 1 =
// after a failed combine, combine again with the quantum ten times finer while it stays <= 1e12 and the
// largest absolute coordinate of a triangle corner times it stays below 2^52.
extern "C" void *sbo_run_robust(const double *va, size_t nva, const uint32_t *ta, size_t nta, const double *vb,
                                size_t nvb, const uint32_t *tb, size_t ntb, long quantum, int flags)
{
    g_robust = flags;
    sbo::Dump *d = run_once(va, nva, ta, nta, vb, nvb, tb, ntb, quantum);
    long attempts = 1;
    if ((flags & 2) && d->i64["status"][0] == 0) {
        double maxAbs = 0.0;
        auto scan = [&](const double *v, const uint32_t *t, size_t nt) {
            for (size_t i = 0; i < 3 * nt; ++i)
                for (int k = 0; k < 3; ++k)
                    maxAbs = std::max(maxAbs, std::abs(v[3 * (size_t)t[i] + k]));
        };
        scan(va, ta, nta);
        scan(vb, tb, ntb);
        while (d->i64["status"][0] == 0 && quantum <= 100000000000L &&
               maxAbs * (double)(quantum * 10) < 4503599627370496.0) {
            quantum *= 10;
            delete d;
            d = run_once(va, nva, ta, nta, vb, nvb, tb, ntb, quantum);
            ++attempts;
        }
    }
    d->i64["attempts"] = {attempts};
    d->i64["weld_factor_used"] = {quantum};
    g_robust = 0;
    return d;
}

extern "C" long sbo_earcut(const double *xy, const int64_t *ring_off, long nrings, int64_t *out, long cap)
{
    std::vector<std::vector<std::array<double, 2>>> rings(nrings);
    for (long r = 0; r < nrings; ++r)
        for (int64_t i = ring_off[r]; i < ring_off[r + 1]; ++i)
            rings[r].push_back({xy[2 * i], xy[2 * i + 1]});
    Earcut ec;
    ec.run(rings);
    for (long i = 0; i < (long)ec.indices.size() && i < cap; ++i)
        out[i] = ec.indices[i];
    return (long)ec.indices.size();
}

extern "C" int sbo_tritri(const double *p1, const double *q1, const double *r1, const double *p2, const double *q2,
                          const double *r2, int *coplanar, double *seg)
{
    for (int k = 0; k < 6; ++k)
        seg[k] = 0.0;
    int r = gd::intersect(p1, q1, r1, p2, q2, r2, seg, seg + 3);
    *coplanar = r < 0 ? 1 : 0;
    return r;
}

SBO_DUMP_ACCESSORS
