/*
 * Test-only dump harness around the UNMODIFIED reference sources (compiled in place by oracle/Makefile
 * into oracle/_ref/libsbref.so, never shipped). It drives the reference exactly like its own driver does
 * (test/main.cpp:92-103: SolidMesh setVertices/setTriangles/prepare, SolidBoolean(&a,&b).combine(),
 * fetchUnion/fetchDiff/fetchIntersect, resultVertices) and exposes the private stage state through the
 * sbo_* dump interface of sb_oracle.h. Private members are reached by re-declaring `private` as `public`
 * for the reference headers only (after every standard and Eigen header is already included).
 */
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <limits>
#include <map>
#include <queue>
#include <set>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#include <Eigen/Dense>
#include <earcut.hpp>

#define private public
#include "solidboolean.h"
#include "solidmesh.h"
#include "positionkey.h"
#include "axisalignedboundingboxtree.h"
#undef private
#include "tri_tri_intersect.h"
#include "sb_oracle_dump.hpp"

using Clock = std::chrono::steady_clock;
static double ms(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}
template <class TP>
static double msHR(TP a, TP b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

static void leafOrder(const AxisAlignedBoudingBoxTree::Node *n, std::vector<int64_t> &out)
{
    if (!n)
        return;
    if (n->isLeaf()) {
        for (auto i : n->boxIndices)
            out.push_back((int64_t)i);
        return;
    }
    leafOrder(n->left, out);
    leafOrder(n->right, out);
}

extern "C" void *sbo_run(const double *va, size_t nva, const uint32_t *ta, size_t nta,
                         const double *vb, size_t nvb, const uint32_t *tb, size_t ntb, long quantum)
{
    PositionKey::m_toIntFactor = quantum;
    auto *d = new sbo::Dump;
    std::vector<Vector3> av(nva), bv(nvb);
    std::vector<std::vector<size_t>> at(nta), bt(ntb);
    for (size_t i = 0; i < nva; ++i)
        av[i] = Vector3(va[3 * i], va[3 * i + 1], va[3 * i + 2]);
    for (size_t i = 0; i < nvb; ++i)
        bv[i] = Vector3(vb[3 * i], vb[3 * i + 1], vb[3 * i + 2]);
    for (size_t i = 0; i < nta; ++i)
        at[i] = {ta[3 * i], ta[3 * i + 1], ta[3 * i + 2]};
    for (size_t i = 0; i < ntb; ++i)
        bt[i] = {tb[3 * i], tb[3 * i + 1], tb[3 * i + 2]};

    auto t0 = Clock::now();
    SolidMesh a;
    a.setVertices(&av);
    a.setTriangles(&at);
    a.prepare();
    auto t1 = Clock::now();
    SolidMesh b;
    b.setVertices(&bv);
    b.setTriangles(&bt);
    b.prepare();
    auto t2 = Clock::now();
    SolidBoolean sb(&a, &b);
    bool ok = sb.combine();

    d->i64["status"] = {ok ? 1 : 0};
    auto &cand = d->i64["cand"];
    auto &isect = d->i64["isect"];
    auto &seg = d->f64["seg"];
    for (const auto &p : sb.m_potentialIntersectedPairs) {
        cand.push_back((int64_t)p.first);
        cand.push_back((int64_t)p.second);
        std::pair<Vector3, Vector3> e;
        bool hit = sb.intersectTwoFaces(p.first, p.second, e);
        isect.push_back(hit ? 1 : 0);
        for (int k = 0; k < 3; ++k)
            seg.push_back(hit ? e.first[k] : 0.0);
        for (int k = 0; k < 3; ++k)
            seg.push_back(hit ? e.second[k] : 0.0);
    }
    auto &nv = d->f64["newv"];
    for (const auto &v : sb.m_newVertices) {
        nv.push_back(v.x());
        nv.push_back(v.y());
        nv.push_back(v.z());
    }
    auto &nt = d->i64["newt"];
    for (const auto &t : sb.m_newTriangles)
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
    groups(sb.m_firstTriangleGroups, "groups_a_off", "groups_a");
    groups(sb.m_secondTriangleGroups, "groups_b_off", "groups_b");
    for (bool s : sb.m_firstGroupSides)
        d->i64["sides_a"].push_back(s ? 1 : 0);
    for (bool s : sb.m_secondGroupSides)
        d->i64["sides_b"].push_back(s ? 1 : 0);
    d->i64["sides_a"];
    d->i64["sides_b"];
    auto fetch = [&](int op, const char *name) {
        std::vector<std::vector<size_t>> r;
        if (op == 0)
            sb.fetchUnion(r);
        else if (op == 1)
            sb.fetchDiff(r);
        else
            sb.fetchIntersect(r);
        auto &o = d->i64[name];
        for (const auto &t : r)
            for (int k = 0; k < 3; ++k)
                o.push_back((int64_t)t[k]);
    };
    fetch(0, "union");
    fetch(1, "diff");
    fetch(2, "intersect");
    leafOrder(a.axisAlignedBoundingBoxTree()->root(), d->i64["leaforder_a"]);
    leafOrder(b.axisAlignedBoundingBoxTree()->root(), d->i64["leaforder_b"]);
    auto &tm = d->f64["time_ms"];
    tm = {ms(t0, t1), ms(t1, t2),
          msHR(sb.benchBegin_searchPotentialIntersectedPairs, sb.benchEnd_searchPotentialIntersectedPairs),
          msHR(sb.benchBegin_processPotentialIntersectedPairs, sb.benchEnd_processPotentialIntersectedPairs),
          msHR(sb.benchBegin_addUnintersectedTriangles, sb.benchEnd_addUnintersectedTriangles),
          msHR(sb.benchBegin_reTriangulate, sb.benchEnd_reTriangulate),
          msHR(sb.benchBegin_buildPolygonsFromEdges, sb.benchEnd_buildPolygonsFromEdges),
          msHR(sb.benchBegin_buildFaceGroups, sb.benchEnd_buildFaceGroups),
          msHR(sb.benchBegin_decideGroupSide, sb.benchEnd_decideGroupSide)};
    if (!ok)
        for (size_t k = 5; k < tm.size(); ++k)
            tm[k] = 0.0;
    PositionKey::m_toIntFactor = 100000;
    return d;
}

extern "C" long sbo_earcut(const double *xy, const int64_t *ring_off, long nrings, int64_t *out, long cap)
{
    std::vector<std::vector<std::array<double, 2>>> poly(nrings);
    for (long r = 0; r < nrings; ++r)
        for (int64_t i = ring_off[r]; i < ring_off[r + 1]; ++i)
            poly[r].push_back({xy[2 * i], xy[2 * i + 1]});
    std::vector<size_t> idx = mapbox::earcut<size_t>(poly);
    for (long i = 0; i < (long)idx.size() && i < cap; ++i)
        out[i] = (int64_t)idx[i];
    return (long)idx.size();
}

extern "C" int sbo_tritri(const double *p1, const double *q1, const double *r1, const double *p2,
                          const double *q2, const double *r2, int *coplanar, double *seg)
{
    double a[3], b[3], c[3], d[3], e[3], f[3];
    std::memcpy(a, p1, sizeof a);
    std::memcpy(b, q1, sizeof b);
    std::memcpy(c, r1, sizeof c);
    std::memcpy(d, p2, sizeof d);
    std::memcpy(e, q2, sizeof e);
    std::memcpy(f, r2, sizeof f);
    *coplanar = 0;
    for (int k = 0; k < 6; ++k)
        seg[k] = 0.0;
    return tri_tri_intersection_test_3d(a, b, c, d, e, f, coplanar, seg, seg + 3);
}

SBO_DUMP_ACCESSORS
