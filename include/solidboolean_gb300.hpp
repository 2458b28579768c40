// Header-only C++ facade with the reference's class names and signatures (src/solidmesh.h:29-74,
// src/solidboolean.h:33-58) over the C ABI of libsolidboolean_gb300.so. A caller of the reference switches
// by including this header instead of solidmesh.h / solidboolean.h and linking the library; Vector3 is
// any type with x(), y(), z() accessors and a (x, y, z) constructor (the reference's Vector3 works).
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "solidboolean_gb300.h"

namespace solidboolean_gb300 {

template <class Vector3> class SolidMesh {
public:
    ~SolidMesh() { sb_mesh_destroy(m_mesh); }
    void setVertices(const std::vector<Vector3> *vertices) { m_vertices = vertices; }
    void setTriangles(const std::vector<std::vector<size_t>> *triangles) { m_triangles = triangles; }
    const std::vector<Vector3> *vertices() const { return m_vertices; }
    const std::vector<std::vector<size_t>> *triangles() const { return m_triangles; }
    // uploads the mesh and builds its GPU acceleration structures (the reference's prepare())
    void prepare(const sb_options *opts = nullptr)
    {
        std::vector<double> xyz;
        std::vector<uint32_t> tris;
        if (m_vertices)
            for (const auto &v : *m_vertices) {
                xyz.push_back(v.x());
                xyz.push_back(v.y());
                xyz.push_back(v.z());
            }
        if (m_triangles)
            for (const auto &t : *m_triangles)
                for (int k = 0; k < 3; ++k)
                    tris.push_back((uint32_t)t[k]);
        sb_mesh_destroy(m_mesh);
        m_mesh = nullptr;
        check(sb_mesh_create(xyz.data(), xyz.size() / 3, tris.data(), tris.size() / 3, &m_mesh));
        check(sb_mesh_prepare(m_mesh, opts));
    }
    sb_mesh *handle() const { return m_mesh; }

    static void check(sb_status s)
    {
        if (s != SB_OK && s != SB_FAIL_ATTACH && s != SB_FAIL_LINK && s != SB_FAIL_LOOP)
            throw std::runtime_error(std::string(sb_status_string(s)) + ": " + sb_last_error());
    }

private:
    const std::vector<Vector3> *m_vertices = nullptr;
    const std::vector<std::vector<size_t>> *m_triangles = nullptr;
    sb_mesh *m_mesh = nullptr;
};

template <class Vector3> class SolidBoolean {
public:
    // The results are read on the host through this class, so combine() stages them in page-locked memory
    // (sb_options.stage_results): the reads below convert from there instead of copying from the device.
    SolidBoolean(const SolidMesh<Vector3> *firstMesh, const SolidMesh<Vector3> *secondMesh,
                 const sb_options *opts = nullptr)
    {
        sb_options o;
        if (opts)
            o = *opts;
        else
            sb_default_options(&o);
        o.stage_results = 1;
        SolidMesh<Vector3>::check(sb_boolean_create(firstMesh->handle(), secondMesh->handle(), &o, &m_b));
    }
    ~SolidBoolean() { sb_boolean_destroy(m_b); }
    bool combine()
    {
        m_haveVertices = false;
        return sb_combine(m_b, nullptr) == SB_OK;
    }
    void fetchUnion(std::vector<std::vector<size_t>> &out) { fetch(SB_UNION, out); }
    void fetchDiff(std::vector<std::vector<size_t>> &out) { fetch(SB_DIFF, out); }
    void fetchIntersect(std::vector<std::vector<size_t>> &out) { fetch(SB_INTERSECT, out); }
    // built once per combine, like the reference's member (src/solidboolean.h:44)
    const std::vector<Vector3> &resultVertices()
    {
        if (m_haveVertices)
            return m_resultVertices;
        m_resultVertices.clear();
        size_t n = 0;
        void *staged = nullptr;
        if (sb_take_staged(m_b, SB_STAGED_VERTICES, &staged, &n) != SB_OK)
            return m_resultVertices;
        std::vector<double> copy;
        const double *xyz = static_cast<const double *>(staged);
        if (!staged && n) {
            copy.resize(3 * n);
            SolidMesh<Vector3>::check(sb_result_vertices(m_b, copy.data(), n, &n));
            xyz = copy.data();
        }
        m_resultVertices.reserve(n);
        for (size_t i = 0; i < n; ++i)
            m_resultVertices.emplace_back(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        sb_host_free(staged);
        m_haveVertices = true;
        return m_resultVertices;
    }

private:
    // appends, like the reference (src/solidboolean.cpp:512-565)
    void fetch(sb_op op, std::vector<std::vector<size_t>> &out)
    {
        size_t n = 0;
        void *staged = nullptr;
        if (sb_take_staged(m_b, op, &staged, &n) != SB_OK || n == 0) {
            sb_host_free(staged);
            return;
        }
        std::vector<uint32_t> copy;
        const uint32_t *t = static_cast<const uint32_t *>(staged);
        if (!staged) {
            copy.resize(3 * n);
            SolidMesh<Vector3>::check(sb_fetch(m_b, op, copy.data(), n, &n));
            t = copy.data();
        }
        out.reserve(out.size() + n);
        for (size_t i = 0; i < n; ++i)
            out.push_back({t[3 * i], t[3 * i + 1], t[3 * i + 2]});
        sb_host_free(staged);
    }
    sb_boolean *m_b = nullptr;
    std::vector<Vector3> m_resultVertices;
    bool m_haveVertices = false;
};

} // namespace solidboolean_gb300
