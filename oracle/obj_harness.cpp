// Test infrastructure only: the reference test driver's OBJ loading (test/main.cpp:31-71: tinyobjloader with
// its default triangulation, vertices widened from tinyobj's float to double, triangles in shape order),
// compiled against the reference's own tiny_obj_loader.h so tests can pin solidboolean_gb300.objio to it.
// sbo_obj_load returns the counts; with room it also copies the vertices (x, y, z doubles) and triangles.
#include <string>
#include <vector>

#define TINYOBJLOADER_IMPLEMENTATION
#include "tiny_obj_loader.h"

extern "C" int sbo_obj_load(const char *path, double *verts, long vcap, unsigned int *tris, long tcap, long *nv,
                            long *nt)
{
    tinyobj::attrib_t attributes;
    std::vector<tinyobj::shape_t> shapes;
    std::vector<tinyobj::material_t> materials;
    std::string warn, err;
    if (!tinyobj::LoadObj(&attributes, &shapes, &materials, &warn, &err, path))
        return 1;
    const long n = (long)(attributes.vertices.size() / 3);
    long m = 0;
    for (const auto &shape : shapes)
        m += (long)(shape.mesh.indices.size() / 3);
    *nv = n;
    *nt = m;
    if (verts && vcap >= n)
        for (long i = 0; i < 3 * n; ++i)
            verts[i] = (double)attributes.vertices[(size_t)i];
    if (tris && tcap >= m) {
        long k = 0;
        for (const auto &shape : shapes)
            for (size_t i = 0; i + 2 < shape.mesh.indices.size(); i += 3) {
                for (int c = 0; c < 3; ++c)
                    tris[3 * k + c] = (unsigned int)shape.mesh.indices[i + c].vertex_index;
                ++k;
            }
    }
    return 0;
}
