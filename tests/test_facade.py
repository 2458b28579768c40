"""The header-only C++ facade (include/solidboolean_gb300.hpp) used the way the reference's own caller uses
the reference classes (test/main.cpp:92-152: setVertices / setTriangles / prepare, SolidBoolean, combine,
fetchUnion / fetchDiff / fetchIntersect appending to a vector, resultVertices). CPU: the caller compiles
against the header and links against the library. GPU: it runs, and its results equal the Python API's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import solidboolean_gb300 as sbg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CALLER = r"""
#include <cstdio>
#include <vector>
#include "solidboolean_gb300.hpp"

// the reference's Vector3 interface as the facade needs it
struct Vector3 {
    double v[3];
    Vector3(double x, double y, double z) : v{x, y, z} {}
    double x() const { return v[0]; }
    double y() const { return v[1]; }
    double z() const { return v[2]; }
};

static void readMesh(const char *vf, const char *tf, std::vector<Vector3> &verts,
                     std::vector<std::vector<size_t>> &tris)
{
    FILE *f = std::fopen(vf, "rb");
    double p[3];
    while (std::fread(p, sizeof p, 1, f) == 1)
        verts.emplace_back(p[0], p[1], p[2]);
    std::fclose(f);
    f = std::fopen(tf, "rb");
    unsigned int t[3];
    while (std::fread(t, sizeof t, 1, f) == 1)
        tris.push_back({t[0], t[1], t[2]});
    std::fclose(f);
}

static void writeTris(const char *path, const std::vector<std::vector<size_t>> &tris)
{
    FILE *f = std::fopen(path, "wb");
    for (const auto &t : tris) {
        unsigned int v[3] = {(unsigned int)t[0], (unsigned int)t[1], (unsigned int)t[2]};
        std::fwrite(v, sizeof v, 1, f);
    }
    std::fclose(f);
}

int main(int argc, char **argv)
{
    using SolidMesh = solidboolean_gb300::SolidMesh<Vector3>;
    using SolidBoolean = solidboolean_gb300::SolidBoolean<Vector3>;
    std::vector<Vector3> firstVertices, secondVertices;
    std::vector<std::vector<size_t>> firstTriangles, secondTriangles;
    readMesh(argv[1], argv[2], firstVertices, firstTriangles);
    readMesh(argv[3], argv[4], secondVertices, secondTriangles);

    SolidMesh firstMesh;
    firstMesh.setVertices(&firstVertices);
    firstMesh.setTriangles(&firstTriangles);
    firstMesh.prepare();
    SolidMesh secondMesh;
    secondMesh.setVertices(&secondVertices);
    secondMesh.setTriangles(&secondTriangles);
    secondMesh.prepare();

    SolidBoolean solidBoolean(&firstMesh, &secondMesh);
    if (!solidBoolean.combine()) {
        std::printf("combine failed\n");
        return 3;
    }
    std::vector<std::vector<size_t>> u, d, x;
    solidBoolean.fetchUnion(u);
    solidBoolean.fetchDiff(d);
    solidBoolean.fetchIntersect(x);
    writeTris(argv[6], u);
    writeTris(argv[7], d);
    writeTris(argv[8], x);
    const std::vector<Vector3> &verts = solidBoolean.resultVertices();
    FILE *f = std::fopen(argv[5], "wb");
    for (const auto &p : verts)
        std::fwrite(p.v, sizeof p.v, 1, f);
    std::fclose(f);
    std::printf("ok %zu vertices\n", verts.size());
    return 0;
}
"""


def _build_caller(tmp_path) -> str:
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    if not os.path.exists(sbg.LIB_PATH):
        from solidboolean_gb300 import build as b
        b.build()
    src = tmp_path / "caller.cpp"
    src.write_text(CALLER)
    exe = str(tmp_path / "caller")
    libdir = os.path.dirname(sbg.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-L", libdir,
                    "-lsolidboolean_gb300", f"-Wl,-rpath,{libdir}", "-o", exe], check=True, capture_output=True)
    return exe


def test_facade_compiles_and_links(tmp_path):
    exe = _build_caller(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_facade_caller_matches_python_api(gpu_lib, tmp_path):
    from solidboolean_gb300 import meshgen as mg
    exe = _build_caller(tmp_path)
    va, fa, vb, fb = mg.pair_small(1234)
    names = ["va", "fa", "vb", "fb"]
    for n, a, dt in zip(names, (va, fa, vb, fb), (np.float64, np.uint32, np.float64, np.uint32)):
        np.ascontiguousarray(a, dtype=dt).tofile(str(tmp_path / f"{n}.bin"))
    outs = ["verts", "union", "diff", "intersect"]
    args = [str(tmp_path / f"{n}.bin") for n in names + outs]
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ref = sbg.run_boolean(va, fa, vb, fb, 100000)
    assert ref["status"] == 1
    verts = np.fromfile(args[4], dtype=np.float64).reshape(-1, 3)
    assert np.array_equal(verts, ref["newv"])
    for k, name in enumerate(("union", "diff", "intersect")):
        tris = np.fromfile(args[5 + k], dtype=np.uint32).reshape(-1, 3).astype(np.int64)
        assert np.array_equal(tris, ref[name]), name
