"""CPU: the oracle restatement pinned against the reference (golden fixtures made from the compiled
reference sources, and the compiled reference itself where its sources are present)."""
import glob
import os
import re

import numpy as np
import pytest

from oracle import oracle
from solidboolean_gb300 import meshgen as mg

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ARRAYS = ["cand", "isect", "seg", "newv", "newt", "groups_a_off", "groups_a", "groups_b_off", "groups_b",
          "sides_a", "sides_b", "union", "diff", "intersect", "leaforder_a", "leaforder_b"]


def _eq(x, y) -> bool:
    x, y = np.asarray(x), np.asarray(y)
    if x.dtype.kind == "f" or y.dtype.kind == "f":
        return np.array_equal(x, y, equal_nan=True)  # degenerate constructions give NaN in both
    return np.array_equal(x, y)


def _same(a: dict, b: dict, keys=ARRAYS):
    bad = [k for k in keys if not _eq(a[k], b[k])]
    if int(a["status"]) != int(b["status"]):
        bad.append("status")
    return bad


def _boolean_fixtures():
    return [p for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))) if "va" in np.load(p).files]


@pytest.mark.parametrize("path", _boolean_fixtures())
def test_port_matches_golden(port, path):
    g = dict(np.load(path))
    d = port.run(g["va"], g["fa"], g["vb"], g["fb"], int(g["quantum"]))
    assert _same(g, d) == []


def test_port_earcut_matches_golden(port):
    g = np.load(os.path.join(GOLDEN, "earcut_random.npz"))
    xy, ro, po, idx, io = g["xy"], g["ring_off"], g["poly_off"], g["idx"], g["idx_off"]
    for p in range(len(po) - 1):
        rings = [xy[ro[r]:ro[r + 1]] for r in range(po[p], po[p + 1])]
        assert np.array_equal(port.earcut(rings), idx[io[p]:io[p + 1]]), p


def _workloads():
    yield "pair_small_3", mg.pair_small(3)
    yield "pair_large_L5", mg.pair_large(1234, 5)
    yield "near_tangent_L5", mg.near_tangent(1234, 5)
    va, fa, vb, fb, off = mg.diff_volume(1234, 4)
    yield "diff_volume_L4_offsets", (va, fa, vb + off, fb)
    rng = mg.SplitMix64(21)
    for i in range(12):
        va, fa, vb, fb, _ = mg.batch_pair(rng, 4)
        yield f"batch_{i}", (va, fa, vb, fb)
    # edge inputs: no candidates (apart, nested), every pair coplanar (identical meshes: combine fails),
    # a lone crossing triangle pair (open loop: combine fails), an empty second mesh, touching spheres
    v2, f2 = mg.icosphere(2)
    f2 = np.ascontiguousarray(f2, dtype=np.uint32)
    yield "edge_disjoint", (v2, f2, mg.transform(v2, 0.5, None, (5.0, 0.0, 0.0)), f2)
    yield "edge_nested", (v2, f2, mg.transform(v2, 0.5, None, (0.1, 0.0, 0.0)), f2)
    yield "edge_identical", (v2, f2, v2.copy(), f2.copy())
    tri = np.array([[0, 1, 2]], dtype=np.uint32)
    yield "edge_single", (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float), tri,
                          np.array([[0.2, 0.2, -1], [0.2, 0.2, 1], [1, 1, 0.5]], float), tri)
    yield "edge_empty_second", (v2, f2, np.zeros((0, 3)), np.zeros((0, 3), dtype=np.uint32))
    yield "edge_touching", (v2, f2, mg.transform(v2, 1.0, None, (2.0, 0.0, 0.0)), f2)


@pytest.mark.parametrize("name,meshes", list(_workloads()))
@pytest.mark.parametrize("quantum", [100000, 100000000])
def test_port_matches_reference(port, name, meshes, quantum):
    ref = oracle.reference()
    if ref is None:
        pytest.skip("reference sources not present")
    a = ref.run(*meshes, quantum)
    b = port.run(*meshes, quantum)
    assert _same(a, b) == []


def _earcut_fixtures():
    root = os.path.join(oracle.REF_ROOT, "thirdparty", "earcut.hpp", "test", "fixtures")
    for path in sorted(glob.glob(os.path.join(root, "*.cpp"))):
        text = open(path).read()
        m = re.search(r"Fixture<\w+>\s+\w+\(\"(\w+)\",\s*\d+,[^{]*\{(.*)\}\);", text, re.S)
        if not m:
            continue
        rings = []
        for ring in re.findall(r"\{((?:\{[-0-9.eE+]+,[-0-9.eE+]+\},?)+)\}", m.group(2)):
            pts = re.findall(r"\{([-0-9.eE+]+),([-0-9.eE+]+)\}", ring)
            rings.append(np.array([[float(x), float(y)] for x, y in pts]))
        if rings:
            yield m.group(1), rings


def test_port_earcut_matches_reference_fixtures(port):
    """The reference's own earcut fixtures, read from its test files, triangulated by both."""
    ref = oracle.reference()
    if ref is None:
        pytest.skip("reference sources not present")
    n = 0
    for name, rings in _earcut_fixtures():
        assert np.array_equal(port.earcut(rings), ref.earcut(rings)), name
        n += 1
    assert n >= 40


TRITRI = [
    # generic crossing
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.2, 0.2, -1], [0.2, 0.2, 1], [1, 1, 0.5]),
    # separated by the plane of the first
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 2]),
    # coplanar overlapping (rejected by the boolean)
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0.1, 0.1, 0], [2, 0.1, 0], [0.1, 2, 0]),
    # touching at a vertex
    ([0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 0], [0, 0, 1], [-1, -1, 1]),
    # edge through the interior, vertex on the plane
    ([0, 0, 0], [2, 0, 0], [0, 2, 0], [0.5, 0.5, 0], [0.5, 0.5, 1], [1.5, -0.5, 1]),
    # crossing with permuted vertex order
    ([0, 1, 0], [0, 0, 0], [1, 0, 0], [1, 1, 0.5], [0.2, 0.2, 1], [0.2, 0.2, -1]),
]


@pytest.mark.parametrize("case", range(len(TRITRI)))
def test_tritri_known_cases(port, case):
    p = [np.array(x, dtype=np.float64) for x in TRITRI[case]]
    r, cop, seg = port.tritri(*p)
    ref = oracle.reference()
    if ref is not None:
        r2, cop2, seg2 = ref.tritri(*p)
        assert (r == 1 and not cop) == (r2 == 1 and not cop2)
        if r == 1 and not cop:
            assert np.array_equal(seg, seg2)
    if case == 0:
        assert r == 1 and not cop
    if case == 1:
        assert r == 0
    if case == 2:
        assert cop == 1


def _cube():
    v = np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)], float)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    f = []
    for a, b, c, d in quads:
        f += [(a, b, c), (a, c, d)]
    return v, np.array(f, dtype=np.uint32)


def test_port_matches_reference_on_cubes(port):
    """Flat-faced inputs (a cube, two triangles per face, against a cube or an icosphere, random scales,
    rotations and offsets): most of these make the reference fail (its loop building on two-triangle faces),
    and the restatement must fail at the same stage with the same arrays, or succeed identically."""
    ref = oracle.reference()
    if ref is None:
        pytest.skip("reference sources not present")
    rng = mg.SplitMix64(3)
    failures = 0
    for i in range(60):
        va, fa = _cube()
        vb, fb = (_cube() if i % 3 == 0 else mg.icosphere(2 if i % 3 == 1 else 1))
        va = np.ascontiguousarray(mg.transform(va, rng.uniform(0.5, 1.5), mg.rotation_matrix(rng.unit_quaternion())))
        vb = np.ascontiguousarray(mg.transform(vb, rng.uniform(0.5, 1.5), mg.rotation_matrix(rng.unit_quaternion()),
                                               tuple(rng.unit_vector() * rng.uniform(0.2, 1.5))))
        fb = np.ascontiguousarray(fb, dtype=np.uint32)
        for quantum in (100000, 100000000):
            a = ref.run(va, fa, vb, fb, quantum)
            b = port.run(va, fa, vb, fb, quantum)
            assert _same(a, b) == [], (i, quantum)
            failures += int(a["status"]) == 0
    assert 0 < failures < 120  # both outcomes are exercised
