"""CPU: the reference's own test meshes (test/cases/*/{a,b}.obj, Dust3D models with quads), read the way
its test driver reads them (solidboolean_gb300.objio), through the oracle restatement and the compiled
reference: every stage array must agree. Skipped where the reference sources are absent. Also checks that
OBJ output reads back."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle
from solidboolean_gb300 import meshgen as mg
from solidboolean_gb300 import objio

from test_oracle import _same


def _cases():
    root = os.path.join(oracle.REF_ROOT, "test", "cases")
    for d in sorted(glob.glob(os.path.join(root, "*"))):
        a, b = os.path.join(d, "a.obj"), os.path.join(d, "b.obj")
        if os.path.isfile(a) and os.path.isfile(b):
            yield os.path.basename(d), a, b


@pytest.mark.parametrize("quantum", [100000, 100000000])
def test_port_matches_reference_on_reference_meshes(port, quantum):
    ref = oracle.reference()
    cases = list(_cases())
    if ref is None or not cases:
        pytest.skip("reference sources not present")
    for name, a, b in cases:
        va, fa = objio.load_obj(a)
        vb, fb = objio.load_obj(b)
        assert len(fa) > 0 and len(fb) > 0, name
        r = ref.run(va, fa, vb, fb, quantum)
        p = port.run(va, fa, vb, fb, quantum)
        assert _same(r, p) == [], (name, quantum)


def test_quads_split_into_two_triangles():
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], dtype=np.float32)
    assert objio._triangulate([0, 1, 2, 3], v) == [(0, 1, 2), (0, 2, 3)]


def test_obj_round_trip(tmp_path):
    v, f = mg.icosphere(2)
    v = v.astype(np.float32).astype(np.float64)
    path = str(tmp_path / "m.obj")
    objio.save_obj(path, v, f)
    v2, f2 = objio.load_obj(path)
    assert np.array_equal(f2, f.astype(np.uint32))
    assert np.allclose(v2, v, atol=1e-6)


def test_reader_matches_reference_loader():
    """objio against the reference test driver's own loader (tinyobjloader compiled from the reference's
    header): identical vertices and triangles on every test mesh."""
    load = oracle.obj_reference()
    cases = list(_cases())
    if load is None or not cases:
        pytest.skip("reference sources not present")
    for name, a, b in cases:
        for path in (a, b):
            v_ref, t_ref = load(path)
            v, t = objio.load_obj(path)
            assert np.array_equal(v, v_ref), (name, path)
            assert np.array_equal(t, t_ref), (name, path)


def test_reader_matches_reference_loader_on_polygons(tmp_path):
    """Faces of 4 to 9 corners, convex and concave (random star-shaped polygons in random planes), written
    as OBJ and read by both loaders: same triangles, same vertices."""
    load = oracle.obj_reference()
    if load is None:
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(11)
    lines, nv = [], 0
    for _ in range(300):
        k = int(rng.integers(4, 10))
        ang = np.sort(rng.uniform(0, 2 * np.pi, k))
        rad = rng.uniform(0.3, 1.0, k)
        pts2 = np.stack([rad * np.cos(ang), rad * np.sin(ang)], 1)
        basis = np.linalg.qr(rng.standard_normal((3, 3)))[0]
        pts = pts2 @ basis[:2] + rng.uniform(-5, 5, 3)
        for p in pts:
            lines.append(f"v {p[0]:.6f} {p[1]:.6f} {p[2]:.6f}")
        order = list(range(nv + 1, nv + k + 1))
        if rng.random() < 0.5:
            order = order[::-1]
        lines.append("f " + " ".join(str(i) for i in order))
        nv += k
    path = str(tmp_path / "polys.obj")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    v_ref, t_ref = load(path)
    v, t = objio.load_obj(path)
    assert np.array_equal(v, v_ref)
    assert np.array_equal(t, t_ref)
