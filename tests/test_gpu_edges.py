"""GPU parity beyond the synthetic spheres: the reference's own test meshes, edge inputs, flat-faced cubes,
and the device ear-clipper on the reference's earcut fixtures.

* The reference's test meshes (test/cases/*/{a,b}.obj: Dust3D models with quads, read like its test driver
  reads them) travel as tests/golden/reference_meshes.npz; the CUDA path must reproduce the compiled
  reference's digests (reference_meshes_digests.json) and equal the oracle element by element.
* Edge inputs (no candidates, every pair coplanar, a lone crossing pair, an empty mesh, touching meshes) and
  60 cube/cube and cube/sphere pairs, where many orientation determinants are exactly zero (the FP32
  filter's uncertified path) and most combines fail: the CUDA path must fail or succeed like the oracle,
  with the same arrays.
* The device ear-clipper (sb_debug_earcut) on the reference's earcut fixtures, polygons of up to 1,500
  points (13 of them beyond the 80 points where earcut switches to z-order hashing): the same triangle
  indices as the reference's earcut. The CPU tests cover the larger fixtures on the oracle.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import solidboolean_gb300 as sbg
from solidboolean_gb300 import meshgen as mg
from parity import compare, digests, input_digest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _reference_meshes():
    g = np.load(os.path.join(GOLDEN, "reference_meshes.npz"))
    names = sorted({k.split(":")[0] for k in g.files})
    return {n: (g[f"{n}:va"], g[f"{n}:fa"], g[f"{n}:vb"], g[f"{n}:fb"]) for n in names}


@pytest.mark.parametrize("weld", [100000, 100000000])
@pytest.mark.parametrize("precision", ["filtered", "fp64"])
def test_reference_meshes(gpu_lib, port, weld, precision):
    with open(os.path.join(GOLDEN, "reference_meshes_digests.json")) as f:
        table = json.load(f)
    meshes = _reference_meshes()
    assert len(meshes) == 4
    for name, (va, fa, vb, fb) in meshes.items():
        want = table[f"{name}:{weld}"]
        assert input_digest(va, fa, vb, fb) == want["inputs"]
        got = sbg.run_boolean(va, fa, vb, fb, weld, precision)
        assert digests(got, len(va) + len(vb), weld) == {k: v for k, v in want.items()
                                                         if k not in ("inputs", "quantum")}, name
        ref = port.run(va, fa, vb, fb, weld)
        bad = compare(ref, got, len(va) + len(vb), weld, strict=True)
        assert not bad, (name, bad)


def _edge_inputs():
    v2, f2 = mg.icosphere(2)
    f2 = np.ascontiguousarray(f2, dtype=np.uint32)
    yield "disjoint", (v2, f2, mg.transform(v2, 0.5, None, (5.0, 0.0, 0.0)), f2)
    yield "nested", (v2, f2, mg.transform(v2, 0.5, None, (0.1, 0.0, 0.0)), f2)
    yield "identical", (v2, f2, v2.copy(), f2.copy())
    tri = np.array([[0, 1, 2]], dtype=np.uint32)
    yield "single", (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float), tri,
                     np.array([[0.2, 0.2, -1], [0.2, 0.2, 1], [1, 1, 0.5]], float), tri)
    yield "touching", (v2, f2, mg.transform(v2, 1.0, None, (2.0, 0.0, 0.0)), f2)


@pytest.mark.parametrize("weld", [100000, 100000000])
@pytest.mark.parametrize("precision", ["filtered", "fp64"])
def test_edge_inputs(gpu_lib, port, weld, precision):
    for name, (va, fa, vb, fb) in _edge_inputs():
        ref = port.run(va, fa, vb, fb, weld)
        got = sbg.run_boolean(va, fa, vb, fb, weld, precision)
        bad = compare(ref, got, len(va) + len(vb), weld, strict=True)
        assert not bad, (name, bad, got["stats"])


def test_empty_mesh_is_rejected_or_matches(gpu_lib, port):
    """An empty second mesh: the reference combines nothing with it; the library either does the same or
    rejects the empty mesh at creation (it holds no triangles to build a tree over)."""
    v2, f2 = mg.icosphere(2)
    f2 = np.ascontiguousarray(f2, dtype=np.uint32)
    va, fa, vb, fb = v2, f2, np.zeros((0, 3)), np.zeros((0, 3), dtype=np.uint32)
    ref = port.run(va, fa, vb, fb, 100000)
    try:
        got = sbg.run_boolean(va, fa, vb, fb, 100000)
    except (RuntimeError, ValueError) as e:
        pytest.skip(f"empty meshes are rejected: {e}")
    assert not compare(ref, got, len(va) + len(vb), 100000, strict=True)


def _cube():
    v = np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)], float)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    f = []
    for a, b, c, d in quads:
        f += [(a, b, c), (a, c, d)]
    return v, np.array(f, dtype=np.uint32)


@pytest.mark.parametrize("precision", ["filtered", "fp64"])
def test_cubes(gpu_lib, port, precision):
    """The oracle's cube set (pinned to the compiled reference on the CPU): same seeds, same statuses, same
    arrays."""
    rng = mg.SplitMix64(3)
    failures = 0
    for i in range(60):
        va, fa = _cube()
        vb, fb = (_cube() if i % 3 == 0 else mg.icosphere(2 if i % 3 == 1 else 1))
        va = np.ascontiguousarray(mg.transform(va, rng.uniform(0.5, 1.5), mg.rotation_matrix(rng.unit_quaternion())))
        vb = np.ascontiguousarray(mg.transform(vb, rng.uniform(0.5, 1.5), mg.rotation_matrix(rng.unit_quaternion()),
                                               tuple(rng.unit_vector() * rng.uniform(0.2, 1.5))))
        fb = np.ascontiguousarray(fb, dtype=np.uint32)
        for weld in (100000, 100000000):
            ref = port.run(va, fa, vb, fb, weld)
            got = sbg.run_boolean(va, fa, vb, fb, weld, precision)
            bad = compare(ref, got, len(va) + len(vb), weld, strict=True)
            assert not bad, (i, weld, bad, got["stats"])
            failures += int(ref["status"]) == 0
    assert 0 < failures < 120


def _earcut(L, rings):
    f = L.sb_debug_earcut
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                  ctypes.POINTER(ctypes.c_size_t)]
    xy = np.ascontiguousarray(np.concatenate([np.asarray(r, np.float64).reshape(-1, 2) for r in rings]))
    off = np.zeros(len(rings) + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(r) for r in rings])
    n = ctypes.c_size_t(0)
    r = f(xy.ctypes.data, off.ctypes.data, len(rings), None, 0, ctypes.byref(n))
    assert r == sbg.SB_OK, L.sb_last_error()
    out = np.zeros(max(n.value, 1), dtype=np.int64)
    r = f(xy.ctypes.data, off.ctypes.data, len(rings), out.ctypes.data, len(out), ctypes.byref(n))
    assert r == sbg.SB_OK, L.sb_last_error()
    return out[:n.value]


def test_device_earcut_reference_fixtures(gpu_lib):
    g = np.load(os.path.join(GOLDEN, "earcut_reference_fixtures.npz"))
    xy, ro, po, idx, io, names = g["xy"], g["ring_off"], g["poly_off"], g["idx"], g["idx_off"], g["names"]
    hashed = 0
    for p in range(len(names)):
        rings = [xy[ro[r]:ro[r + 1]] for r in range(po[p], po[p + 1])]
        npts = sum(len(r) for r in rings)
        if npts > 1500:
            continue
        got = _earcut(gpu_lib, rings)
        assert np.array_equal(got, idx[io[p]:io[p + 1]]), str(names[p])
        hashed += npts > 80
    assert hashed >= 13


def test_device_earcut_random_polygons(gpu_lib):
    g = np.load(os.path.join(GOLDEN, "earcut_random.npz"))
    xy, ro, po, idx, io = g["xy"], g["ring_off"], g["poly_off"], g["idx"], g["idx_off"]
    for p in range(len(po) - 1):
        rings = [xy[ro[r]:ro[r + 1]] for r in range(po[p], po[p + 1])]
        assert np.array_equal(_earcut(gpu_lib, rings), idx[io[p]:io[p + 1]]), p


def test_out_of_range_triangle_is_rejected(gpu_lib):
    """A triangle index at or past the vertex count is an argument error (SB_ERR_INVALID), from the host and
    the device variant alike; nothing is left allocated or pending."""
    import ctypes
    torch = pytest.importorskip("torch")
    L = sbg.lib()
    v, f = mg.icosphere(1)
    bad = np.ascontiguousarray(f, dtype=np.uint32).copy()
    bad[7, 1] = len(v)  # one past the last vertex
    v = np.ascontiguousarray(v)
    h = ctypes.c_void_p()
    assert L.sb_mesh_create(v.ctypes.data, len(v), bad.ctypes.data, len(bad), ctypes.byref(h)) == sbg.SB_ERR_INVALID
    assert not h.value
    dv = torch.from_numpy(v).cuda()
    dt = torch.from_numpy(bad.astype(np.int32)).cuda()
    opts = sbg.make_options()
    assert L.sb_mesh_create_device(dv.data_ptr(), len(v), dt.data_ptr(), len(bad), ctypes.byref(opts),
                                   ctypes.byref(h)) == sbg.SB_ERR_INVALID
    assert not h.value
    # a valid mesh still works afterwards
    good = np.ascontiguousarray(f, dtype=np.uint32)
    assert L.sb_mesh_create(v.ctypes.data, len(v), good.ctypes.data, len(good), ctypes.byref(h)) == sbg.SB_OK
    L.sb_mesh_destroy(h)
