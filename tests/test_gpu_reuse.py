"""GPU: one prepared mesh reused by several booleans (the reference's SolidMesh is prepared once and may be
combined with many others, src/solidmesh.cpp:42-76, src/solidboolean.h:36-37), with preparation and combines
on different streams; every result must equal the oracle's (strict parity) and a boolean of freshly created
meshes."""
import ctypes

import numpy as np
import pytest

import solidboolean_gb300 as sbg
from solidboolean_gb300 import meshgen as mg
from parity import compare

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

WELD = 100000000


def _device_mesh(L, v, t, opts):
    dev = torch.device("cuda", 0)
    dv = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
    dt = torch.from_numpy(np.ascontiguousarray(t.astype(np.int32))).to(dev)
    h = ctypes.c_void_p()
    sbg._check(L.sb_mesh_create_device(dv.data_ptr(), len(v), dt.data_ptr(), len(t), ctypes.byref(opts),
                                       ctypes.byref(h)), "sb_mesh_create_device")
    torch.cuda.synchronize()
    return h, (dv, dt)


def _results(L, x):
    out = {}
    for name, op in (("union", sbg.SB_UNION), ("diff", sbg.SB_DIFF), ("intersect", sbg.SB_INTERSECT)):
        n = ctypes.c_size_t()
        sbg._check(L.sb_fetch(x, op, None, 0, ctypes.byref(n)), "sb_fetch")
        a = np.zeros((n.value, 3), dtype=np.uint32)
        if n.value:
            sbg._check(L.sb_fetch(x, op, a.ctypes.data, n.value, ctypes.byref(n)), "sb_fetch")
        out[name] = a.astype(np.int64)
    n = ctypes.c_size_t()
    sbg._check(L.sb_result_vertices(x, None, 0, ctypes.byref(n)), "sb_result_vertices")
    v = np.zeros((n.value, 3), dtype=np.float64)
    if n.value:
        sbg._check(L.sb_result_vertices(x, v.ctypes.data, n.value, ctypes.byref(n)), "sb_result_vertices")
    out["newv"] = v

    def dump(name, dtype, cols):
        nb = ctypes.c_size_t()
        sbg._check(L.sb_debug_dump(x, name.encode(), None, 0, ctypes.byref(nb)), "sb_debug_dump")
        a = np.zeros(nb.value // np.dtype(dtype).itemsize, dtype=dtype)
        if nb.value:
            sbg._check(L.sb_debug_dump(x, name.encode(), a.ctypes.data, nb.value, ctypes.byref(nb)), "sb_debug_dump")
        return a.reshape(-1, cols) if cols > 1 else a
    out["cand"] = dump("candidates", np.uint32, 2).astype(np.int64)
    out["isect_pairs"] = dump("intersection_pairs", np.uint32, 2).astype(np.int64)
    out["isect_segs"] = dump("intersection_segments", np.float64, 6)
    out["newt"] = dump("arrangement", np.uint32, 3).astype(np.int64)
    out["labels"] = dump("labels", np.int8, 1)
    return out


def test_prepared_mesh_reused_across_booleans_and_streams(gpu_lib, port):
    L = sbg.lib()
    va, fa, vb, fb = mg.pair_large(1234, 5)
    rng = mg.SplitMix64(99)
    seconds = [(vb, fb)]
    for _ in range(2):
        v2, f2 = mg.icosphere(4)
        v2 = mg.transform(v2, 0.7, mg.rotation_matrix(rng.unit_quaternion()), (0.5, -0.2, 0.1))
        seconds.append((np.ascontiguousarray(v2), f2))

    s_prep = torch.cuda.Stream()
    o_prep = sbg.make_options(WELD, "filtered", "reference", s_prep.cuda_stream)
    hA, keepA = _device_mesh(L, va, fa, o_prep)
    sbg._check(L.sb_mesh_prepare(hA, ctypes.byref(o_prep)), "sb_mesh_prepare A")  # returns before the build ends

    handles = []
    try:
        for k, (v2, f2) in enumerate(seconds):
            s_k = torch.cuda.Stream()  # every combine on its own stream, none on the preparation stream
            o_k = sbg.make_options(WELD, "filtered", "reference", s_k.cuda_stream)
            hB, keepB = _device_mesh(L, v2, f2, o_k)
            x = ctypes.c_void_p()
            sbg._check(L.sb_boolean_create(hA, hB, ctypes.byref(o_k), ctypes.byref(x)), "sb_boolean_create")
            handles.append((x, hB, keepB))
            st = sbg.Stats()
            code = L.sb_combine(x, ctypes.byref(st))
            fresh = sbg.run_boolean(va, fa, v2, f2, WELD)
            ref = port.run(va, fa, v2, f2, WELD)
            assert (code == sbg.SB_OK) == (fresh["status"] == 1) == (ref["status"] == 1), k
            if code != sbg.SB_OK:
                continue
            got = _results(L, x)
            got["status"] = 1
            bad = compare(ref, got, len(va) + len(v2), WELD, strict=True)
            assert not bad, (k, bad)
            assert np.array_equal(got["newv"], fresh["newv"]), k
            for name in ("union", "diff", "intersect"):
                assert np.array_equal(got[name], fresh[name]), (k, name)
    finally:
        for x, hB, _ in handles:
            L.sb_boolean_destroy(x)
            L.sb_mesh_destroy(hB)
        L.sb_mesh_destroy(hA)
