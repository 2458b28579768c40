"""GPU: results staged in page-locked host memory by combine() (sb_options.stage_results, sb_take_staged) are
the same arrays the device copies return (sb_fetch, sb_result_vertices), each is handed over once, and with
staging off nothing is staged."""
import ctypes

import numpy as np
import pytest

import solidboolean_gb300 as sbg
from solidboolean_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

OPS = (("union", sbg.SB_UNION), ("diff", sbg.SB_DIFF), ("intersect", sbg.SB_INTERSECT))


def _device_copies(L, h):
    out = {}
    for name, op in OPS:
        n = ctypes.c_size_t()
        sbg._check(L.sb_fetch(h, op, None, 0, ctypes.byref(n)), "sb_fetch")
        a = np.zeros((n.value, 3), dtype=np.uint32)
        if n.value:
            sbg._check(L.sb_fetch(h, op, a.ctypes.data, n.value, ctypes.byref(n)), "sb_fetch")
        out[name] = a
    n = ctypes.c_size_t()
    sbg._check(L.sb_result_vertices(h, None, 0, ctypes.byref(n)), "sb_result_vertices")
    v = np.zeros((n.value, 3), dtype=np.float64)
    sbg._check(L.sb_result_vertices(h, v.ctypes.data, n.value, ctypes.byref(n)), "sb_result_vertices")
    out["vertices"] = v
    return out


@pytest.mark.parametrize("weld", [100000, 100000000])
def test_staged_results_equal_device_copies(gpu_lib, weld):
    L = gpu_lib
    va, fa, vb, fb = mg.pair_small(1234)
    opts = sbg.make_options(weld, "filtered", "reference")
    a = sbg.SolidMesh(opts)
    a.setVertices(va)
    a.setTriangles(fa)
    b = sbg.SolidMesh(opts)
    b.setVertices(vb)
    b.setTriangles(fb)
    x = sbg.SolidBoolean(a, b, opts)  # the Python class turns staging on
    assert x.options.stage_results == 1 and opts.stage_results == 0
    assert x.combine()
    staged = {name: x.fetch(name) for name, _ in OPS}
    staged["vertices"] = x.resultVertices()
    ref = _device_copies(L, x._handle())
    for k in ref:
        assert staged[k].shape == ref[k].shape and staged[k].size > 0, k
        assert np.array_equal(staged[k], ref[k]), k
    # each staged buffer is handed over once; afterwards nothing is staged and the device copy serves
    for what in (sbg.SB_UNION, sbg.SB_DIFF, sbg.SB_INTERSECT, sbg.SB_STAGED_VERTICES):
        ptr, n = ctypes.c_void_p(), ctypes.c_size_t()
        sbg._check(L.sb_take_staged(x._handle(), what, ctypes.byref(ptr), ctypes.byref(n)), "sb_take_staged")
        assert not ptr.value and n.value > 0
    assert np.array_equal(x.fetch("union"), ref["union"])
    assert np.array_equal(x.resultVertices(), ref["vertices"])
    # a second combine stages afresh (and releases what was not taken)
    assert x.combine()
    assert np.array_equal(x.fetch("diff"), ref["diff"])


def test_nothing_staged_without_the_option(gpu_lib):
    L = gpu_lib
    va, fa, vb, fb = mg.pair_small(1234)
    opts = sbg.make_options(100000000, "filtered", "reference")
    ha, hb, hx = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    for v, t, h in ((va, fa, ha), (vb, fb, hb)):
        v = np.ascontiguousarray(v, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.uint32)
        sbg._check(L.sb_mesh_create(v.ctypes.data, len(v), t.ctypes.data, len(t), ctypes.byref(h)), "create")
    try:
        sbg._check(L.sb_boolean_create(ha, hb, ctypes.byref(opts), ctypes.byref(hx)), "boolean")
        ptr, n = ctypes.c_void_p(), ctypes.c_size_t()
        assert L.sb_take_staged(hx, sbg.SB_UNION, ctypes.byref(ptr), ctypes.byref(n)) == sbg.SB_ERR_NOT_COMBINED
        assert sbg._check(L.sb_combine(hx, None), "combine") == sbg.SB_OK
        for what in (sbg.SB_UNION, sbg.SB_DIFF, sbg.SB_INTERSECT, sbg.SB_STAGED_VERTICES):
            sbg._check(L.sb_take_staged(hx, what, ctypes.byref(ptr), ctypes.byref(n)), "sb_take_staged")
            assert not ptr.value and n.value > 0
        assert L.sb_take_staged(hx, 4, ctypes.byref(ptr), ctypes.byref(n)) == sbg.SB_ERR_INVALID
    finally:
        if hx:
            L.sb_boolean_destroy(hx)
        L.sb_mesh_destroy(ha)
        L.sb_mesh_destroy(hb)
