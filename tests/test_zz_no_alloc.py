"""The allocation-free face re-triangulation entry point against the regular path.

sb_retriangulate_faces_noalloc serves callers that cannot allocate device memory (a framework that owns all
device memory through its own pool, real-time loops where an allocation could stall): its workspace is a
static device array in the library.
This test feeds it the cut faces of a boolean computed by the regular entry points (sb_combine), twice in
a row, and checks that both calls return the same triangles, and that those triangles, mapped to result
vertex ids, are exactly the re-triangulated part of the regular arrangement. The file sorts last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import solidboolean_gb300 as sbg
from solidboolean_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

WELD = 100000


def _bind(L):
    f = L.sb_retriangulate_faces_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                  ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p]
    return f


def _faces_from_combine(va, fa, vb, fb):
    opts = sbg.make_options(WELD, "filtered", "reference")
    a, b = sbg.SolidMesh(opts), sbg.SolidMesh(opts)
    a.setVertices(va), a.setTriangles(fa), b.setVertices(vb), b.setTriangles(fb)
    a.prepare(), b.prepare()
    x = sbg.SolidBoolean(a, b, opts)
    assert x.combine()
    pairs = x.dump("intersection_pairs", np.uint32, 2).astype(np.int64)
    segs = x.dump("intersection_segments", np.float64, 6)
    ra = x.dump("rank_first", np.int32, 1)
    rb = x.dump("rank_second", np.int32, 1)
    # each face sees its pairs in the other mesh's reference leaf order, as inside sb_combine
    oa = np.lexsort((rb[pairs[:, 1]], pairs[:, 0]))
    ob = np.lexsort((ra[pairs[:, 0]], pairs[:, 1]))
    faces, corners, seg_list, begin = [], [], [], [0]
    for side, order, col, V, F in ((0, oa, 0, va, fa), (1, ob, 1, vb, fb)):
        ids = pairs[order, col]
        starts = np.flatnonzero(np.r_[True, ids[1:] != ids[:-1]])
        ends = np.r_[starts[1:], len(ids)]
        for s0, e0 in zip(starts, ends):
            t = int(ids[s0])
            faces.append((side, t))
            corners.append(V[F[t]].reshape(-1))
            seg_list.append(segs[order[s0:e0]])
            begin.append(begin[-1] + (e0 - s0))
    return x, faces, np.array(corners), np.concatenate(seg_list), np.array(begin, dtype=np.int32)


def test_noalloc_matches_combine_twice(gpu_lib):
    import torch
    L = gpu_lib
    fn = _bind(L)
    va, fa, vb, fb = mg.pair_small(1234)
    x, faces, corners, segs, begin = _faces_from_combine(va, fa, vb, fb)
    nf, ns, cap = len(faces), len(segs), 64
    dev = torch.device("cuda", 0)
    d_corners = torch.from_numpy(np.ascontiguousarray(corners)).to(dev)
    d_begin = torch.from_numpy(begin).to(dev)
    d_segs = torch.from_numpy(np.ascontiguousarray(segs)).to(dev)
    outs, frees = [], []
    for _ in range(2):
        d_tris = torch.full((nf * cap * 3,), -7, dtype=torch.int32, device=dev)
        d_tc = torch.zeros(nf, dtype=torch.int32, device=dev)
        d_pts = torch.zeros(2 * ns * 3, dtype=torch.float64, device=dev)
        d_pc = torch.zeros(nf, dtype=torch.int32, device=dev)
        d_st = torch.full((nf,), -1, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(dev)[0]
        r = fn(d_corners.data_ptr(), d_begin.data_ptr(), d_segs.data_ptr(), nf, ns, WELD, d_tris.data_ptr(), cap,
               d_tc.data_ptr(), d_pts.data_ptr(), d_pc.data_ptr(), d_st.data_ptr(), None)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(dev)[0]
        assert r == sbg.SB_OK, L.sb_last_error()
        frees.append((free_before, free_after))
        outs.append([t.cpu().numpy() for t in (d_tris, d_tc, d_pts, d_pc, d_st)])
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    # the second call (its kernels already loaded by the first) leaves the device's free memory unchanged
    assert frees[1][0] == frees[1][1], frees
    tris, tc, pts, pc, st = outs[0]
    assert (st == 0).all()

    # map local ids to result-vertex ids and compare with the re-triangulated part of the arrangement
    rv = x.resultVertices()
    n_orig = len(va) + len(vb)
    newkeys = {tuple(k): n_orig + i for i, k in enumerate(np.trunc(rv[n_orig:] * WELD).astype(np.int64))}
    got = []
    for f, (side, t) in enumerate(faces):
        F = fa if side == 0 else fb
        base = 0 if side == 0 else len(va)
        local = tris[f * cap * 3:(f * cap + tc[f]) * 3].reshape(-1, 3)
        for tri in local:
            g = []
            for l in tri:
                if l < 3:
                    g.append(int(F[t][l]) + base)
                else:
                    p = pts[(2 * begin[f] + l - 3) * 3:(2 * begin[f] + l - 2) * 3]
                    k = tuple(np.trunc(p * WELD).astype(np.int64))
                    q = newkeys[k]
                    assert np.allclose(p, rv[q], rtol=1e-12, atol=0)
                    g.append(q)
            got.append(g)
    got = np.array(got, dtype=np.int64)
    arr = x.dump("arrangement", np.uint32, 3).astype(np.int64)
    st_ = x.stats
    n_uncut = (len(fa) - st_.cut_faces_first) + (len(fb) - st_.cut_faces_second)
    want = arr[n_uncut:]

    def canon(t):
        r = np.argmin(t, axis=1)
        t = np.take_along_axis(t, (r[:, None] + np.arange(3)[None, :]) % 3, axis=1)
        return t[np.lexsort((t[:, 2], t[:, 1], t[:, 0]))]

    assert got.shape == want.shape
    assert np.array_equal(canon(got), canon(want))


def test_noalloc_rejects_oversized_request(gpu_lib):
    """More faces than the static workspace can describe: rejected with a clear error, nothing launched."""
    import torch
    L = gpu_lib
    fn = _bind(L)
    dev = torch.device("cuda", 0)
    small = torch.zeros(16, dtype=torch.float64, device=dev)
    ismall = torch.zeros(16, dtype=torch.int32, device=dev)
    r = fn(small.data_ptr(), ismall.data_ptr(), small.data_ptr(), 20_000_000, 1, WELD, ismall.data_ptr(), 1,
           ismall.data_ptr(), small.data_ptr(), ismall.data_ptr(), ismall.data_ptr(), None)
    assert r == sbg.SB_ERR_CAPACITY
    assert b"64 MiB" in L.sb_last_error()
