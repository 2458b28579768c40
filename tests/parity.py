"""Canonical comparison of boolean results (used by the parity tests, smoke() and the bench's self-check).

Vertex ids: the input vertices keep their ids (first mesh, then second mesh). Every appended cut point is
renamed by the rank of its PositionKey (trunc(c * factor) per coordinate), which is unique among the
appended points because the global weld merges equal keys. Triangles are rotated to start at their
smallest canonical id (winding kept) and sorted, so two results are equal iff they contain the same
oriented triangles.
"""
from __future__ import annotations

import numpy as np


def position_keys(xyz: np.ndarray, factor: int) -> np.ndarray:
    k = np.trunc(np.asarray(xyz, dtype=np.float64) * float(factor))
    return k.astype(np.int64)


def canonical_ids(newv: np.ndarray, n_orig: int, factor: int):
    """old id -> canonical id, plus the canonical order of the appended points"""
    new = newv[n_orig:]
    keys = position_keys(new, factor)
    order = np.lexsort((keys[:, 2], keys[:, 1], keys[:, 0])) if len(keys) else np.zeros(0, dtype=np.int64)
    remap = np.arange(len(newv), dtype=np.int64)
    remap[n_orig + order] = n_orig + np.arange(len(order))
    return remap, order


def canonical_tris(tris: np.ndarray, remap: np.ndarray) -> np.ndarray:
    t = remap[np.asarray(tris, dtype=np.int64).reshape(-1, 3)]
    if len(t) == 0:
        return t
    r = np.argmin(t, axis=1)
    idx = (r[:, None] + np.arange(3)[None, :]) % 3
    t = np.take_along_axis(t, idx, axis=1)
    o = np.lexsort((t[:, 2], t[:, 1], t[:, 0]))
    return t[o]


def oracle_labels(d: dict) -> np.ndarray:
    """per-arrangement-triangle label from the reference's groups and sides (-1 = in no group)"""
    lab = np.full(len(d["newt"]), -1, dtype=np.int64)
    for side in ("a", "b"):
        off, idx, sides = d[f"groups_{side}_off"], d[f"groups_{side}"], d[f"sides_{side}"]
        for g in range(len(off) - 1):
            lab[idx[off[g]:off[g + 1]]] = sides[g]
    return lab


def labelled_tris(tris, labels, remap) -> np.ndarray:
    t = canonical_tris(tris, remap)  # sorted; sort labels alongside
    tt = remap[np.asarray(tris, dtype=np.int64).reshape(-1, 3)]
    if len(tt) == 0:
        return np.zeros((0, 4), dtype=np.int64)
    r = np.argmin(tt, axis=1)
    idx = (r[:, None] + np.arange(3)[None, :]) % 3
    tt = np.take_along_axis(tt, idx, axis=1)
    rows = np.concatenate([tt, np.asarray(labels, dtype=np.int64).reshape(-1, 1)], axis=1)
    o = np.lexsort((rows[:, 3], rows[:, 2], rows[:, 1], rows[:, 0]))
    del t
    return rows[o]


def float_bits(x) -> np.ndarray:
    """The bit patterns of float64 values with every NaN written as one NaN. A degenerate construction (an
    all-coplanar pair's segment) gives NaN on both sides, but x86 and the GPU encode the default NaN
    differently (sign and payload); every other value must match bit for bit."""
    y = np.array(x, dtype=np.float64, copy=True)
    y[np.isnan(y)] = np.nan
    return y.view(np.int64)


def sorted_pairs(p: np.ndarray) -> np.ndarray:
    p = np.asarray(p, dtype=np.int64).reshape(-1, 2)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def compare(oracle: dict, gpu: dict, n_orig: int, factor: int, coord_rtol: float = 1e-12,
            check_labels: bool = True, strict: bool = False) -> dict:
    """Returns a dict of named mismatches (empty when the results agree).

    strict: also the reference's own numbering and order, element by element: the result vertices (ids and
    bit-exact coordinates), the arrangement's triangles in m_newTriangles order, and each triangle's label."""
    bad: dict = {}
    if oracle["status"] != gpu["status"]:
        bad["status"] = (oracle["status"], gpu["status"])
    # candidate pairs: same set
    oc, gc = sorted_pairs(oracle["cand"]), sorted_pairs(gpu["cand"])
    if oc.shape != gc.shape or not np.array_equal(oc, gc):
        bad["candidates"] = (len(oc), len(gc))
    # intersecting pairs and their segments, bit-exact
    hit = oracle["isect"].astype(bool)
    op = np.asarray(oracle["cand"]).reshape(-1, 2)[hit]
    osg = np.asarray(oracle["seg"]).reshape(-1, 6)[hit]
    o1 = np.lexsort((op[:, 1], op[:, 0]))
    gp = np.asarray(gpu["isect_pairs"]).reshape(-1, 2)
    gsg = np.asarray(gpu["isect_segs"]).reshape(-1, 6)
    g1 = np.lexsort((gp[:, 1], gp[:, 0]))
    if op.shape != gp.shape or not np.array_equal(op[o1], gp[g1]):
        bad["intersecting_pairs"] = (len(op), len(gp))
    elif not np.array_equal(float_bits(osg[o1]), float_bits(gsg[g1])):
        diff = int(np.count_nonzero(float_bits(osg[o1]) != float_bits(gsg[g1])))
        bad["segments"] = diff
    if oracle["status"] != 1 or gpu["status"] != 1:
        return bad
    ro, order_o = canonical_ids(oracle["newv"], n_orig, factor)
    rg, order_g = canonical_ids(gpu["newv"], n_orig, factor)
    nvo, nvg = len(oracle["newv"]), len(gpu["newv"])
    if nvo != nvg:
        bad["vertex_count"] = (nvo, nvg)
        return bad
    vo = oracle["newv"][n_orig:][order_o]
    vg = gpu["newv"][n_orig:][order_g]
    if not np.array_equal(position_keys(vo, factor), position_keys(vg, factor)):
        bad["point_keys"] = True
        return bad
    if not np.array_equal(oracle["newv"][:n_orig], gpu["newv"][:n_orig]):
        bad["input_vertices"] = True
    err = np.abs(vo - vg) / np.maximum(np.abs(vo), 1e-300)
    err = np.where(vo == vg, 0.0, err)
    if err.size and float(err.max()) > coord_rtol:
        bad["coordinates"] = float(err.max())
    # the arrangement's triangles as a set; what is inside or outside (labels, and the fetched
    # operations built from them) only when asked
    at = canonical_tris(oracle["newt"], ro)
    bt = canonical_tris(gpu["newt"], rg)
    if at.shape != bt.shape or not np.array_equal(at, bt):
        bad["arrangement"] = (len(at), len(bt))
    if check_labels:
        for op_name in ("union", "diff", "intersect"):
            a = canonical_tris(oracle[op_name], ro)
            b = canonical_tris(gpu[op_name], rg)
            if a.shape != b.shape or not np.array_equal(a, b):
                bad[op_name] = (len(a), len(b))
        lo = labelled_tris(oracle["newt"], oracle_labels(oracle), ro)
        lg = labelled_tris(gpu["newt"], gpu["labels"], rg)
        if lo.shape != lg.shape or not np.array_equal(lo, lg):
            bad["labels"] = (len(lo), len(lg))
    if strict:
        ov, gv = np.asarray(oracle["newv"]), np.asarray(gpu["newv"])
        if ov.shape != gv.shape or not np.array_equal(float_bits(ov), float_bits(gv)):
            bad["strict_vertices"] = int(np.count_nonzero(np.any(ov != gv, axis=1))) if ov.shape == gv.shape else -1
        ot, gt = np.asarray(oracle["newt"]).reshape(-1, 3), np.asarray(gpu["newt"]).reshape(-1, 3)
        if ot.shape != gt.shape or not np.array_equal(ot, gt):
            bad["strict_arrangement"] = int(np.count_nonzero(np.any(ot != gt, axis=1))) if ot.shape == gt.shape else -1
        elif check_labels:
            ol = oracle_labels(oracle)
            gl = np.asarray(gpu["labels"]).astype(np.int64)
            if not np.array_equal(ol, gl):
                bad["strict_labels"] = int(np.count_nonzero(ol != gl))
    return bad


def max_coord_error(oracle: dict, gpu: dict, n_orig: int, factor: int) -> float:
    ro, order_o = canonical_ids(oracle["newv"], n_orig, factor)
    rg, order_g = canonical_ids(gpu["newv"], n_orig, factor)
    vo = oracle["newv"][n_orig:][order_o]
    vg = gpu["newv"][n_orig:][order_g]
    if vo.shape != vg.shape or vo.size == 0:
        return 0.0
    err = np.abs(vo - vg) / np.maximum(np.abs(vo), 1e-300)
    return float(np.where(vo == vg, 0.0, err).max())


def _sha(a) -> str:
    import hashlib
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.dtype.str.encode() + str(a.shape).encode() + a.tobytes()).hexdigest()


def input_digest(va, fa, vb, fb) -> str:
    return _sha(np.concatenate([np.asarray(va, np.float64).ravel(), np.asarray(vb, np.float64).ravel()])) + \
        _sha(np.concatenate([np.asarray(fa, np.int64).ravel(), np.asarray(fb, np.int64).ravel()]))[:16]


def digests(d: dict, n_orig: int, factor: int) -> dict:
    """SHA-256 digests of a boolean's stage arrays, from an oracle dump or a GPU result (run_boolean):
    candidate pairs (sorted), intersecting pairs and their segments (sorted by pair), and for a successful
    combine the result vertices and arrangement triangles in the reference's own order, every triangle's
    label, and the three fetch results after canonical ordering."""
    gpu = "isect_pairs" in d
    out = {"status": int(d["status"])}
    out["candidates"] = _sha(sorted_pairs(d["cand"]))
    if gpu:
        ip, sg = np.asarray(d["isect_pairs"]).reshape(-1, 2), np.asarray(d["isect_segs"]).reshape(-1, 6)
    else:
        hit = np.asarray(d["isect"]).astype(bool)
        ip, sg = np.asarray(d["cand"]).reshape(-1, 2)[hit], np.asarray(d["seg"]).reshape(-1, 6)[hit]
    o = np.lexsort((ip[:, 1], ip[:, 0]))
    out["intersecting_pairs"] = _sha(ip[o].astype(np.int64))
    out["segments"] = _sha(float_bits(sg[o]))
    if out["status"] != 1:
        return out
    out["vertices"] = _sha(float_bits(np.asarray(d["newv"], np.float64).reshape(-1, 3)))
    out["arrangement"] = _sha(np.asarray(d["newt"], np.int64).reshape(-1, 3))
    labels = np.asarray(d["labels"], np.int64) if gpu else oracle_labels(d)
    out["labels"] = _sha(labels.astype(np.int64))
    remap, _ = canonical_ids(d["newv"], n_orig, factor)
    for op in ("union", "diff", "intersect"):
        out[op] = _sha(canonical_tris(d[op], remap))
    return out
