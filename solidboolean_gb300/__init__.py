"""GB300 mesh boolean: Python mirror of the reference's SolidMesh / SolidBoolean interface over the C ABI.

    a = SolidMesh(); a.setVertices(va); a.setTriangles(fa); a.prepare()       # src/solidmesh.h:33-61
    sb = SolidBoolean(a, b)                                                     # src/solidboolean.h:36-37
    ok = sb.combine()                                                           # src/solidboolean.h:39
    tris = []; sb.fetchUnion(tris); sb.fetchDiff(tris); sb.fetchIntersect(tris) # src/solidboolean.h:40-42
    verts = sb.resultVertices()                                                 # src/solidboolean.h:44

As in the reference, the fetch calls append to the list they are given, combine() returns False when the
reference would, and all three results index into resultVertices(). Everything runs on the GPU through
libsolidboolean_gb300.so; there is no CPU fallback: importing works anywhere, but creating a mesh without
the built library or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes
import weakref
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsolidboolean_gb300.so")

SB_OK, SB_FAIL_ATTACH, SB_FAIL_LINK, SB_FAIL_LOOP = 0, 1, 2, 3
SB_ERR_INVALID, SB_ERR_CUDA, SB_ERR_CAPACITY, SB_ERR_NOT_COMBINED = 10, 11, 12, 13
SB_UNION, SB_DIFF, SB_INTERSECT = 0, 1, 2
SB_STAGED_VERTICES = 3  # sb_take_staged: the result vertices
PRECISION = {"filtered": 0, "fp64": 1}
ORDER = {"reference": 0, "index": 1}
# sb_robust flags (include/solidboolean_gb300.h): 0 keeps the reference's behaviour
SB_ROBUST_EDGE_TOLERANCE, SB_ROBUST_WELD_RETRY = 1, 2
SB_ROBUST_ALL = SB_ROBUST_EDGE_TOLERANCE | SB_ROBUST_WELD_RETRY

EXPORTS = ["sb_default_options", "sb_status_string", "sb_last_error", "sb_kernel_launches", "sb_mesh_create",
           "sb_mesh_create_device",
           "sb_mesh_update_vertices_device", "sb_mesh_prepare", "sb_mesh_destroy", "sb_boolean_create",
           "sb_combine", "sb_fetch", "sb_result_vertices", "sb_fetch_device", "sb_result_vertices_device",
           "sb_debug_dump", "sb_boolean_destroy", "sb_host_alloc", "sb_host_free", "sb_take_staged"]


class Options(ctypes.Structure):
    _fields_ = [("weld_factor", ctypes.c_int64), ("precision", ctypes.c_int32), ("order", ctypes.c_int32),
                ("stream", ctypes.c_void_p), ("robust", ctypes.c_uint32), ("stage_results", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("candidate_pairs", ctypes.c_uint64), ("intersecting_pairs", ctypes.c_uint64),
                ("cut_faces_first", ctypes.c_uint64), ("cut_faces_second", ctypes.c_uint64),
                ("new_points", ctypes.c_uint64), ("result_vertices", ctypes.c_uint64),
                ("result_triangles", ctypes.c_uint64), ("sign_tests", ctypes.c_uint64),
                ("sign_fallbacks", ctypes.c_uint64), ("box_tests", ctypes.c_uint64),
                ("box_fallbacks", ctypes.c_uint64), ("regions_first", ctypes.c_uint32),
                ("regions_second", ctypes.c_uint32), ("failed_faces", ctypes.c_uint32),
                ("loop_vertices", ctypes.c_uint32), ("loop_bad_degree", ctypes.c_uint32),
                ("duplicate_halfedges", ctypes.c_uint32), ("loops", ctypes.c_uint32),
                ("order_fallbacks", ctypes.c_uint32), ("attempts", ctypes.c_uint32), ("robust", ctypes.c_uint32),
                ("weld_factor_used", ctypes.c_int64), ("stage_ms", ctypes.c_double * 8)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "stage_ms"}
        d["stage_ms"] = list(self.stage_ms)
        return d


_lib = None


def lib() -> ctypes.CDLL:
    """Loads the built library (raises when it is missing: there is no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built; run solidboolean_gb300.build.build() first")
    L = ctypes.CDLL(LIB_PATH)
    vp, sz, st = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    L.sb_default_options.argtypes = [ctypes.POINTER(Options)]
    L.sb_status_string.restype = ctypes.c_char_p
    L.sb_status_string.argtypes = [st]
    L.sb_last_error.restype = ctypes.c_char_p
    L.sb_kernel_launches.restype = ctypes.c_uint64
    L.sb_mesh_create.restype = st
    L.sb_mesh_create.argtypes = [vp, sz, vp, sz, ctypes.POINTER(vp)]
    L.sb_mesh_create_device.restype = st
    L.sb_mesh_create_device.argtypes = [vp, sz, vp, sz, ctypes.POINTER(Options), ctypes.POINTER(vp)]
    L.sb_mesh_update_vertices_device.restype = st
    L.sb_mesh_update_vertices_device.argtypes = [vp, vp, ctypes.POINTER(Options)]
    L.sb_mesh_prepare.restype = st
    L.sb_mesh_prepare.argtypes = [vp, ctypes.POINTER(Options)]
    L.sb_mesh_destroy.argtypes = [vp]
    L.sb_boolean_create.restype = st
    L.sb_boolean_create.argtypes = [vp, vp, ctypes.POINTER(Options), ctypes.POINTER(vp)]
    L.sb_combine.restype = st
    L.sb_combine.argtypes = [vp, ctypes.POINTER(Stats)]
    L.sb_fetch.restype = st
    L.sb_fetch.argtypes = [vp, st, vp, sz, ctypes.POINTER(sz)]
    L.sb_fetch_device.restype = st
    L.sb_fetch_device.argtypes = [vp, st, ctypes.POINTER(vp), ctypes.POINTER(sz)]
    L.sb_result_vertices.restype = st
    L.sb_result_vertices.argtypes = [vp, vp, sz, ctypes.POINTER(sz)]
    L.sb_result_vertices_device.restype = st
    L.sb_result_vertices_device.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(sz)]
    L.sb_debug_dump.restype = st
    L.sb_debug_dump.argtypes = [vp, ctypes.c_char_p, vp, sz, ctypes.POINTER(sz)]
    L.sb_boolean_destroy.argtypes = [vp]
    L.sb_batch_combine.restype = st
    L.sb_batch_combine.argtypes = [sz, vp, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.POINTER(Options), ctypes.c_int32,
                                   vp, ctypes.POINTER(vp)]
    L.sb_batch_result_size.restype = st
    L.sb_batch_result_size.argtypes = [vp, sz, ctypes.POINTER(sz), ctypes.POINTER(sz)]
    L.sb_batch_result.restype = st
    L.sb_batch_result.argtypes = [vp, sz, vp, vp]
    L.sb_batch_destroy.argtypes = [vp]
    L.sb_host_alloc.restype = st
    L.sb_host_alloc.argtypes = [sz, ctypes.POINTER(vp)]
    L.sb_host_free.restype = None
    L.sb_host_free.argtypes = [vp]
    L.sb_take_staged.restype = st
    L.sb_take_staged.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(vp), ctypes.POINTER(sz)]
    L.sb_adjoint.restype = st
    L.sb_adjoint.argtypes = [vp, vp, vp, vp, vp]
    _lib = L
    return L


class SolidBooleanError(RuntimeError):
    pass


def _check(code: int, what: str) -> int:
    if code in (SB_OK, SB_FAIL_ATTACH, SB_FAIL_LINK, SB_FAIL_LOOP):
        return code
    L = lib()
    raise SolidBooleanError(f"{what}: {L.sb_status_string(code).decode()} ({L.sb_last_error().decode()})")


def make_options(weld_factor: int = 100000, precision: str = "filtered", order: str = "reference",
                 stream: int | None = None, robust: int = 0, stage_results: bool = False) -> Options:
    o = Options()
    lib().sb_default_options(ctypes.byref(o))
    o.weld_factor = int(weld_factor)
    o.precision = PRECISION[precision]
    o.order = ORDER[order]
    o.stream = stream or None
    o.robust = int(robust)
    o.stage_results = 1 if stage_results else 0
    return o


class SolidMesh:
    """src/solidmesh.h: non-owning in the reference; here setVertices/setTriangles take copies."""

    def __init__(self, options: Options | None = None):
        self._v = None
        self._t = None
        self._h = ctypes.c_void_p()
        self.options = options

    def setVertices(self, vertices) -> None:
        self._v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        self._release()

    def setTriangles(self, triangles) -> None:
        self._t = np.ascontiguousarray(triangles, dtype=np.uint32).reshape(-1, 3)
        self._release()

    def vertices(self):
        return self._v

    def triangles(self):
        return self._t

    def _release(self):
        if self._h:
            lib().sb_mesh_destroy(self._h)
            self._h = ctypes.c_void_p()

    def handle(self) -> ctypes.c_void_p:
        if not self._h:
            v = self._v if self._v is not None else np.zeros((0, 3))
            t = self._t if self._t is not None else np.zeros((0, 3), dtype=np.uint32)
            _check(lib().sb_mesh_create(v.ctypes.data, len(v), t.ctypes.data, len(t), ctypes.byref(self._h)),
                   "sb_mesh_create")
        return self._h

    def prepare(self) -> None:
        opts = self.options or make_options()
        _check(lib().sb_mesh_prepare(self.handle(), ctypes.byref(opts)), "sb_mesh_prepare")

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass


def _host_array(rows: int, cols: int, dtype) -> np.ndarray:
    """A result array in page-locked memory from the library's cache (returned to it when the array is
    collected), so result reads run at DMA speed; plain numpy memory when none can be had."""
    nbytes = rows * cols * np.dtype(dtype).itemsize
    if nbytes == 0:
        return np.zeros((rows, cols), dtype=dtype)
    L = lib()
    ptr = ctypes.c_void_p()
    if L.sb_host_alloc(nbytes, ctypes.byref(ptr)) != SB_OK or not ptr.value:
        return np.zeros((rows, cols), dtype=dtype)
    raw = (ctypes.c_char * nbytes).from_address(ptr.value)
    weakref.finalize(raw, L.sb_host_free, ptr.value)
    return np.frombuffer(raw, dtype=dtype).reshape(rows, cols)


class SolidBoolean:
    """src/solidboolean.h:33-58"""

    def __init__(self, first: SolidMesh, second: SolidMesh, options: Options | None = None):
        self.first, self.second = first, second
        # results are read on the host here: combine() stages them in page-locked memory (sb_take_staged)
        self.options = Options.from_buffer_copy(options) if options is not None else make_options()
        self.options.stage_results = 1
        self._h = ctypes.c_void_p()
        self.status = None
        self.stats = Stats()

    def _handle(self):
        if not self._h:
            _check(lib().sb_boolean_create(self.first.handle(), self.second.handle(), ctypes.byref(self.options),
                                           ctypes.byref(self._h)), "sb_boolean_create")
        return self._h

    def combine(self) -> bool:
        self.status = _check(lib().sb_combine(self._handle(), ctypes.byref(self.stats)), "sb_combine")
        return self.status == SB_OK

    def _take_staged(self, what: int, cols: int, dtype) -> np.ndarray | None:
        """The result combine() staged in page-locked host memory, handed over (None when not staged)."""
        L = lib()
        ptr, n = ctypes.c_void_p(), ctypes.c_size_t()
        _check(L.sb_take_staged(self._handle(), what, ctypes.byref(ptr), ctypes.byref(n)), "sb_take_staged")
        if n.value == 0:
            if ptr.value:
                L.sb_host_free(ptr.value)
            return np.zeros((0, cols), dtype=dtype)
        if not ptr.value:
            return None
        nbytes = n.value * cols * np.dtype(dtype).itemsize
        raw = (ctypes.c_char * nbytes).from_address(ptr.value)
        weakref.finalize(raw, L.sb_host_free, ptr.value)
        return np.frombuffer(raw, dtype=dtype).reshape(n.value, cols)

    def _fetch(self, op: int) -> np.ndarray:
        staged = self._take_staged(op, 3, np.uint32)
        if staged is not None:
            return staged
        L = lib()
        n = ctypes.c_size_t()
        _check(L.sb_fetch(self._handle(), op, None, 0, ctypes.byref(n)), "sb_fetch")
        out = _host_array(n.value, 3, np.uint32)
        if n.value:
            _check(L.sb_fetch(self._handle(), op, out.ctypes.data, n.value, ctypes.byref(n)), "sb_fetch")
        return out

    def fetch(self, op: str) -> np.ndarray:
        return self._fetch({"union": SB_UNION, "diff": SB_DIFF, "intersect": SB_INTERSECT}[op])

    def fetchUnion(self, resultTriangles: list) -> None:
        resultTriangles.extend(self._fetch(SB_UNION).tolist())

    def fetchDiff(self, resultTriangles: list) -> None:
        resultTriangles.extend(self._fetch(SB_DIFF).tolist())

    def fetchIntersect(self, resultTriangles: list) -> None:
        resultTriangles.extend(self._fetch(SB_INTERSECT).tolist())

    def resultVertices(self) -> np.ndarray:
        staged = self._take_staged(SB_STAGED_VERTICES, 3, np.float64)
        if staged is not None:
            return staged
        L = lib()
        n = ctypes.c_size_t()
        _check(L.sb_result_vertices(self._handle(), None, 0, ctypes.byref(n)), "sb_result_vertices")
        out = _host_array(n.value, 3, np.float64)
        if n.value:
            _check(L.sb_result_vertices(self._handle(), out.ctypes.data, n.value, ctypes.byref(n)),
                   "sb_result_vertices")
        return out

    def dump(self, name: str, dtype, cols: int) -> np.ndarray:
        L = lib()
        nbytes = ctypes.c_size_t()
        _check(L.sb_debug_dump(self._handle(), name.encode(), None, 0, ctypes.byref(nbytes)), "sb_debug_dump")
        out = np.zeros(nbytes.value // np.dtype(dtype).itemsize, dtype=dtype)
        if nbytes.value:
            _check(L.sb_debug_dump(self._handle(), name.encode(), out.ctypes.data, nbytes.value,
                                   ctypes.byref(nbytes)), "sb_debug_dump")
        return out.reshape(-1, cols) if cols > 1 else out

    def __del__(self):
        try:
            if self._h:
                lib().sb_boolean_destroy(self._h)
        except Exception:
            pass


def run_boolean(va, fa, vb, fb, weld_factor: int = 100000, precision: str = "filtered",
                order: str = "reference", robust: int = 0) -> dict:
    """One boolean with every result and stage dump copied to the host (used by tests and smoke)."""
    opts = make_options(weld_factor, precision, order, robust=robust)
    a = SolidMesh(opts)
    a.setVertices(va)
    a.setTriangles(fa)
    b = SolidMesh(opts)
    b.setVertices(vb)
    b.setTriangles(fb)
    a.prepare()
    b.prepare()
    sb = SolidBoolean(a, b, opts)
    ok = sb.combine()
    out = {"status": 1 if ok else 0, "code": sb.status, "stats": sb.stats.as_dict(),
           "cand": sb.dump("candidates", np.uint32, 2).astype(np.int64),
           "isect_pairs": sb.dump("intersection_pairs", np.uint32, 2).astype(np.int64),
           "isect_segs": sb.dump("intersection_segments", np.float64, 6),
           "newv": sb.resultVertices(),
           "newt": sb.dump("arrangement", np.uint32, 3).astype(np.int64),
           "labels": sb.dump("labels", np.int8, 1),
           "tri_mesh": sb.dump("tri_mesh", np.int8, 1)}
    for op in ("union", "diff", "intersect"):
        out[op] = sb.fetch(op).astype(np.int64)
    return out


OP_CODES = {"union": SB_UNION, "diff": SB_DIFF, "intersect": SB_INTERSECT}


def batch_combine(pairs, weld_factor: int = 100000, precision: str = "filtered", order: str = "reference",
                  workers: int = 0, keep: bool = True, robust: int = 0):
    """Many independent booleans in one call (sb_batch_combine). pairs: sequence of (va, fa, vb, fb, op) with
    op in "union" / "diff" / "intersect". Returns (statuses, results): statuses an int32 array of per-pair
    sb_combine codes; results (when keep) a list of (result vertices, the op's triangles) per pair, empty
    arrays for pairs that did not combine."""
    L = lib()
    n = len(pairs)

    def csr(items, width, dtype):
        off = np.zeros(n + 1, dtype=np.uint64)
        for i, x in enumerate(items):
            off[i + 1] = off[i] + len(x)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(x, dtype=dtype).reshape(-1, width) for x in items])
                                    if n else np.zeros((0, width), dtype=dtype))
        return flat, off

    va, vao = csr([p[0] for p in pairs], 3, np.float64)
    ta, tao = csr([p[1] for p in pairs], 3, np.uint32)
    vb, vbo = csr([p[2] for p in pairs], 3, np.float64)
    tb, tbo = csr([p[3] for p in pairs], 3, np.uint32)
    ops = np.array([OP_CODES[p[4]] for p in pairs], dtype=np.int32)
    statuses = np.zeros(n, dtype=np.int32)
    opts = make_options(weld_factor, precision, order, robust=robust)
    handle = ctypes.c_void_p()
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    code = L.sb_batch_combine(n, ptr(va), ptr(vao), ptr(ta), ptr(tao), ptr(vb), ptr(vbo), ptr(tb), ptr(tbo),
                              ptr(ops), ctypes.byref(opts), workers, ptr(statuses),
                              ctypes.byref(handle) if keep else None)
    _check(code, "sb_batch_combine")
    results = None
    if keep:
        results = []
        try:
            for i in range(n):
                nv, nt = ctypes.c_size_t(), ctypes.c_size_t()
                _check(L.sb_batch_result_size(handle, i, ctypes.byref(nv), ctypes.byref(nt)), "sb_batch_result_size")
                xyz = np.empty((nv.value, 3), dtype=np.float64)
                tris = np.empty((nt.value, 3), dtype=np.uint32)
                _check(L.sb_batch_result(handle, i, ptr(xyz), ptr(tris)), "sb_batch_result")
                results.append((xyz, tris))
        finally:
            L.sb_batch_destroy(handle)
    return statuses, results
