"""ctypes loader for the two CPU checkers (test infrastructure only; the product never imports this).

  port()       -> our C++ restatement of the reference path (oracle/sb_oracle.cpp), built by `make port`
  reference()  -> the reference's own sources compiled here (oracle/_ref/libsbref.so), built by `make ref`;
                  only available where the reference sources exist (None elsewhere)
  obj_reference() -> the reference test driver's OBJ loader (oracle/_ref/libobjref.so, `make objref`), a
                  function path -> (vertices, triangles); None where the reference sources are absent

Both return a Checker whose run() gives a dict of numpy arrays named as in oracle/sb_oracle.h.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libsb_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsbref.so")
# the reference sources: $SB_REFERENCE_ROOT, else a checkout named "reference" beside this repository
REF_ROOT = os.environ.get("SB_REFERENCE_ROOT") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))

_NAMES_I64 = ["status", "cand", "isect", "newt", "groups_a_off", "groups_a", "groups_b_off", "groups_b",
              "sides_a", "sides_b", "union", "diff", "intersect", "leaforder_a", "leaforder_b", "ctx_a", "ctx_b",
              "loops_a_off", "loops_a", "tri_ranges", "attempts", "weld_factor_used"]
_NAMES_F64 = ["seg", "newv", "time_ms"]
_SHAPES = {"cand": (-1, 2), "seg": (-1, 6), "newv": (-1, 3), "newt": (-1, 3), "union": (-1, 3),
           "diff": (-1, 3), "intersect": (-1, 3)}


def build(target: str = "port") -> None:
    subprocess.check_call(["make", "-s", "-C", HERE, target, f"REF_ROOT={REF_ROOT}"])


class Checker:
    def __init__(self, path: str):
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.sbo_run.restype = ctypes.c_void_p
        L.sbo_run.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                              ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                              ctypes.c_long]
        L.sbo_len.restype = ctypes.c_long
        L.sbo_len.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.sbo_get_i64.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        L.sbo_get_f64.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        L.sbo_free.argtypes = [ctypes.c_void_p]
        L.sbo_earcut.restype = ctypes.c_long
        L.sbo_earcut.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p,
                                 ctypes.c_long]
        L.sbo_tritri.restype = ctypes.c_int
        L.sbo_tritri.argtypes = [ctypes.c_void_p] * 6 + [ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]

    def run(self, va, fa, vb, fb, quantum: int = 100000, robust: int = 0) -> dict:
        """One boolean. robust: the robust mode's flags (sb_robust; the restatement only, which checks that
        mode: the reference has none), 0 for the reference's behaviour."""
        va = np.ascontiguousarray(va, dtype=np.float64)
        vb = np.ascontiguousarray(vb, dtype=np.float64)
        fa = np.ascontiguousarray(fa, dtype=np.uint32)
        fb = np.ascontiguousarray(fb, dtype=np.uint32)
        args = (va.ctypes.data, len(va), fa.ctypes.data, len(fa), vb.ctypes.data, len(vb), fb.ctypes.data,
                len(fb), int(quantum))
        if robust:
            f = self.lib.sbo_run_robust
            f.restype = ctypes.c_void_p
            f.argtypes = self.lib.sbo_run.argtypes + [ctypes.c_int]
            h = f(*args, int(robust))
        else:
            h = self.lib.sbo_run(*args)
        out = {}
        try:
            for names, dt, getter in ((_NAMES_I64, np.int64, self.lib.sbo_get_i64),
                                      (_NAMES_F64, np.float64, self.lib.sbo_get_f64)):
                for n in names:
                    ln = self.lib.sbo_len(h, n.encode())
                    if ln < 0:
                        continue
                    arr = np.zeros(ln, dtype=dt)
                    getter(h, n.encode(), arr.ctypes.data)
                    out[n] = arr.reshape(_SHAPES[n]) if n in _SHAPES else arr
        finally:
            self.lib.sbo_free(h)
        out["status"] = int(out["status"][0])
        return out

    def earcut(self, rings) -> np.ndarray:
        xy = np.ascontiguousarray(np.concatenate([np.asarray(r, dtype=np.float64).reshape(-1, 2)
                                                  for r in rings]))
        off = np.zeros(len(rings) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(r) for r in rings])
        cap = max(16, 3 * 3 * len(xy))
        out = np.zeros(cap, dtype=np.int64)
        n = self.lib.sbo_earcut(xy.ctypes.data, off.ctypes.data, len(rings), out.ctypes.data, cap)
        assert n <= cap
        return out[:n].copy()

    def tritri(self, p1, q1, r1, p2, q2, r2):
        args = [np.ascontiguousarray(x, dtype=np.float64) for x in (p1, q1, r1, p2, q2, r2)]
        cop = ctypes.c_int(0)
        seg = np.zeros(6)
        r = self.lib.sbo_tritri(*[a.ctypes.data for a in args], ctypes.byref(cop), seg.ctypes.data)
        return r, cop.value, seg


_cache: dict[str, Checker] = {}


def port() -> Checker:
    if "port" not in _cache:
        build("port")
        _cache["port"] = Checker(PORT_SO)
    return _cache["port"]


def reference() -> Checker | None:
    if "ref" not in _cache:
        if not os.path.isdir(os.path.join(REF_ROOT, "src")):
            return None
        build("ref")
        _cache["ref"] = Checker(REF_SO)
    return _cache["ref"]


def obj_reference():
    if "objref" not in _cache:
        if not os.path.isfile(os.path.join(REF_ROOT, "test", "tiny_obj_loader.h")):
            return None
        build("objref")
        L = ctypes.CDLL(os.path.join(HERE, "_ref", "libobjref.so"))
        L.sbo_obj_load.restype = ctypes.c_int
        L.sbo_obj_load.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p, ctypes.c_long,
                                   ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long)]

        def load(path: str):
            nv, nt = ctypes.c_long(), ctypes.c_long()
            if L.sbo_obj_load(path.encode(), None, 0, None, 0, ctypes.byref(nv), ctypes.byref(nt)) != 0:
                raise RuntimeError(f"tinyobj could not read {path}")
            v = np.zeros((nv.value, 3), dtype=np.float64)
            t = np.zeros((nt.value, 3), dtype=np.uint32)
            L.sbo_obj_load(path.encode(), v.ctypes.data, nv.value, t.ctypes.data, nt.value, ctypes.byref(nv),
                           ctypes.byref(nt))
            return v, t

        _cache["objref"] = load
    return _cache["objref"]
