"""CPU: the C ABI library builds for sm_103a, loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    from solidboolean_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    header = open(os.path.join(ROOT, "include", "solidboolean_gb300.h")).read()
    header = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    names = sorted(set(re.findall(r"\b(sb_[a-z0-9_]+)\s*\(", header)))
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_without_device():
    import solidboolean_gb300 as sbg
    L = sbg.lib()
    assert L.sb_status_string(0) == b"ok"
    assert b"attach" in L.sb_status_string(1)
    o = sbg.Options()
    L.sb_default_options(ctypes.byref(o))
    assert o.weld_factor == 100000 and o.precision == 0 and o.order == 0


def test_python_mirror_has_reference_names():
    import solidboolean_gb300 as sbg
    for cls, names in ((sbg.SolidMesh, ["setVertices", "setTriangles", "prepare"]),
                       (sbg.SolidBoolean, ["combine", "fetchUnion", "fetchDiff", "fetchIntersect",
                                           "resultVertices"])):
        for n in names:
            assert callable(getattr(cls, n))
