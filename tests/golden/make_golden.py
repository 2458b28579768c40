"""Generates the golden fixtures from the reference itself (oracle/_ref, compiled from the reference
sources by oracle/Makefile). Run here, where the reference sources exist:

    python tests/golden/make_golden.py             # small fixtures with full arrays, earcut fixtures
    python tests/golden/make_golden.py --headline  # digests of the benchmark-sized workloads
    python tests/golden/make_golden.py --cases     # the reference's test meshes and earcut fixtures

Each fixture stores the input meshes (so no generator drift can hide a change) and the reference's dumps.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from solidboolean_gb300 import meshgen as mg  # noqa: E402

KEEP = ["cand", "isect", "seg", "newv", "newt", "groups_a_off", "groups_a", "groups_b_off", "groups_b",
        "sides_a", "sides_b", "union", "diff", "intersect", "leaforder_a", "leaforder_b"]


def cases():
    yield "pair_small_1234", mg.pair_small(1234), 100000
    yield "near_tangent_L3", mg.near_tangent(1234, level=3), 100000
    va, fa, vb, fb, off = mg.diff_volume(1234, level=3)
    yield "diff_volume_L3_offsets", (va, fa, vb + off, fb), 100000
    rng = mg.SplitMix64(7)
    picked = {}
    for i in range(200):
        va, fa, vb, fb, _ = mg.batch_pair(rng, 3)
        if len(fa) + len(fb) > 3000:
            continue
        ref = oracle.reference().run(va, fa, vb, fb, 100000)
        key = "ok" if ref["status"] else "fail"
        if key not in picked:
            picked[key] = (va, fa, vb, fb)
        if len(picked) == 2:
            break
    for key, m in picked.items():
        yield f"batch_pair_{key}", m, 100000


def headline_cases():
    """The benchmark-sized workloads, pinned by digests (their full arrays are tens of megabytes)."""
    yield "pair_large_L7_weld1e8", lambda: mg.pair_large(1234, 7), 100000000
    yield "pair_large_L7_weld1e5", lambda: mg.pair_large(1234, 7), 100000
    yield "near_tangent_L6", lambda: mg.near_tangent(1234, 6), 100000

    def dv():
        va, fa, vb, fb, off = mg.diff_volume(1234, 5)
        return va, fa, vb + off, fb
    yield "diff_volume_L5_offsets", dv, 100000
    yield "diff_volume_L5_offsets_weld1e8", dv, 100000000


def make_headline(ref):
    import json
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from parity import digests, input_digest
    table = {}
    for name, gen, q in headline_cases():
        va, fa, vb, fb = gen()
        d = ref.run(va, fa, vb, fb, q)
        table[name] = {"quantum": q, "inputs": input_digest(va, fa, vb, fb), "candidates_count": len(d["cand"]),
                       "triangles_count": len(d["newt"]), **digests(d, len(va) + len(vb), q)}
        print(name, "status", d["status"], "candidates", len(d["cand"]), "triangles", len(d["newt"]))
    with open(os.path.join(HERE, "headline_digests.json"), "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)


def earcut_fixture_polygons():
    """The reference's earcut fixtures (thirdparty/earcut.hpp/test/fixtures/*.cpp), read from its test files."""
    import glob
    import re
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


def make_cases(ref):
    """The reference's own test meshes (test/cases/*/{a,b}.obj, read like its test driver reads them) with
    digests of the reference's results at both weld factors, and its earcut fixtures with the reference's
    triangle indices."""
    import glob
    import json
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from parity import digests, input_digest
    from solidboolean_gb300 import objio
    arrays, table = {}, {}
    root = os.path.join(oracle.REF_ROOT, "test", "cases")
    for d in sorted(glob.glob(os.path.join(root, "*"))):
        name = os.path.basename(d)
        a, b = os.path.join(d, "a.obj"), os.path.join(d, "b.obj")
        if not (os.path.isfile(a) and os.path.isfile(b)):
            continue
        va, fa = objio.load_obj(a)
        vb, fb = objio.load_obj(b)
        arrays.update({f"{name}:va": va, f"{name}:fa": fa, f"{name}:vb": vb, f"{name}:fb": fb})
        for q in (100000, 100000000):
            r = ref.run(va, fa, vb, fb, q)
            table[f"{name}:{q}"] = {"inputs": input_digest(va, fa, vb, fb), "quantum": q,
                                    **digests(r, len(va) + len(vb), q)}
            print(name, q, "status", r["status"], "triangles", len(r["newt"]))
    np.savez_compressed(os.path.join(HERE, "reference_meshes.npz"), **arrays)
    with open(os.path.join(HERE, "reference_meshes_digests.json"), "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    xy, ring_off, poly_off, idx, idx_off, names = [], [0], [0], [], [0], []
    for name, rings in earcut_fixture_polygons():
        for r in rings:
            xy.append(r)
            ring_off.append(ring_off[-1] + len(r))
        poly_off.append(poly_off[-1] + len(rings))
        ix = ref.earcut(rings)
        idx.append(ix)
        idx_off.append(idx_off[-1] + len(ix))
        names.append(name)
    np.savez_compressed(os.path.join(HERE, "earcut_reference_fixtures.npz"), xy=np.concatenate(xy),
                        ring_off=np.array(ring_off), poly_off=np.array(poly_off), idx=np.concatenate(idx),
                        idx_off=np.array(idx_off), names=np.array(names))
    print("earcut fixtures", len(names))


def main():
    ref = oracle.reference()
    assert ref is not None, "the reference sources are needed to generate golden fixtures"
    if "--headline" in sys.argv:
        make_headline(ref)
        return
    if "--cases" in sys.argv:
        make_cases(ref)
        return
    for name, (va, fa, vb, fb), q in cases():
        d = ref.run(va, fa, vb, fb, q)
        out = {k: d[k] for k in KEEP}
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), va=va, fa=fa, vb=vb, fb=fb, quantum=q,
                            status=d["status"], **out)
        print(name, "status", d["status"], "candidates", len(d["cand"]), "triangles", len(d["newt"]))
    # earcut: random star polygons with holes, reference indices
    rng = np.random.default_rng(5)
    polys = []
    for i in range(40):
        n = int(rng.integers(3, 120))
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        rad = rng.uniform(0.5, 1.0, n)
        outer = np.stack([rad * np.cos(ang), rad * np.sin(ang)], 1)
        rings = [outer]
        for h in range(int(rng.integers(0, 3))):
            m = int(rng.integers(3, 8))
            a = np.sort(rng.uniform(0, 2 * np.pi, m))
            c = rng.uniform(-0.15, 0.15, 2)
            rings.append(np.stack([c[0] + 0.1 * np.cos(a), c[1] + 0.1 * np.sin(a)], 1))
        polys.append(rings)
    flat, offs, per, idx_all, idx_off = [], [0], [0], [], [0]
    for rings in polys:
        for r in rings:
            flat.append(r)
            offs.append(offs[-1] + len(r))
        per.append(per[-1] + len(rings))
        idx = ref.earcut(rings)
        idx_all.append(idx)
        idx_off.append(idx_off[-1] + len(idx))
    np.savez_compressed(os.path.join(HERE, "earcut_random.npz"), xy=np.concatenate(flat), ring_off=np.array(offs),
                        poly_off=np.array(per), idx=np.concatenate(idx_all), idx_off=np.array(idx_off))
    print("earcut fixtures", len(polys))


if __name__ == "__main__":
    main()
