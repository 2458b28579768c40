"""CPU: the oracle restatement pinned to the reference on the benchmark-sized workloads.

tests/golden/headline_digests.json holds digests of the compiled reference's stage arrays (made by
`python tests/golden/make_golden.py --headline`): the icosphere L7 pair at weld factors 1e8 (full pipeline)
and 1e5 (where the reference fails: status, candidate and intersecting pairs), the near-tangent L6 pair and
the leaky L5 pair with offsets. The restatement must reproduce every digest; where the reference sources are
present it is also compared with the compiled reference array by array.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle
from parity import digests, input_digest
from solidboolean_gb300 import meshgen as mg

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "headline_digests.json")
META = ("quantum", "inputs", "candidates_count", "triangles_count")


def headline_inputs(name):
    if name.startswith("pair_large_L7"):
        return mg.pair_large(1234, 7)
    if name == "near_tangent_L6":
        return mg.near_tangent(1234, 6)
    va, fa, vb, fb, off = mg.diff_volume(1234, 5)
    return va, fa, vb + off, fb


def load_table():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.mark.parametrize("name", sorted(load_table()))
def test_port_matches_reference_digests(port, name):
    want = load_table()[name]
    va, fa, vb, fb = headline_inputs(name)
    assert input_digest(va, fa, vb, fb) == want["inputs"], "the generator no longer reproduces the inputs"
    d = port.run(va, fa, vb, fb, want["quantum"])
    got = digests(d, len(va) + len(vb), want["quantum"])
    assert got == {k: v for k, v in want.items() if k not in META}
    assert len(d["cand"]) == want["candidates_count"]
    ref = oracle.reference()
    if ref is not None and name in ("pair_large_L7_weld1e8", "pair_large_L7_weld1e5", "near_tangent_L6"):
        r = ref.run(va, fa, vb, fb, want["quantum"])
        for k in ("status", "cand", "isect", "seg", "newv", "newt", "groups_a_off", "groups_a", "groups_b_off",
                  "groups_b", "sides_a", "sides_b", "union", "diff", "intersect", "leaforder_a", "leaforder_b"):
            x, y = np.asarray(r[k]), np.asarray(d[k])
            assert x.shape == y.shape and np.array_equal(x, y, equal_nan=x.dtype.kind == "f"), k


def test_port_matches_reference_meshes_digests(port):
    """The reference's own test meshes (tests/golden/reference_meshes.npz): the restatement reproduces the
    compiled reference's digests at both weld factors."""
    g = np.load(os.path.join(os.path.dirname(GOLDEN), "reference_meshes.npz"))
    with open(os.path.join(os.path.dirname(GOLDEN), "reference_meshes_digests.json")) as f:
        table = json.load(f)
    for key, want in table.items():
        name = key.split(":")[0]
        va, fa, vb, fb = (g[f"{name}:{x}"] for x in ("va", "fa", "vb", "fb"))
        assert input_digest(va, fa, vb, fb) == want["inputs"]
        d = port.run(va, fa, vb, fb, want["quantum"])
        assert digests(d, len(va) + len(vb), want["quantum"]) == {k: v for k, v in want.items()
                                                                  if k not in ("inputs", "quantum")}, key


def test_port_earcut_matches_reference_fixture_file(port):
    """The reference's earcut fixtures with the reference's indices (tests/golden/earcut_reference_fixtures.npz)."""
    g = np.load(os.path.join(os.path.dirname(GOLDEN), "earcut_reference_fixtures.npz"))
    xy, ro, po, idx, io = g["xy"], g["ring_off"], g["poly_off"], g["idx"], g["idx_off"]
    for p in range(len(po) - 1):
        rings = [xy[ro[r]:ro[r + 1]] for r in range(po[p], po[p + 1])]
        assert np.array_equal(port.earcut(rings), idx[io[p]:io[p + 1]]), str(g["names"][p])
