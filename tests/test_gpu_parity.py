"""GPU results against the oracle restatement of the reference path, through the C ABI.

Strict parity: besides the canonical comparisons, the result vertices (ids and bit-exact coordinates), the
arrangement's triangles in the reference's m_newTriangles order and every triangle's label equal the
oracle's element by element."""
import numpy as np
import pytest

import solidboolean_gb300 as sbg
from solidboolean_gb300 import meshgen as mg
from parity import compare

pytestmark = pytest.mark.gpu

CASES = {
    "pair_small": lambda: mg.pair_small(1234),
    "pair_small_s7": lambda: mg.pair_small(7),
    "near_tangent_L4": lambda: mg.near_tangent(1234, level=4),
    "pair_large_L4": lambda: mg.pair_large(1234, level=4),
    "diff_volume_L3": lambda: mg.diff_volume(1234, level=3)[:4],
    # meshes that hold a directed edge twice: the grouping cannot use the input adjacency and hashes every
    # half-edge of the arrangement, as the reference does
    "pair_small_flipped_triangle": lambda: _flipped(mg.pair_small(1234), 5),
    "pair_small_repeated_triangle": lambda: _repeated(mg.pair_small(1234), 7),
}


def _flipped(pair, i):
    va, fa, vb, fb = pair
    fa = fa.copy()
    fa[i] = fa[i][::-1]
    return va, fa, vb, fb


def _repeated(pair, i):
    va, fa, vb, fb = pair
    return va, np.vstack([fa, fa[i:i + 1]]), vb, fb


@pytest.mark.parametrize("precision", ["filtered", "fp64"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_parity(gpu_lib, port, case, precision):
    va, fa, vb, fb = CASES[case]()
    ref = port.run(va, fa, vb, fb, 100000)
    got = sbg.run_boolean(va, fa, vb, fb, 100000, precision)
    bad = compare(ref, got, len(va) + len(vb), 100000, strict=True)
    assert not bad, (case, precision, bad, got["stats"])
    assert got["stats"]["order_fallbacks"] == 0


@pytest.mark.parametrize("case", ["pair_small", "pair_large_L5", "near_tangent_L5", "batch"])
def test_reference_leaf_order(gpu_lib, port, case):
    """The GPU-built leaf order of the reference tree equals the oracle's, triangle for triangle."""
    if case == "pair_small":
        va, fa, vb, fb = mg.pair_small(1234)
    elif case == "pair_large_L5":
        va, fa, vb, fb = mg.pair_large(1234, level=5)
    elif case == "near_tangent_L5":
        va, fa, vb, fb = mg.near_tangent(1234, level=5)
    else:
        va, fa, vb, fb, _ = mg.batch_pair(mg.SplitMix64(11), 5)
    ref = port.run(va, fa, vb, fb, 100000)
    opts = sbg.make_options(100000, "filtered", "reference")
    a, b = sbg.SolidMesh(opts), sbg.SolidMesh(opts)
    a.setVertices(va), a.setTriangles(fa), b.setVertices(vb), b.setTriangles(fb)
    a.prepare(), b.prepare()
    x = sbg.SolidBoolean(a, b, opts)
    x.combine()
    for side in ("a", "b"):
        rank = x.dump("rank_first" if side == "a" else "rank_second", np.int32, 1)
        order = np.empty_like(rank)
        order[rank] = np.arange(len(rank), dtype=np.int32)
        assert np.array_equal(order, ref[f"leaforder_{side}"].astype(np.int32)), side
