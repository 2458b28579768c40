"""Parity on the benchmark-sized workloads and on sampled pairs of the batched workload (mixed
subdivision levels, so faces with closed inner loops and failing pairs occur)."""
import numpy as np
import pytest

import solidboolean_gb300 as sbg
from solidboolean_gb300 import meshgen as mg
from parity import compare

pytestmark = pytest.mark.gpu


def _check(port, va, fa, vb, fb, q, precision="filtered"):
    ref = port.run(va, fa, vb, fb, q)
    got = sbg.run_boolean(va, fa, vb, fb, q, precision)
    bad = compare(ref, got, len(va) + len(vb), q, strict=True)
    assert not bad, (bad, got["stats"])
    assert got["stats"]["order_fallbacks"] == 0
    return ref, got


def test_pair_large_L7_fine_weld(gpu_lib, port):
    """327,680 x 327,680 triangles at weld factor 1e8: the full pipeline, bit-exact."""
    va, fa, vb, fb = mg.pair_large(1234, 7)
    ref, got = _check(port, va, fa, vb, fb, 100000000)
    assert ref["status"] == 1


def test_pair_large_L7_reference_weld_fails_like_reference(gpu_lib, port):
    """At the reference's default weld factor the reference fails on this workload; so must we, with the
    same candidate and intersecting pairs."""
    va, fa, vb, fb = mg.pair_large(1234, 7)
    ref, got = _check(port, va, fa, vb, fb, 100000)
    assert ref["status"] == 0 and got["code"] in (sbg.SB_FAIL_ATTACH, sbg.SB_FAIL_LINK, sbg.SB_FAIL_LOOP)


def test_near_tangent_L6(gpu_lib, port):
    va, fa, vb, fb = mg.near_tangent(1234, 6)
    _check(port, va, fa, vb, fb, 100000)


@pytest.mark.parametrize("weld", [100000, 100000000])
def test_diff_volume_L5_with_offsets(gpu_lib, port, weld):
    """A leaky arrangement (the cut loops do not close every region, so some flood regions hold groups the
    reference decides differently): labels follow the reference's first-in-first-out flood in the
    iteration order of its hash containers, triangle for triangle."""
    va, fa, vb, fb, off = mg.diff_volume(1234, 5)
    ref, got = _check(port, va, fa, vb + off, fb, weld)
    assert ref["status"] == 1 and got["stats"]["loops"] > 1


@pytest.mark.parametrize("precision", ["filtered", "fp64"])
def test_batch_sample(gpu_lib, port, precision):
    rng = mg.SplitMix64(99)
    fails = 0
    for i in range(24):
        va, fa, vb, fb, _ = mg.batch_pair(rng, 5)
        ref, got = _check(port, va, fa, vb, fb, 100000, precision)
        fails += ref["status"] == 0


@pytest.mark.parametrize("name", ["pair_large_L7_weld1e8", "pair_large_L7_weld1e5", "near_tangent_L6",
                                  "diff_volume_L5_offsets", "diff_volume_L5_offsets_weld1e8"])
def test_headline_reference_digests(gpu_lib, name):
    """The CUDA path against digests of the compiled reference's own arrays (not only against the port):
    candidate and intersecting pairs, segments, and for a successful combine the result vertices and the
    arrangement in the reference's order, the labels and the three results."""
    from test_golden_headline import META, headline_inputs, load_table
    from parity import digests, input_digest
    want = load_table()[name]
    va, fa, vb, fb = headline_inputs(name)
    assert input_digest(va, fa, vb, fb) == want["inputs"]
    got = sbg.run_boolean(va, fa, vb, fb, want["quantum"])
    assert digests(got, len(va) + len(vb), want["quantum"]) == {k: v for k, v in want.items() if k not in META}


@pytest.mark.parametrize("level", [5, 6])
def test_interpenetrating_many_cut_faces(gpu_lib, port, level):
    """Two jittered unit spheres crossing each other everywhere: 15.7 k (level 5) and 63 k (level 6) cut faces
    per mesh, tens of thousands of small loops. Past 8,192 faces per mesh the faces are sorted device-wide,
    past 65,536 faces the face layout is scanned device-wide, and the loop order's work arrays leave shared
    memory. Strict at weld factor 1e8; at 1e5 the reference fails and so must the library."""
    va, fa, vb, fb = mg.interpenetrating(7, level)
    ref, got = _check(port, va, fa, vb, fb, 100000000)
    assert ref["status"] == 1 and got["stats"]["cut_faces_first"] > 8192
    ref, got = _check(port, va, fa, vb, fb, 100000)
    assert ref["status"] == 0 and got["code"] in (sbg.SB_FAIL_ATTACH, sbg.SB_FAIL_LINK, sbg.SB_FAIL_LOOP)
