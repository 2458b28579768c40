"""CPU: the robustness mode's checker (the oracle with sb_robust flags, oracle/sb_oracle.cpp sbo_run_robust).

Pairs of the batched workload (mg.batch, seed 1234) on which the reference fails at its weld factor 1e5: on
these the reference's point-on-edge test (an absolute bound of one epsilon, src/vector2.h:212-215) rejects cut
points that lie on the edge up to rounding, or its quantum merges distinct cut points. With both robust flags
every one of them combines, and the results are closed and volume-consistent."""
import ctypes

import numpy as np
import pytest

from solidboolean_gb300 import meshgen as mg
from robust_props import check_closed_and_volumes

# indices into mg.batch(seed 1234) where the reference fails at weld factor 1e5 (first 300 pairs)
FAILING = [3, 62, 122, 136, 154, 172, 273, 288]


@pytest.fixture(scope="module")
def pairs():
    return mg.batch(300, 1234, 5)


@pytest.mark.parametrize("i", FAILING)
def test_robust_mode_combines_where_the_reference_fails(port, pairs, i):
    va, fa, vb, fb, _ = pairs[i]
    ref = port.run(va, fa, vb, fb, 100000)
    assert ref["status"] == 0
    r = port.run(va, fa, vb, fb, 100000, robust=3)
    assert r["status"] == 1
    assert int(r["attempts"][0]) >= 1 and int(r["weld_factor_used"][0]) >= 100000
    bad = check_closed_and_volumes(va, fa, vb, fb, r["newv"], r)
    assert not bad, bad


def test_robust_flags_zero_is_the_reference(port, pairs):
    va, fa, vb, fb, _ = pairs[0]
    a = port.run(va, fa, vb, fb, 100000)
    b = port.run(va, fa, vb, fb, 100000, robust=0)
    for k in ("status", "newt", "union", "diff", "intersect"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


# the two causes, one flag each: (status with the edge bound only, status with the weld retry only,
# weld factor the retry ends at)
CAUSES = {3: (0, 1, 1000000), 62: (1, 0, 10 ** 12), 122: (0, 1, 1000000), 136: (1, 0, 10 ** 12),
          154: (1, 0, 10 ** 12), 172: (1, 0, 10 ** 12), 273: (0, 1, 1000000), 288: (1, 0, 10 ** 12)}


@pytest.mark.parametrize("i", FAILING)
def test_each_flag_alone(port, pairs, i):
    """Some pairs fail only because of the absolute point-on-edge bound (no quantum helps: the retry runs up
    to 1e12 and gives up), others only because the quantum merges cut points (one step finer suffices)."""
    va, fa, vb, fb, _ = pairs[i]
    e = port.run(va, fa, vb, fb, 100000, robust=1)
    w = port.run(va, fa, vb, fb, 100000, robust=2)
    assert (e["status"], w["status"], int(w["weld_factor_used"][0])) == CAUSES[i]
    assert int(e["attempts"][0]) == 1


def test_options_layout_matches_header():
    import solidboolean_gb300 as sbg
    assert ctypes.sizeof(sbg.Options) == 32
    assert sbg.Options.robust.offset == 24
    assert sbg.Stats.weld_factor_used.offset % 8 == 0
    import pathlib, re
    h = (pathlib.Path(__file__).resolve().parents[1] / "include" / "solidboolean_gb300.h").read_text()
    assert re.search(r"SB_ROBUST_EDGE_TOLERANCE\s*=\s*1\b", h) and re.search(r"SB_ROBUST_WELD_RETRY\s*=\s*2\b", h)
    assert sbg.SB_ROBUST_EDGE_TOLERANCE == 1 and sbg.SB_ROBUST_WELD_RETRY == 2
