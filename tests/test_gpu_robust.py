"""GPU: the robustness mode (sb_options.robust, include/solidboolean_gb300.h sb_robust).

With flags 0 every result is the reference's (all other parity tests). With flags set, the CUDA path must
equal the robust mode's checker (the oracle's sbo_run_robust, same rules) element by element, the combines the
reference fails must go through, and their results must be closed and volume-consistent. The pairs are from
the batched workload (mg.batch, seed 1234) where the reference fails at its weld factor 1e5."""
import numpy as np
import pytest

import solidboolean_gb300 as sbg
from solidboolean_gb300 import meshgen as mg
from parity import compare
from robust_props import check_closed_and_volumes

pytestmark = pytest.mark.gpu

FAILING = [3, 62, 122, 136, 154, 172, 273, 288]


@pytest.fixture(scope="module")
def pairs():
    return mg.batch(300, 1234, 5)


@pytest.mark.parametrize("i", FAILING)
@pytest.mark.parametrize("precision", ["filtered", "fp64"])
def test_robust_equals_its_checker(gpu_lib, port, pairs, i, precision):
    va, fa, vb, fb, _ = pairs[i]
    plain = sbg.run_boolean(va, fa, vb, fb, 100000, precision)
    assert plain["code"] in (sbg.SB_FAIL_ATTACH, sbg.SB_FAIL_LINK, sbg.SB_FAIL_LOOP)
    ref = port.run(va, fa, vb, fb, 100000, robust=sbg.SB_ROBUST_ALL)
    got = sbg.run_boolean(va, fa, vb, fb, 100000, precision, robust=sbg.SB_ROBUST_ALL)
    st = got["stats"]
    assert got["code"] == sbg.SB_OK and ref["status"] == 1
    assert st["attempts"] == int(ref["attempts"][0])
    assert st["weld_factor_used"] == int(ref["weld_factor_used"][0])
    assert st["robust"] == sbg.SB_ROBUST_ALL
    bad = compare(ref, got, len(va) + len(vb), st["weld_factor_used"], strict=True)
    assert not bad, bad
    assert not check_closed_and_volumes(va, fa, vb, fb, got["newv"], got)


@pytest.mark.parametrize("flags", [sbg.SB_ROBUST_EDGE_TOLERANCE, sbg.SB_ROBUST_WELD_RETRY])
def test_single_flags_equal_their_checker(gpu_lib, port, pairs, flags):
    for i in FAILING:
        va, fa, vb, fb, _ = pairs[i]
        ref = port.run(va, fa, vb, fb, 100000, robust=flags)
        got = sbg.run_boolean(va, fa, vb, fb, 100000, robust=flags)
        assert (got["code"] == sbg.SB_OK) == (ref["status"] == 1), i
        assert got["stats"]["attempts"] == int(ref["attempts"][0]), i
        assert got["stats"]["weld_factor_used"] == int(ref["weld_factor_used"][0]), i
        bad = compare(ref, got, len(va) + len(vb), got["stats"]["weld_factor_used"], strict=True)
        assert not bad, (i, bad)


def test_robust_on_succeeding_pairs_equals_its_checker(gpu_lib, port):
    """Where the reference succeeds the robust mode's results follow the same rules (strict against its
    checker); the bound is looser, so they may differ from the reference's in principle."""
    for va, fa, vb, fb in (mg.pair_small(1234), mg.pair_large(1234, 5)):
        ref = port.run(va, fa, vb, fb, 100000, robust=sbg.SB_ROBUST_ALL)
        got = sbg.run_boolean(va, fa, vb, fb, 100000, robust=sbg.SB_ROBUST_ALL)
        bad = compare(ref, got, len(va) + len(vb), got["stats"]["weld_factor_used"], strict=True)
        assert not bad, bad


def test_batch_robust_removes_failures(gpu_lib):
    """The batch API with the robust flags on the first 1,024 pairs of the batched workload: the reference's
    parity mode fails 32 of them (status parity is tested elsewhere); the robust mode fails none, and every
    result is closed."""
    pairs = mg.batch(1024, 1234, 5)
    plain, _ = sbg.batch_combine(pairs, keep=False)
    st, res = sbg.batch_combine(pairs, robust=sbg.SB_ROBUST_ALL)
    assert int(np.count_nonzero(plain != sbg.SB_OK)) == 32
    assert int(np.count_nonzero(st != sbg.SB_OK)) == 0
    from robust_props import open_edges
    for k in np.nonzero(plain != sbg.SB_OK)[0]:
        xyz, tris = res[k]
        assert open_edges(tris) == 0, k
