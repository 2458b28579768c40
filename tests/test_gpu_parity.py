"""GPU results against the oracle restatement of the reference path, through the C ABI."""
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
}


@pytest.mark.parametrize("precision", ["filtered", "fp64"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_parity(gpu_lib, port, case, precision):
    va, fa, vb, fb = CASES[case]()
    ref = port.run(va, fa, vb, fb, 100000)
    got = sbg.run_boolean(va, fa, vb, fb, 100000, precision)
    bad = compare(ref, got, len(va) + len(vb), 100000)
    assert not bad, (case, precision, bad, got["stats"])
