"""GPU: the batched entry point (sb_batch_combine) against single booleans through sb_combine, whose
parity with the oracle the other GPU tests establish, and its statuses against the oracle."""
import numpy as np
import pytest

import solidboolean_gb300 as sbg
from solidboolean_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _pairs(n, seed, max_level):
    rng = mg.SplitMix64(seed)
    return [mg.batch_pair(rng, max_level) for _ in range(n)]


@pytest.mark.parametrize("workers", [1, 6])
def test_batch_matches_single_booleans(gpu_lib, workers):
    pairs = _pairs(40, 2024, 4)
    statuses, results = sbg.batch_combine(pairs, workers=workers)
    for i, (va, fa, vb, fb, op) in enumerate(pairs):
        single = sbg.run_boolean(va, fa, vb, fb, 100000)
        assert (statuses[i] == sbg.SB_OK) == (single["status"] == 1), i
        if statuses[i] != sbg.SB_OK:
            assert len(results[i][1]) == 0
            continue
        xyz, tris = results[i]
        assert np.array_equal(xyz, single["newv"]), i
        assert np.array_equal(tris.astype(np.int64), single[op]), i


def test_batch_statuses_match_oracle(gpu_lib, port):
    pairs = _pairs(24, 77, 5)
    statuses, _ = sbg.batch_combine(pairs, keep=False, workers=8)
    for i, (va, fa, vb, fb, op) in enumerate(pairs):
        ref = port.run(va, fa, vb, fb, 100000)
        assert (statuses[i] == sbg.SB_OK) == (ref["status"] == 1), i
