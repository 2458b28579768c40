"""GPU: the batched entry point (sb_batch_combine) against single booleans through sb_combine, whose
parity with the oracle the other GPU tests establish, and its statuses against the oracle."""
import numpy as np
import pytest

import solidboolean_gb300 as sbg
from solidboolean_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _oriented_set(t):
    """triangles rotated to start at their smallest index (winding kept), sorted"""
    t = np.asarray(t, dtype=np.int64).reshape(-1, 3)
    if len(t) == 0:
        return t
    r = np.argmin(t, axis=1)
    t = np.take_along_axis(t, (r[:, None] + np.arange(3)[None, :]) % 3, axis=1)
    return t[np.lexsort((t[:, 2], t[:, 1], t[:, 0]))]


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


def test_batch_full_arrays_match_oracle_on_workload_sample(gpu_lib, port):
    """The batched workload itself (4,096 pairs, seed 1234): 98 pairs sampled across it go through one
    sb_batch_combine call, and each pair's result vertices (bit for bit, the reference's numbering) and the
    triangles of its operation (the same oriented triangles; the reference lists them group by group in flood
    order, this library in arrangement order) equal the oracle's; statuses agree on every sampled pair,
    failing ones included."""
    pairs = mg.batch(4096, 1234, 5)
    sample = [pairs[i] for i in range(0, 4096, 42)]
    statuses, results = sbg.batch_combine(sample, workers=8)
    ok = 0
    for k, (va, fa, vb, fb, op) in enumerate(sample):
        ref = port.run(va, fa, vb, fb, 100000)
        assert (statuses[k] == sbg.SB_OK) == (ref["status"] == 1), k
        if ref["status"] != 1:
            continue
        xyz, tris = results[k]
        assert np.array_equal(xyz.view(np.uint64), np.asarray(ref["newv"]).view(np.uint64)), k
        assert np.array_equal(_oriented_set(tris), _oriented_set(np.asarray(ref[op]))), k
        ok += 1
    assert ok >= 64
