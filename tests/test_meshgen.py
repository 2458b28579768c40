"""CPU: the seeded workload generator."""
import hashlib

import numpy as np
import pytest

from solidboolean_gb300 import meshgen as mg


@pytest.mark.parametrize("level", [0, 1, 3, 5])
def test_icosphere_counts_and_closed(level):
    v, f = mg.icosphere(level)
    assert len(v) == 10 * 4 ** level + 2 and len(f) == 20 * 4 ** level
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]).astype(np.int64)
    d = e[:, 0] * len(v) + e[:, 1]
    tw = e[:, 1] * len(v) + e[:, 0]
    assert len(np.unique(d)) == len(d)          # no repeated half-edge
    assert np.isin(tw, d).all()                  # every half-edge has its twin: closed 2-manifold
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0, atol=1e-15)


def test_generator_is_deterministic():
    a = mg.pair_large(1234, 4)
    b = mg.pair_large(1234, 4)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    h = hashlib.sha256(np.ascontiguousarray(a[2]).tobytes()).hexdigest()
    assert len(h) == 64


def test_batch_pairs_cover_levels_and_ops():
    pairs = mg.batch(64, 1234)
    levels = {len(p[1]) for p in pairs} | {len(p[3]) for p in pairs}
    ops = {p[4] for p in pairs}
    assert ops == {"union", "intersect", "diff"}
    assert {80, 320, 1280, 5120, 20480} <= levels


def test_normal_offsets_statistics():
    _, _, vb, _, off = mg.diff_volume(1234, 4)
    assert off.shape == vb.shape
    assert abs(off.std() - 0.01) < 5e-4 and abs(off.mean()) < 5e-4
