"""Seeded synthetic closed meshes for the boolean workloads (icospheres, rotations, jitter).

Only +, -, *, / and sqrt are used (all correctly rounded), and the random stream is a self-contained
splitmix64, so the same seed yields bit-identical FP64 buffers on every machine and numpy version.

Workloads (sizes as quoted for the reference path):
  * pair_small   : icosphere L3 (642 v / 1,280 t), r=1 at the origin, and r=0.8 at (0.5, 0.3, 0.2),
                   randomly rotated.
  * pair_large   : icosphere L7 (163,842 v / 327,680 t) x 2, every vertex jittered radially by
                   U(-0.5%, +0.5%) of the radius; B has r=0.9, offset (0.4, 0.1, -0.2), rotated.
  * near_tangent : icosphere L6 x 2, r=1, centre distance 2 - 1e-3 along a random axis, +-1e-7 jitter.
  * batch        : many independent pairs, L ~ U{1..5}, scale U[0.5, 2], random rotations, centre
                   distance U[0.2, 0.9] * (r1 + r2), op ~ U{union, intersection, difference}.
  * diff_volume  : icosphere L5 x 2, r=1 and r=0.85, offset (0.35, 0, 0); B carries N(0, 0.01^2)
                   per-vertex offsets (normal deviates by the sum of 12 uniforms, no transcendental calls).
"""
from __future__ import annotations

import numpy as np

_M64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 stream (Steele, Lea, Flood 2014); uniform doubles use the top 53 bits."""

    def __init__(self, seed: int):
        self.state = seed & _M64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _M64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        u = (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def uniform_array(self, n: int, lo: float, hi: float) -> np.ndarray:
        # vectorised splitmix64 over a counter block, identical to n scalar draws
        base = self.state
        k = np.arange(1, n + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            z = np.uint64(base) + k * np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        self.state = (base + n * 0x9E3779B97F4A7C15) & _M64
        u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def randint(self, lo: int, hi: int) -> int:
        """uniform integer in [lo, hi]"""
        return lo + int(self.uniform() * (hi - lo + 1)) if hi > lo else lo

    def unit_quaternion(self) -> np.ndarray:
        """uniform rotation: rejection-sample the unit 4-ball, then normalise"""
        while True:
            q = np.array([self.uniform(-1.0, 1.0) for _ in range(4)])
            s = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]
            if 1e-6 < s <= 1.0:
                return q / np.sqrt(s)

    def unit_vector(self) -> np.ndarray:
        while True:
            v = np.array([self.uniform(-1.0, 1.0) for _ in range(3)])
            s = v[0] * v[0] + v[1] * v[1] + v[2] * v[2]
            if 1e-6 < s <= 1.0:
                return v / np.sqrt(s)

    def normal_array(self, n: int, sigma: float) -> np.ndarray:
        acc = np.zeros(n)
        for _ in range(12):
            acc = acc + self.uniform_array(n, 0.0, 1.0)
        return (acc - 6.0) * sigma


_PHI = (1.0 + 5.0 ** 0.5) / 2.0
_ICO_V = np.array([
    [-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
    [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
    [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1]], dtype=np.float64)
_ICO_F = np.array([
    [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
    [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
    [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
    [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)


def _normalize_rows(v: np.ndarray) -> np.ndarray:
    n = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    return v / n[:, None]


_ICO_CACHE: dict[int, tuple[np.ndarray, np.ndarray]] = {}


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: 10*4^L + 2 vertices, 20*4^L outward-facing triangles (FP64, uint32)."""
    if level in _ICO_CACHE:
        v, f = _ICO_CACHE[level]
        return v.copy(), f.copy()
    v = _normalize_rows(_ICO_V)
    f = _ICO_F.copy()
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (len(v) + 1) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (len(v) + 1)
        b = uniq % (len(v) + 1)
        mid = _normalize_rows((v[a] + v[b]) * 0.5)
        nf = len(f)
        m = inv.reshape(3, nf) + len(v)
        ab, bc, ca = m[0], m[1], m[2]
        v = np.concatenate([v, mid])
        f = np.concatenate([
            np.stack([f[:, 0], ab, ca], 1), np.stack([f[:, 1], bc, ab], 1),
            np.stack([f[:, 2], ca, bc], 1), np.stack([ab, bc, ca], 1)])
    f = f.astype(np.uint32)
    _ICO_CACHE[level] = (v, f)
    return v.copy(), f.copy()


def rotation_matrix(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def transform(v: np.ndarray, scale: float = 1.0, rot: np.ndarray | None = None,
              offset=(0.0, 0.0, 0.0)) -> np.ndarray:
    """scale, then rotate (explicit per-component sums, no BLAS), then translate"""
    v = v * scale
    if rot is not None:
        x, y, z = v[:, 0], v[:, 1], v[:, 2]
        v = np.stack([rot[i, 0] * x + rot[i, 1] * y + rot[i, 2] * z for i in range(3)], 1)
    return np.ascontiguousarray(v + np.asarray(offset, dtype=np.float64)[None, :])


def jitter_radial(v: np.ndarray, rng: SplitMix64, rel: float) -> np.ndarray:
    return v * rng.uniform_array(len(v), 1.0 - rel, 1.0 + rel)[:, None]


def pair_small(seed: int = 1234):
    rng = SplitMix64(seed)
    va, fa = icosphere(3)
    vb, fb = icosphere(3)
    vb = transform(vb, 0.8, rotation_matrix(rng.unit_quaternion()), (0.5, 0.3, 0.2))
    return va, fa, vb, fb


def pair_large(seed: int = 1234, level: int = 7):
    rng = SplitMix64(seed)
    va, fa = icosphere(level)
    vb, fb = icosphere(level)
    va = jitter_radial(va, rng, 0.005)
    vb = jitter_radial(vb, rng, 0.005)
    vb = transform(vb, 0.9, rotation_matrix(rng.unit_quaternion()), (0.4, 0.1, -0.2))
    return np.ascontiguousarray(va), fa, vb, fb


def near_tangent(seed: int = 1234, level: int = 6):
    rng = SplitMix64(seed)
    va, fa = icosphere(level)
    vb, fb = icosphere(level)
    va = jitter_radial(va, rng, 1e-7)
    vb = jitter_radial(vb, rng, 1e-7)
    axis = rng.unit_vector()
    vb = transform(vb, 1.0, rotation_matrix(rng.unit_quaternion()), tuple(axis * (2.0 - 1e-3)))
    return np.ascontiguousarray(va), fa, vb, fb


OPS = ("union", "intersect", "diff")


def batch_pair(rng: SplitMix64, max_level: int = 5):
    la = rng.randint(1, max_level)
    lb = rng.randint(1, max_level)
    sa = rng.uniform(0.5, 2.0)
    sb = rng.uniform(0.5, 2.0)
    va, fa = icosphere(la)
    vb, fb = icosphere(lb)
    va = transform(va, sa, rotation_matrix(rng.unit_quaternion()))
    d = rng.uniform(0.2, 0.9) * (sa + sb)
    axis = rng.unit_vector()
    vb = transform(vb, sb, rotation_matrix(rng.unit_quaternion()), tuple(axis * d))
    op = OPS[rng.randint(0, 2)]
    return va, fa, vb, fb, op


def batch(n_pairs: int = 4096, seed: int = 1234, max_level: int = 5):
    rng = SplitMix64(seed)
    return [batch_pair(rng, max_level) for _ in range(n_pairs)]


def interpenetrating(seed: int = 7, level: int = 5, rel: float = 0.005):
    """Two unit icospheres of one level, the second randomly rotated, both jittered radially by U(-rel, +rel):
    the surfaces cross each other all over, so a large share of both meshes' triangles is cut (about 15.7 k
    cut faces per mesh at level 5, 63 k at level 6) into many small loops."""
    rng = SplitMix64(seed)
    va, fa = icosphere(level)
    vb, fb = icosphere(level)
    va = jitter_radial(va, rng, rel)
    vb = transform(vb, 1.0, rotation_matrix(rng.unit_quaternion()))
    vb = jitter_radial(np.ascontiguousarray(vb), rng, rel)
    return np.ascontiguousarray(va), fa, np.ascontiguousarray(vb), fb


def diff_volume(seed: int = 1234, level: int = 5, sigma: float = 0.01):
    rng = SplitMix64(seed)
    va, fa = icosphere(level)
    vb, fb = icosphere(level)
    vb = transform(vb, 0.85, None, (0.35, 0.0, 0.0))
    offs = rng.normal_array(vb.size, sigma).reshape(vb.shape)
    return va, fa, vb, fb, offs
