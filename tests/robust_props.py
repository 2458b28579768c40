"""Properties a boolean's results must have whatever their numbering (used by the robust-mode tests, where the
reference has no result to compare with): every result is closed (each directed edge meets its reverse
exactly once) and the volumes add up, vol(union) + vol(intersect) = vol(A) + vol(B) and
vol(diff) = vol(A) - vol(intersect)."""
from __future__ import annotations

import numpy as np


def volume(v: np.ndarray, t: np.ndarray) -> float:
    t = np.asarray(t, dtype=np.int64).reshape(-1, 3)
    if len(t) == 0:
        return 0.0
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


def open_edges(t: np.ndarray) -> int:
    """directed edges without their reverse, plus directed edges held more than once"""
    t = np.asarray(t, dtype=np.int64).reshape(-1, 3)
    if len(t) == 0:
        return 0
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    fw = set(map(tuple, e.tolist()))
    return sum(1 for (u, v) in fw if (v, u) not in fw) + (len(e) - len(fw))


def check_closed_and_volumes(va, fa, vb, fb, newv, results: dict, rtol: float = 1e-9) -> list[str]:
    """results: {"union", "diff", "intersect"} triangle arrays over newv. Returns the violated properties."""
    bad = []
    for op in ("union", "diff", "intersect"):
        n = open_edges(results[op])
        if n:
            bad.append(f"{op}: {n} open edges")
    VA, VB = volume(va, fa), volume(vb, fb)
    U, D, I = (volume(newv, results[op]) for op in ("union", "diff", "intersect"))
    if abs(U + I - VA - VB) > rtol * (abs(VA) + abs(VB)):
        bad.append(f"vol(union)+vol(intersect)={U + I!r} vs vol(A)+vol(B)={VA + VB!r}")
    if abs(D - (VA - I)) > rtol * (abs(VA) + abs(VB)):
        bad.append(f"vol(diff)={D!r} vs vol(A)-vol(intersect)={VA - I!r}")
    return bad
