"""OBJ input and output for the boolean, as the reference's test driver uses them (test/main.cpp:9-71).

Reading follows tinyobjloader as vendored by the reference (test/tiny_obj_loader.h, `triangulate = true`):
coordinates are parsed into single precision (its `real_t` is float) and widened to double by the caller
(test/main.cpp:49-55); a polygon with more than three corners is split by its ear-clipping scheme
(test/tiny_obj_loader.h:1367-1575): the two projection axes are taken from the first corner whose cross
product exceeds float epsilon, the signed area fixes the orientation, and ears are cut starting from a guessed
corner that advances past reflex corners and corners whose triangle holds another corner (crossing-number
test, test/tiny_obj_loader.h:1330-1340). All of that arithmetic is single precision. Only `v` and `f`
records matter here (texture and normal indices are ignored; negative indices count from the end).

Writing follows exportObject (test/main.cpp:9-29): `v %f %f %f`, then `f a b c` with 1-based indices.
"""
from __future__ import annotations

import numpy as np

_f32 = np.float32


def _pnpoly(vx, vy, tx, ty) -> bool:
    c = False
    j = 2
    for i in range(3):
        if (vy[i] > ty) != (vy[j] > ty):
            x = _f32(_f32(_f32(vx[j] - vx[i]) * _f32(ty - vy[i])) / _f32(vy[j] - vy[i])) + vx[i]
            if tx < _f32(x):
                c = not c
        j = i
    return c


def _triangulate(face: list[int], v: np.ndarray) -> list[tuple[int, int, int]]:
    n = len(face)
    if n < 3:
        return []
    if n == 3:
        return [(face[0], face[1], face[2])]
    eps = np.finfo(np.float32).eps
    axes = [1, 2]
    for k in range(n):
        p0, p1, p2 = v[face[k % n]], v[face[(k + 1) % n]], v[face[(k + 2) % n]]
        e0 = [_f32(p1[a] - p0[a]) for a in range(3)]
        e1 = [_f32(p2[a] - p1[a]) for a in range(3)]
        cx = abs(_f32(_f32(e0[1] * e1[2]) - _f32(e0[2] * e1[1])))
        cy = abs(_f32(_f32(e0[2] * e1[0]) - _f32(e0[0] * e1[2])))
        cz = abs(_f32(_f32(e0[0] * e1[1]) - _f32(e0[1] * e1[0])))
        if cx > eps or cy > eps or cz > eps:
            if not (cx > cy and cx > cz):
                axes[0] = 0
                if cz > cx and cz > cy:
                    axes[1] = 1
            break
    ax, ay = axes
    area = _f32(0.0)
    for k in range(n):
        a, b = v[face[k]], v[face[(k + 1) % n]]
        area = _f32(area + _f32(_f32(_f32(a[ax] * b[ay]) - _f32(a[ay] * b[ax])) * _f32(0.5)))
    rem = list(face)
    out = []
    guess = 0
    iters = len(face)
    prev = len(rem)
    while len(rem) > 3 and iters > 0:
        m = len(rem)
        if guess >= m:
            guess -= m
        if prev != m:
            prev = m
            iters = m
        else:
            iters -= 1
        ind = [rem[(guess + k) % m] for k in range(3)]
        vx = [v[i][ax] for i in ind]
        vy = [v[i][ay] for i in ind]
        e0x, e0y = _f32(vx[1] - vx[0]), _f32(vy[1] - vy[0])
        e1x, e1y = _f32(vx[2] - vx[1]), _f32(vy[2] - vy[1])
        cross = _f32(_f32(e0x * e1y) - _f32(e0y * e1x))
        if _f32(cross * area) < 0:
            guess += 1
            continue
        overlap = False
        for other in range(3, m):
            t = v[rem[(guess + other) % m]]
            if _pnpoly(vx, vy, t[ax], t[ay]):
                overlap = True
                break
        if overlap:
            guess += 1
            continue
        out.append((ind[0], ind[1], ind[2]))
        del rem[(guess + 1) % m]
    if len(rem) == 3:
        out.append((rem[0], rem[1], rem[2]))
    return out


def load_obj(path: str) -> tuple[np.ndarray, np.ndarray]:
    """(vertices [n, 3] float64 holding single-precision values, triangles [m, 3] uint32)."""
    verts: list[list[float]] = []
    faces: list[list[int]] = []
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "v" and len(parts) >= 4:
                verts.append([float(x) for x in parts[1:4]])
            elif parts[0] == "f":
                idx = []
                for p in parts[1:]:
                    i = int(p.split("/")[0])
                    idx.append(i - 1 if i > 0 else len(verts) + i)
                faces.append(idx)
    v32 = np.asarray(verts, dtype=np.float32).reshape(-1, 3)
    tris: list[tuple[int, int, int]] = []
    for f in faces:
        tris.extend(_triangulate(f, v32))
    return v32.astype(np.float64), np.asarray(tris, dtype=np.uint32).reshape(-1, 3)


def save_obj(path: str, vertices: np.ndarray, triangles: np.ndarray) -> None:
    with open(path, "w") as fh:
        for x, y, z in np.asarray(vertices, dtype=np.float64):
            fh.write(f"v {x:f} {y:f} {z:f}\n")
        for a, b, c in np.asarray(triangles, dtype=np.int64):
            fh.write(f"f {a + 1} {b + 1} {c + 1}\n")
