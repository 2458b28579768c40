"""GPU: the adjoint of the boolean (sb_adjoint, through the test-only torch binding) against central finite
differences. Workload: intersection of two level-5 icospheres (radius 1 and 0.85, offset (0.35, 0, 0)), B's
vertices carrying seeded N(0, 0.01^2) offsets; loss = enclosed volume + 0.1 x squared norms of the result's
vertices; h = 1e-6 on 64 seeded vertices near the intersection (half of each mesh), each checked only where
both perturbed runs keep the combinatorics of the base run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_adjoint_matches_finite_differences(gpu_lib):
    from solidboolean_gb300 import meshgen as mg
    from autograd_binding import BooleanFn, _Run, volume_loss

    va_np, fa_np, vb_np, fb_np, offs = mg.diff_volume(1234, 5)
    dev = torch.device("cuda", 0)
    va = torch.from_numpy(va_np).to(dev).requires_grad_(True)
    off = torch.from_numpy(offs).to(dev).requires_grad_(True)
    fa = torch.from_numpy(fa_np.astype(np.int64)).to(dev)
    fb = torch.from_numpy(fb_np.astype(np.int64)).to(dev)
    vb0 = torch.from_numpy(vb_np).to(dev)
    q = 100000000
    verts, tris = BooleanFn.apply(va, vb0 + off, fa, fb, "intersect", q)
    loss = volume_loss(verts, tris)
    loss.backward()
    ga, goff = va.grad.detach().cpu().numpy(), off.grad.detach().cpu().numpy()
    assert np.isfinite(ga).all() and np.isfinite(goff).all()

    base_tris = tris.cpu().numpy()
    n_vertices = verts.shape[0]

    def loss_at(va_t, vb_t):
        run = _Run(va_t, fa, vb_t, fb, "intersect", q)
        try:
            if not run.ok or run.vertices.shape[0] != n_vertices or not np.array_equal(run.tris.cpu().numpy(),
                                                                                       base_tris):
                return None
            return float(volume_loss(run.vertices, run.tris))
        finally:
            run.close()

    # vertices of triangles that the other mesh cuts: their gradients pass through the intersection points
    from solidboolean_gb300 import run_boolean
    d = run_boolean(va_np, fa_np, vb_np + offs, fb_np, q)
    pairs = d["isect_pairs"]
    near_a = np.unique(fa_np[np.unique(pairs[:, 0])])
    near_b = np.unique(fb_np[np.unique(pairs[:, 1])])
    rng = np.random.default_rng(64)
    pick = [("a", int(i)) for i in rng.choice(near_a, 32, replace=False)] + \
           [("b", int(i)) for i in rng.choice(near_b, 32, replace=False)]
    h = 1e-6
    checked, worst = 0, 0.0
    vb_base = (vb0 + off).detach()
    for side, v in pick:
        for axis in range(3):
            vam, vap = va.detach().clone(), va.detach().clone()
            vbm, vbp = vb_base.clone(), vb_base.clone()
            if side == "a":
                vam[v, axis] -= h
                vap[v, axis] += h
            else:
                vbm[v, axis] -= h
                vbp[v, axis] += h
            lm, lp = loss_at(vam, vbm), loss_at(vap, vbp)
            if lm is None or lp is None:
                continue  # the perturbation changes the combinatorics: no derivative to compare
            fd = (lp - lm) / (2 * h)
            adj = ga[v, axis] if side == "a" else goff[v, axis]
            err = abs(fd - adj) / max(1.0, abs(adj))
            worst = max(worst, err)
            assert err < 1e-6, (side, v, axis, fd, adj)
            checked += 1
    print(f"adjoint vs central differences: {checked} components, worst relative error {worst:.2e}")
    assert checked >= 96, checked  # most of the 192 components keep the combinatorics


def _segment_end(b, o, q0, q1, q2):
    """The intersection of the edge (b, o) with the plane through q0, q1, q2 (any number type)."""
    n = np.cross(q1 - q0, q2 - q0)
    t = np.dot(q0 - b, n) / np.dot(o - b, n)
    return b + t * (o - b)


def test_adjoint_matches_cpu_reference_gradient(gpu_lib):
    """sb_adjoint against an FP64 CPU gradient of the same construction, derived independently of the
    records the GPU keeps: every appended vertex lies on an edge (b, o) of one triangle of its pair and in
    the plane of the other triangle (q0, q1, q2); x = b + t (o - b), t = ((q0 - b).N) / ((o - b).N),
    N = (q1 - q0) x (q2 - q0) depends on the other triangle only through its plane, so its Jacobian is unique.
    The Jacobian is taken by complex-step differentiation (exact to rounding); vertices that lie on two
    edges at once are left out of the comparison (their edge is ambiguous)."""
    from solidboolean_gb300 import meshgen as mg
    from autograd_binding import _Run

    va_np, fa_np, vb_np, fb_np, offs = mg.diff_volume(1234, 5)
    vb_np = vb_np + offs
    dev = torch.device("cuda", 0)
    run = _Run(torch.from_numpy(va_np).to(dev), torch.from_numpy(fa_np.astype(np.int64)).to(dev),
               torch.from_numpy(vb_np).to(dev), torch.from_numpy(fb_np.astype(np.int64)).to(dev),
               "intersect", 100000000)
    try:
        assert run.ok
        import solidboolean_gb300 as sbg
        x = sbg.SolidBoolean.__new__(sbg.SolidBoolean)
        x._h = run.hX
        pairs = x.dump("intersection_pairs", np.uint32, 2).astype(np.int64)
        src = x.dump("new_sources", np.int32, 1).astype(np.int64)
        x._h = None
        nv = run.vertices.shape[0]
        nbase = len(va_np) + len(vb_np)
        assert len(src) == nv - nbase and len(src) > 500
        rng = np.random.default_rng(5)
        g = rng.standard_normal((nv, 3))
        ga, gb = run.adjoint(torch.from_numpy(g).to(dev))
        ga, gb = ga.cpu().numpy(), gb.cpu().numpy()

        ref_a, ref_b = g[:len(va_np)].copy(), g[len(va_np):nbase].copy()
        pos = run.vertices.cpu().numpy()
        skip_a, skip_b = np.zeros(len(va_np), bool), np.zeros(len(vb_np), bool)
        used = 0
        for k, sv in enumerate(src):
            pair, _end = divmod(int(sv), 2)
            ta, tb = fa_np[pairs[pair, 0]], fb_np[pairs[pair, 1]]
            xk = pos[nbase + k]
            # the edge that holds the vertex: (mesh of the edge, its two vertex ids)
            cands = []
            for side, tri, verts in (("a", ta, va_np), ("b", tb, vb_np)):
                for e in range(3):
                    u, w = verts[tri[e]], verts[tri[(e + 1) % 3]]
                    d = w - u
                    t = np.dot(xk - u, d) / np.dot(d, d)
                    dist = np.linalg.norm(u + t * d - xk) / max(1.0, np.linalg.norm(d))
                    cands.append((dist, side, tri[e], tri[(e + 1) % 3]))
            cands.sort(key=lambda c: c[0])
            if cands[1][0] < 1e-9:  # on two edges: ambiguous, the pair's six vertices are not compared
                skip_a[ta] = True
                skip_b[tb] = True
                continue
            _, side, ib, io = cands[0]
            other = tb if side == "a" else ta
            ev, ov = (va_np, vb_np) if side == "a" else (vb_np, va_np)
            args = [ev[ib], ev[io], ov[other[0]], ov[other[1]], ov[other[2]]]
            assert np.allclose(_segment_end(*args), xk, rtol=0, atol=1e-12)
            h = 1e-30
            for arg_i, (mesh_of, vid) in enumerate([(side, ib), (side, io), ("b" if side == "a" else "a", other[0]),
                                                   ("b" if side == "a" else "a", other[1]),
                                                   ("b" if side == "a" else "a", other[2])]):
                for c in range(3):
                    cargs = [a.astype(complex) for a in args]
                    cargs[arg_i][c] += 1j * h
                    dx = _segment_end(*cargs).imag / h  # d x / d (that coordinate)
                    (ref_a if mesh_of == "a" else ref_b)[vid, c] += float(np.dot(g[nbase + k], dx))
            used += 1
        assert used > 500
        scale = max(np.abs(ref_a).max(), np.abs(ref_b).max())
        err_a = np.abs(ga - ref_a)[~skip_a].max() / scale
        err_b = np.abs(gb - ref_b)[~skip_b].max() / scale
        print(f"adjoint vs CPU reference gradient: {used} appended vertices, max error {max(err_a, err_b):.2e}")
        assert err_a < 1e-9 and err_b < 1e-9
    finally:
        run.close()
