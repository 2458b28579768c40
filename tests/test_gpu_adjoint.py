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
            assert err < 1e-5, (side, v, axis, fd, adj)
            checked += 1
    print(f"adjoint vs central differences: {checked} components, worst relative error {worst:.2e}")
    assert checked >= 96, checked  # most of the 192 components keep the combinatorics
