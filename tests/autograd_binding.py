"""Test-only torch binding of the adjoint: a torch.autograd.Function whose forward runs one boolean on
device-resident inputs (sb_mesh_create_device, sb_combine) and returns the result vertices and the
operation's triangles, and whose backward calls sb_adjoint."""
import ctypes

import numpy as np
import torch

import solidboolean_gb300 as sbg


class _Run:
    """Meshes and boolean handle of one forward pass (kept alive for the backward pass)."""

    def __init__(self, va, fa, vb, fb, op, weld_factor):
        L = sbg.lib()
        self.opts = sbg.make_options(weld_factor, "filtered", "reference", torch.cuda.current_stream().cuda_stream)
        self.ta = fa.to(torch.int32).contiguous()
        self.tb = fb.to(torch.int32).contiguous()
        self.va = va.contiguous()
        self.vb = vb.contiguous()
        self.hA, self.hB, self.hX = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        sbg._check(L.sb_mesh_create_device(self.va.data_ptr(), len(va), self.ta.data_ptr(), len(fa),
                                           ctypes.byref(self.opts), ctypes.byref(self.hA)), "create A")
        sbg._check(L.sb_mesh_create_device(self.vb.data_ptr(), len(vb), self.tb.data_ptr(), len(fb),
                                           ctypes.byref(self.opts), ctypes.byref(self.hB)), "create B")
        sbg._check(L.sb_boolean_create(self.hA, self.hB, ctypes.byref(self.opts), ctypes.byref(self.hX)), "boolean")
        stats = sbg.Stats()
        self.code = L.sb_combine(self.hX, ctypes.byref(stats))
        self.ok = self.code == sbg.SB_OK
        x = sbg.SolidBoolean.__new__(sbg.SolidBoolean)
        x._h = self.hX
        self.vertices = torch.from_numpy(x.resultVertices()).to(va.device) if self.ok else None
        self.tris = torch.from_numpy(x.fetch(op).astype(np.int64)).to(va.device) if self.ok else None
        x._h = ctypes.c_void_p()

    def adjoint(self, grad):
        L = sbg.lib()
        ga = torch.zeros_like(self.va)
        gb = torch.zeros_like(self.vb)
        g = grad.contiguous()
        sbg._check(L.sb_adjoint(self.hX, g.data_ptr(), ga.data_ptr(), gb.data_ptr(),
                                torch.cuda.current_stream().cuda_stream), "adjoint")
        torch.cuda.synchronize()
        return ga, gb

    def close(self):
        L = sbg.lib()
        L.sb_boolean_destroy(self.hX)
        L.sb_mesh_destroy(self.hA)
        L.sb_mesh_destroy(self.hB)


class BooleanFn(torch.autograd.Function):
    """(va, vb) -> result vertices; the triangles of the operation are returned through ctx-free side output."""

    @staticmethod
    def forward(ctx, va, vb, fa, fb, op, weld_factor):
        run = _Run(va.detach(), fa, vb.detach(), fb, op, weld_factor)
        if not run.ok:
            run.close()
            raise RuntimeError(f"combine failed with status {run.code}")
        ctx.run = run
        ctx.mark_non_differentiable(run.tris)
        return run.vertices, run.tris

    @staticmethod
    def backward(ctx, g_vertices, g_tris):
        ga, gb = ctx.run.adjoint(g_vertices)
        ctx.run.close()
        return ga, gb, None, None, None, None


def volume_loss(vertices, tris):
    """enclosed volume (divergence theorem) plus 0.1 x the squared norms of the vertices the result uses"""
    v0, v1, v2 = vertices[tris[:, 0]], vertices[tris[:, 1]], vertices[tris[:, 2]]
    vol = (v0 * torch.cross(v1, v2, dim=1)).sum() / 6.0
    used = torch.unique(tris)
    return vol + 0.1 * (vertices[used] ** 2).sum()
