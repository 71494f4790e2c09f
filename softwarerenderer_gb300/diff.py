"""Differentiable rendering: forward through swr_draw_batch, backward through swr_backward.

One mesh of vertex records {x, y, z, r, g, b, u, v} (vertex shader VS.POS_RGB_UV) with an
RGBA32F texture is drawn from several views with the pixel shader PS.DIFF (colour =
interpolated vertex rgb * bilinear texel).  The forward records, per view, the winner
buffer and the primitive-source map; the backward holds that visibility fixed and returns
dL/d(vertex records) and dL/d(texels) for dL/d(colour) given per pixel, or for the fused L2
loss L = loss_scale * sum (colour - target)^2.

    dr = DiffRenderer(problem.indices, n_vertices, 1024, 1024, problem.mvps, 512, 512)
    img = dr.forward(vertices, texture)                  # (views, H, W, 4)
    gv, gt, loss = dr.backward(vertices, texture, target=targets)

`render(vertices, texture, dr)` wraps the pair in a torch.autograd.Function; it exists for
gradient checks against finite differences.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .abi import PS, VS, CullMode, RasterMode, make_uniforms
from .batch import SwrDrawItem
from .renderer import Context, _stream

SWR_F_SRC_OVERFLOW = 64


class SwrGradView(ctypes.Structure):
    _fields_ = [
        ("mvp", ctypes.c_float * 16), ("viewport", ctypes.c_int32 * 4),
        ("width", ctypes.c_int32), ("height", ctypes.c_int32),
        ("winner", ctypes.c_void_p), ("prim_src", ctypes.c_void_p), ("nprims", ctypes.c_uint64),
        ("grad_color", ctypes.c_void_p), ("color", ctypes.c_void_p), ("target", ctypes.c_void_p),
        ("loss_scale", ctypes.c_float), ("_pad", ctypes.c_int32),
    ]


class SwrBackwardArgs(ctypes.Structure):
    _fields_ = [
        ("vertices", ctypes.c_void_p), ("nverts", ctypes.c_uint64),
        ("indices", ctypes.c_void_p), ("count", ctypes.c_uint64),
        ("texture", ctypes.c_void_p), ("tex_w", ctypes.c_int32), ("tex_h", ctypes.c_int32),
        ("grad_vertices", ctypes.c_void_p), ("grad_texture", ctypes.c_void_p),
        ("loss", ctypes.c_void_p),
    ]


assert ctypes.sizeof(SwrGradView) == 144 and ctypes.sizeof(SwrBackwardArgs) == 72


def _bind(L):
    if getattr(L, "_swr_diff_bound", False):
        return
    L.swr_draw_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(SwrDrawItem), ctypes.c_int, ctypes.c_void_p]
    L.swr_draw_batch.restype = ctypes.c_int
    L.swr_set_graph_mode.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.swr_set_graph_mode.restype = ctypes.c_int
    L.swr_backward.argtypes = [ctypes.c_void_p, ctypes.POINTER(SwrBackwardArgs), ctypes.POINTER(SwrGradView),
                               ctypes.c_int, ctypes.c_void_p]
    L.swr_backward.restype = ctypes.c_int
    L.swr_set_primitive_source.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
    L.swr_set_primitive_source.restype = ctypes.c_int
    L._swr_diff_bound = True


def _check_tensor(t, name, shape_tail, dtype=torch.float32):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.is_contiguous()):
        raise ValueError(f"{name}: expected a contiguous CUDA {dtype} tensor")
    if tuple(t.shape[-len(shape_tail):]) != tuple(shape_tail):
        raise ValueError(f"{name}: expected trailing shape {shape_tail}, got {tuple(t.shape)}")


class DiffRenderer:
    """Forward and backward of the differentiable shader over a fixed set of views."""

    def __init__(self, indices, n_vertices, tex_w, tex_h, mvps, width, height, cull=CullMode.CW,
                 raster=RasterMode.Block, tile=16, graph=True):
        self.ctx = Context()
        L = self.ctx.L
        _bind(L)
        _lib.check(L.swr_set_tile_size(self.ctx.h, int(tile)), "tile")
        _lib.check(L.swr_set_graph_mode(self.ctx.h, int(bool(graph))), "graph mode")
        idx = indices if isinstance(indices, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(indices))
        self.indices = idx.to(device="cuda", dtype=torch.int32).contiguous()
        if self.indices.numel() % 3:
            raise ValueError("indices: a triangle list needs a multiple of 3 indices")
        self.n_vertices, self.tex_w, self.tex_h = int(n_vertices), int(tex_w), int(tex_h)
        self.width, self.height = int(width), int(height)
        self.mvps = [np.asarray(m, dtype=np.float32).reshape(16) for m in mvps]
        V, H, W = len(self.mvps), self.height, self.width
        self.n_views = V
        ntris = self.indices.numel() // 3
        self.color = torch.zeros((V, H, W, 4), dtype=torch.float32, device="cuda")
        self.depth = torch.full((V, H, W), float("inf"), dtype=torch.float32, device="cuda")
        self.winner = torch.full((V, H, W), -1, dtype=torch.int32, device="cuda")
        # primitives per view: every triangle, plus the fan triangles of clipped ones
        self.prim_cap = 2 * ntris + 1024
        self.prim_src = torch.full((V, self.prim_cap), -1, dtype=torch.int32, device="cuda")
        self.items = (SwrDrawItem * V)()
        self.uniforms = []
        for v in range(V):
            u = make_uniforms(self.mvps[v], [0, 0, 1, 0], 0, W, H, tex_w=self.tex_w, tex_h=self.tex_h,
                              color=self.color[v].data_ptr(), depth=self.depth[v].data_ptr(),
                              winner=self.winner[v].data_ptr())
            self.uniforms.append(u)
            it = self.items[v]
            it.vs_id, it.ps_id = int(VS.POS_RGB_UV), int(PS.DIFF)
            it.cull_mode, it.raster_mode = int(cull), int(raster)
            for k, val in enumerate((0, 0, W, H)):
                it.viewport[k] = val
                it.scissor[k] = val
            it.depth_range[0], it.depth_range[1] = 0.0, 1.0
            it.attrib_stride[0] = 32
            it.attrib_bytes[0] = 32 * self.n_vertices
            it.indices = self.indices.data_ptr()
            it.count = self.indices.numel()
            it.uniforms = ctypes.pointer(u)
            it.prim_src = self.prim_src[v].data_ptr()
            it.prim_src_capacity = self.prim_cap
        self.views = (SwrGradView * V)()
        for v in range(V):
            g = self.views[v]
            for i in range(16):
                g.mvp[i] = float(self.mvps[v][i])
            for k, val in enumerate((0, 0, W, H)):
                g.viewport[k] = val
            g.width, g.height = W, H
            g.nprims = self.prim_cap
        self.args = SwrBackwardArgs()

    # -- forward ---------------------------------------------------------------------

    def _check_inputs(self, vertices, texture):
        _check_tensor(vertices, "vertices", (8,))
        _check_tensor(texture, "texture", (self.tex_h, self.tex_w, 4))
        if vertices.shape[0] != self.n_vertices:
            raise ValueError(f"vertices: expected {self.n_vertices} records")

    def clear(self):
        self.color.zero_()
        self.depth.fill_(float("inf"))
        self.winner.fill_(-1)

    def forward(self, vertices, texture, sync=True):
        """Renders every view into self.color (views, H, W, 4); records winner and prim_src."""
        self._check_inputs(vertices, texture)
        self.clear()
        for v in range(self.n_views):
            self.items[v].attrib[0] = vertices.data_ptr()
            self.uniforms[v].tex = texture.data_ptr()
        L = self.ctx.L
        for _ in range(4):
            _lib.check(L.swr_draw_batch(self.ctx.h, self.items, self.n_views, _stream()), "swr_draw_batch")
            if not sync:
                return self.color
            rc, st = self.ctx.finish()
            if rc == _lib.SWR_EOVERFLOW:
                self.clear()
                continue
            if rc != _lib.SWR_OK and st["flags"] & SWR_F_SRC_OVERFLOW:
                raise _lib.SwrError(rc, "swr_draw_batch: primitive-source buffer too small")
            _lib.check(rc, "swr_draw_batch")
            return self.color
        raise _lib.SwrError(_lib.SWR_EOVERFLOW, "swr_draw_batch")

    # -- backward --------------------------------------------------------------------

    def backward(self, vertices, texture, grad_color=None, target=None, loss_scale=1.0, grad_vertices=None,
                 grad_texture=None, winner=None, prim_src=None, sync=True):
        """Gradients with the visibility of the last forward (or the given winner / prim_src).

        grad_color (views, H, W, 4): dL/d(colour).  Without it, the fused L2 loss against
        `target` (views, H, W, 4) is used and its value is returned as the third result.
        Returns (grad_vertices (N, 8), grad_texture (T, T, 4), loss or None); gradients
        accumulate into grad_vertices / grad_texture when given."""
        self._check_inputs(vertices, texture)
        V, H, W = self.n_views, self.height, self.width
        if grad_color is not None:
            _check_tensor(grad_color, "grad_color", (V, H, W, 4))
        else:
            _check_tensor(target, "target", (V, H, W, 4))
        winner = self.winner if winner is None else winner
        prim_src = self.prim_src if prim_src is None else prim_src
        _check_tensor(winner, "winner", (V, H, W), torch.int32)
        _check_tensor(prim_src, "prim_src", (V, prim_src.shape[-1]), torch.int32)
        gv = torch.zeros_like(vertices) if grad_vertices is None else grad_vertices
        gt = torch.zeros_like(texture) if grad_texture is None else grad_texture
        _check_tensor(gv, "grad_vertices", (self.n_vertices, 8))
        _check_tensor(gt, "grad_texture", (self.tex_h, self.tex_w, 4))
        loss = None if grad_color is not None else torch.zeros((), dtype=torch.float64, device="cuda")
        a = self.args
        a.vertices, a.nverts = vertices.data_ptr(), self.n_vertices
        a.indices, a.count = self.indices.data_ptr(), self.indices.numel()
        a.texture, a.tex_w, a.tex_h = texture.data_ptr(), self.tex_w, self.tex_h
        a.grad_vertices, a.grad_texture = gv.data_ptr(), gt.data_ptr()
        a.loss = loss.data_ptr() if loss is not None else None
        for v in range(V):
            g = self.views[v]
            g.winner = winner[v].data_ptr()
            g.prim_src = prim_src[v].data_ptr()
            g.nprims = prim_src.shape[-1]
            if grad_color is not None:
                g.grad_color, g.color, g.target = grad_color[v].data_ptr(), None, None
            else:
                g.grad_color, g.color, g.target = None, self.color[v].data_ptr(), target[v].data_ptr()
            g.loss_scale = float(loss_scale)
        L = self.ctx.L
        _lib.check(L.swr_backward(self.ctx.h, ctypes.byref(a), self.views, V, _stream()), "swr_backward")
        if sync:
            rc, _ = self.ctx.finish()
            _lib.check(rc, "swr_backward")
        return gv, gt, loss


class RenderFunction(torch.autograd.Function):
    """image = render(vertices, texture); backward through swr_backward (visibility fixed)."""

    @staticmethod
    def forward(ctx, vertices, texture, renderer):
        img = renderer.forward(vertices, texture)
        ctx.renderer = renderer
        ctx.winner = renderer.winner.clone()
        ctx.prim_src = renderer.prim_src.clone()
        ctx.save_for_backward(vertices, texture)
        return img.clone()

    @staticmethod
    def backward(ctx, grad_img):
        vertices, texture = ctx.saved_tensors
        gv, gt, _ = ctx.renderer.backward(vertices.detach(), texture.detach(), grad_color=grad_img.contiguous(),
                                          winner=ctx.winner, prim_src=ctx.prim_src)
        return gv, gt, None


def render(vertices, texture, renderer):
    return RenderFunction.apply(vertices, texture, renderer)


def main(argv=None):
    """Runs the differentiable-rendering workload (16 views of the level-6 icosphere at
    512 x 512, 1024 x 1024 RGBA32F texture, fused L2 loss): `steps` forward + backward
    passes, then prints the loss and the timing of the last pass."""
    import argparse
    import time

    from . import scenes
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--views", type=int, default=16)
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--texture", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=4)
    a = ap.parse_args(argv)
    P = scenes.diff_problem(n_views=a.views, level=a.level, size=a.size, tex_size=a.texture)
    dr = DiffRenderer(P.indices, P.vertices.shape[0], a.texture, a.texture, P.mvps, a.size, a.size,
                      cull=P.cull, raster=P.raster)
    v, t = torch.from_numpy(P.vertices).cuda(), torch.from_numpy(P.texture).cuda()
    tg = torch.from_numpy(P.targets).cuda()
    for _ in range(a.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dr.forward(v, t)
        gv, gt, loss = dr.backward(v, t, target=tg)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    print(f"views={a.views} loss={float(loss):.6e} |dL/dv|={float(gv.norm()):.6e} "
          f"|dL/dtex|={float(gt.norm()):.6e} last step {dt * 1e3:.3f} ms (host clock)")


if __name__ == "__main__":
    main()
