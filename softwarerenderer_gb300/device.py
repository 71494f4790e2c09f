"""Render a seeded Scene (softwarerenderer_gb300.scenes) through the GPU pipeline.

DeviceScene uploads a scene's vertex/index/texture buffers and allocates a device render
target; `draw()` binds the state on a VertexProcessor/Rasterizer pair exactly as an
application would (setViewport, setCullMode, setVertexShader, setVertexAttribPointer,
setRasterMode, setScissorRect, setPixelShader) and issues drawElements or draw*List.
"""
import numpy as np
import torch

from .abi import DrawMode, make_uniforms
from .renderer import Context, Rasterizer, VertexProcessor


def _dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.view(dtype)
    return t.cuda()


class DeviceTarget:
    def __init__(self, scene, aux=True, clear_color=0, clear_depth=float("inf")):
        h, w = scene.height, scene.width
        if scene.rgba32f:
            self.color = torch.full((h, w, 4), float(clear_color), dtype=torch.float32, device="cuda")
        else:
            self.color = torch.full((h, w), int(clear_color), dtype=torch.int32, device="cuda")
        self.depth = torch.full((h, w), clear_depth, dtype=torch.float32, device="cuda")
        self.frag_count = torch.zeros((h, w), dtype=torch.int32, device="cuda") if aux else None
        self.winner = torch.full((h, w), -1, dtype=torch.int32, device="cuda") if aux else None
        self.clear_color, self.clear_depth = clear_color, clear_depth

    def clear(self):
        """Colour, depth and the per-pixel records in one kernel (swr_clear_target)."""
        import ctypes
        from . import _lib
        from .renderer import _stream
        L = _lib.lib()
        if getattr(self, "_clear_u", None) is None:
            L.swr_clear_target.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_float,
                                           ctypes.c_void_p]
            L.swr_clear_target.restype = ctypes.c_int
            h, w = self.depth.shape
            self._clear_u = make_uniforms(np.eye(4), [0, 0, 1, 0], 0, w, h, color=self.color.data_ptr(),
                                          depth=self.depth.data_ptr(),
                                          frag_count=self.frag_count.data_ptr() if self.frag_count is not None else 0,
                                          winner=self.winner.data_ptr() if self.winner is not None else 0)
            if self.color.dtype == torch.float32:
                self._clear_value = np.full(4, self.clear_color, np.float32)
            else:
                self._clear_value = np.array([int(self.clear_color) & 0xFFFFFFFF], np.uint32)
        nbytes = self._clear_value.nbytes
        _lib.check(L.swr_clear_target(ctypes.byref(self._clear_u), nbytes, self._clear_value.ctypes.data,
                                      float(self.clear_depth), _stream()), "swr_clear_target")

    def to_host(self):
        out = {"color": self.color.cpu().numpy(), "depth": self.depth.cpu().numpy()}
        if out["color"].dtype == np.int32:
            out["color"] = out["color"].view(np.uint32)
        if self.frag_count is not None:
            out["frag_count"] = self.frag_count.cpu().numpy().view(np.uint32)
            out["winner"] = self.winner.cpu().numpy()
        return out


class DeviceScene:
    def __init__(self, scene, ctx: Context = None, tile=16):
        self.scene = scene
        self.rast = Rasterizer(ctx)
        self.vp = VertexProcessor(self.rast)
        self.attribs = [(_dev(a.view(np.uint8).reshape(-1)), s) for a, s in scene.attribs]
        self.indices = _dev(np.asarray(scene.indices, dtype=np.int32))
        self.raster_vertices = (_dev(scene.raster_vertices.astype(np.float32))
                                if scene.raster_vertices is not None else None)
        self.texture = None
        if scene.texture is not None:
            tex = scene.texture
            self.texture = _dev(tex.view(np.int32) if tex.dtype == np.uint32 else tex)
        self.tile = tile

    def uniforms(self, target: DeviceTarget, mvp=None):
        sc = self.scene
        tex = self.texture
        tw, th = sc.texture_wh()
        return make_uniforms(sc.mvp if mvp is None else mvp, sc.light, sc.checker, sc.width, sc.height,
                             tex_ptr=tex.data_ptr() if tex is not None else 0, tex_w=tw, tex_h=th,
                             max_aniso=sc.max_aniso,
                             color=target.color.data_ptr(), depth=target.depth.data_ptr(),
                             frag_count=target.frag_count.data_ptr() if target.frag_count is not None else 0,
                             winner=target.winner.data_ptr() if target.winner is not None else 0)

    def bind(self, target: DeviceTarget, mvp=None):
        sc = self.scene
        r, v = self.rast, self.vp
        r.setRasterMode(sc.raster)
        r.setScissorRect(*sc.scissor)
        r.setTileSize(self.tile)
        r.setPixelShader(sc.ps, self.uniforms(target, mvp))
        if sc.raster_vertices is None:
            v.setViewport(*sc.viewport)
            v.setDepthRange(*sc.depth_range)
            v.setCullMode(sc.cull)
            v.setVertexShader(sc.vs)
            for i, (buf, stride) in enumerate(self.attribs):
                v.setVertexAttribPointer(i, stride, buf)

    def draw(self, target: DeviceTarget, sync=True, mvp=None, bind=True):
        sc = self.scene
        if bind:
            self.bind(target, mvp)
        if sc.raster_vertices is not None:
            return self.rast._draw_list(sc.draw_mode, self.raster_vertices, self.indices, sync)
        return self.vp.drawElements(sc.draw_mode, self.indices.numel(), self.indices, sync)
