"""Batched rendering through swr_draw_batch: many meshes, each with its own target,
camera and texture, in one pass of the pipeline (optionally replayed as a CUDA graph).

    br = BatchRenderer(scenes.batch_scenes(256))
    br.draw()                      # all 256 views; br.targets[i] holds view i
    br.draw_loop()                 # the same views as 256 separate drawElements calls
"""
import ctypes

import torch

from . import _lib
from .abi import SwrUniforms
from .device import DeviceScene, DeviceTarget
from .renderer import Context, _stream


class SwrDrawItem(ctypes.Structure):
    _fields_ = [
        ("vs_id", ctypes.c_int32), ("ps_id", ctypes.c_int32),
        ("cull_mode", ctypes.c_int32), ("raster_mode", ctypes.c_int32),
        ("viewport", ctypes.c_int32 * 4),
        ("depth_range", ctypes.c_float * 2),
        ("scissor", ctypes.c_int32 * 4),
        ("attrib", ctypes.c_void_p * 8),
        ("attrib_stride", ctypes.c_int32 * 8),
        ("attrib_bytes", ctypes.c_uint64 * 8),
        ("indices", ctypes.c_void_p),
        ("count", ctypes.c_uint64),
        ("uniforms", ctypes.POINTER(SwrUniforms)),
        ("prim_src", ctypes.c_void_p),
        ("prim_src_capacity", ctypes.c_uint64),
    ]


assert ctypes.sizeof(SwrDrawItem) == 256


class _PooledTarget:
    """A render target whose colour and depth are views into pooled buffers."""

    def __init__(self, color, depth):
        self.color, self.depth = color, depth
        self.frag_count = self.winner = None

    def to_host(self):
        return {"color": self.color.cpu().numpy().view("uint32"), "depth": self.depth.cpu().numpy()}


class TargetPool:
    """One colour and one depth allocation sliced into per-scene targets (RGBA8 shaders),
    so a whole batch is cleared by two fills."""

    def __init__(self, scenes, clear_color=0, clear_depth=float("inf")):
        sizes = [sc.width * sc.height for sc in scenes]
        total = sum(sizes)
        self.color = torch.full((total,), int(clear_color), dtype=torch.int32, device="cuda")
        self.depth = torch.full((total,), clear_depth, dtype=torch.float32, device="cuda")
        self.clear_color, self.clear_depth = clear_color, clear_depth
        self.targets = []
        off = 0
        for sc, n in zip(scenes, sizes):
            self.targets.append(_PooledTarget(self.color[off:off + n].view(sc.height, sc.width),
                                              self.depth[off:off + n].view(sc.height, sc.width)))
            off += n

    def clear(self):
        self.color.fill_(self.clear_color)
        self.depth.fill_(self.clear_depth)


class BatchRenderer:
    def __init__(self, scenes, aux=False, tile=16, graph=True, targets=None, pooled=False):
        self.ctx = Context()
        L = self.ctx.L
        L.swr_draw_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(SwrDrawItem), ctypes.c_int, ctypes.c_void_p]
        L.swr_draw_batch.restype = ctypes.c_int
        L.swr_set_graph_mode.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.swr_set_graph_mode.restype = ctypes.c_int
        _lib.check(L.swr_set_tile_size(self.ctx.h, int(tile)), "tile")
        _lib.check(L.swr_set_graph_mode(self.ctx.h, int(bool(graph))), "graph mode")
        self.scenes = scenes
        self.dev = [DeviceScene(sc, tile=tile) for sc in scenes]
        # by default one target per scene; `targets` may map scenes onto shared targets
        self.pool = TargetPool(scenes) if pooled and targets is None else None
        if self.pool is not None:
            self.targets = self.pool.targets
        else:
            self.targets = targets if targets is not None else [DeviceTarget(sc, aux=aux) for sc in scenes]
        self.items = (SwrDrawItem * len(scenes))()
        self.uniforms = []
        self._fill()

    def _fill(self, mvps=None):
        self.uniforms = []
        for i, (sc, ds, tg) in enumerate(zip(self.scenes, self.dev, self.targets)):
            u = ds.uniforms(tg, None if mvps is None else mvps[i])
            self.uniforms.append(u)
            it = self.items[i]
            it.vs_id, it.ps_id = int(sc.vs), int(sc.ps)
            it.cull_mode, it.raster_mode = int(sc.cull), int(sc.raster)
            for k in range(4):
                it.viewport[k] = int(sc.viewport[k])
                it.scissor[k] = int(sc.scissor[k])
            it.depth_range[0], it.depth_range[1] = float(sc.depth_range[0]), float(sc.depth_range[1])
            for a, (buf, stride) in enumerate(ds.attribs):
                it.attrib[a] = buf.data_ptr()
                it.attrib_stride[a] = int(stride)
                it.attrib_bytes[a] = buf.numel()
            it.indices = ds.indices.data_ptr()
            it.count = ds.indices.numel()
            it.uniforms = ctypes.pointer(u)

    def clear(self):
        if self.pool is not None:
            self.pool.clear()
            return
        for tg in self.targets:
            tg.clear()

    def draw(self, sync=True, mvps=None):
        """All scenes in one swr_draw_batch call."""
        if mvps is not None:
            self._fill(mvps)
        for _ in range(4):
            rc = self.ctx.L.swr_draw_batch(self.ctx.h, self.items, len(self.scenes), _stream())
            _lib.check(rc, "swr_draw_batch")
            if not sync:
                return None
            rc, st = self.ctx.finish()
            if rc != _lib.SWR_EOVERFLOW:
                _lib.check(rc, "swr_draw_batch")
                return st
        raise _lib.SwrError(_lib.SWR_EOVERFLOW, "swr_draw_batch")

    def draw_loop(self, sync=True):
        """The same scenes as one drawElements call each (the unbatched baseline)."""
        for ds, tg in zip(self.dev, self.targets):
            ds.draw(tg, sync=False)
        if sync:
            for ds in self.dev:
                rc, st = ds.rast.ctx.finish()
                _lib.check(rc, "drawElements")
