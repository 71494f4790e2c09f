"""Python mirror of the reference's public API over the GPU C ABI.

    r = Rasterizer()                       # swr::Rasterizer (Rasterizer.h:52-446)
    r.setRasterMode(RasterMode.Block)
    r.setScissorRect(0, 0, 1920, 1080)
    r.setPixelShader(PS.LAMBERT, uniforms)  # setPixelShader<PS>() + the shader's statics
    v = VertexProcessor(r)                 # swr::VertexProcessor (VertexProcessor.h:56-151)
    v.setViewport(0, 0, 1920, 1080)
    v.setCullMode(CullMode.CW)
    v.setVertexShader(VS.POS_NRM_UV)
    v.setVertexAttribPointer(0, 24, positions_normals)   # CUDA tensors
    v.setVertexAttribPointer(1, 8, uvs)
    v.drawElements(DrawMode.Triangle, n, indices)        # CUDA uint32/int32 tensor

Names, argument meaning and defaults follow the reference (CullMode.CW, depth range
(0, 1), RasterMode.Span, scissor (0, 0, 0, 0)).  Where the reference asserts or has
undefined behaviour (bad attribute index, index count not a multiple of the primitive
size, indices beyond the vertex buffers), these calls raise SwrError.  drawElements and
draw*List are synchronous like the reference's (they return once the pixels are written);
pass sync=False to queue on the current CUDA stream and call finish() later.
"""
import ctypes

import torch

from . import _lib
from .abi import CullMode, DrawMode, RASTER_VERTEX_FLOATS, RasterMode, SwrUniforms


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Context:
    """One swr_context: the joint state of a VertexProcessor and its Rasterizer."""

    def __init__(self):
        L = _lib.lib()
        h = ctypes.c_void_p()
        _lib.check(L.swr_create(ctypes.byref(h)), "swr_create")
        self.h = h
        self.L = L
        self._keep = {}

    def __del__(self):
        if getattr(self, "h", None) is not None and getattr(self, "L", None) is not None:
            self.L.swr_destroy(self.h)
            self.h = None

    def finish(self):
        st = _lib.SwrStats()
        rc = self.L.swr_finish(self.h, _stream(), ctypes.byref(st))
        return rc, {"fragments": st.fragments, "primitives": st.primitives,
                    "bin_pairs": st.bin_pairs, "clip_polygons": st.clip_polygons, "flags": st.flags,
                    "launches": st.launches, "passes": st.passes}

    def set_graph_mode(self, on=True):
        """Replay triangle draws (and batches) as CUDA graphs, captured once per layout."""
        self.L.swr_set_graph_mode.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _lib.check(self.L.swr_set_graph_mode(self.h, int(bool(on))), "set_graph_mode")

    def set_queue_capacity(self, primitives=0, bin_entries=0):
        """Fix the primitive / bin-entry queue sizes (0: automatic); swr_set_queue_capacity."""
        L = self.L
        L.swr_set_queue_capacity.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64]
        L.swr_set_queue_capacity.restype = ctypes.c_int
        _lib.check(L.swr_set_queue_capacity(self.h, int(primitives), int(bin_entries)), "set_queue_capacity")

    def queue_capacity(self):
        L = self.L
        L.swr_get_queue_capacity.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                             ctypes.POINTER(ctypes.c_uint64)]
        L.swr_get_queue_capacity.restype = ctypes.c_int
        p, b = ctypes.c_uint64(0), ctypes.c_uint64(0)
        _lib.check(L.swr_get_queue_capacity(self.h, ctypes.byref(p), ctypes.byref(b)), "queue_capacity")
        return int(p.value), int(b.value)

    def set_memory_limit(self, nbytes=0):
        """Cap the device bytes the context's scratch may hold (0: no cap); beyond it draws
        fail with SWR_ENOMEM and queue nothing."""
        L = self.L
        L.swr_set_memory_limit.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.swr_set_memory_limit.restype = ctypes.c_int
        _lib.check(L.swr_set_memory_limit(self.h, int(nbytes)), "set_memory_limit")

    def memory_used(self):
        L = self.L
        L.swr_memory_used.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
        L.swr_memory_used.restype = ctypes.c_int
        v = ctypes.c_uint64(0)
        _lib.check(L.swr_memory_used(self.h, ctypes.byref(v)), "memory_used")
        return int(v.value)

    def set_persistent_geometry(self, on=True):
        """Vertex shading and triangle assembly as one persistent cooperative launch."""
        self.L.swr_set_persistent_geometry.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self.L.swr_set_persistent_geometry.restype = ctypes.c_int
        _lib.check(self.L.swr_set_persistent_geometry(self.h, int(bool(on))), "set_persistent_geometry")

    def set_tile_split(self, on=True):
        """Heavy 16-px tiles rasterized as four 8 x 8 quadrant CTAs, or whole (the default)."""
        self.L.swr_set_tile_split.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self.L.swr_set_tile_split.restype = ctypes.c_int
        _lib.check(self.L.swr_set_tile_split(self.h, int(bool(on))), "set_tile_split")

    def set_tile_slicing(self, chunks=-1):
        """Tiles of more than `chunks` raster chunks rasterized in four runs (depth-min
        shaders); 0: every tile whole by one CTA; -1: the shader's own setting."""
        self.L.swr_set_tile_slicing.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self.L.swr_set_tile_slicing.restype = ctypes.c_int
        _lib.check(self.L.swr_set_tile_slicing(self.h, int(chunks)), "set_tile_slicing")

    def set_profiling(self, on=True):
        _lib.check(self.L.swr_set_profiling(self.h, int(bool(on))), "set_profiling")

    STAGES = ("vertex", "assemble", "setup", "bin", "raster")

    def stage_times(self):
        """Per-stage durations (ms) summed over the draws since the previous call, measured
        with CUDA events on the stream the stage kernels run on."""
        ms = (ctypes.c_float * 5)()
        _lib.check(self.L.swr_stage_times(self.h, ms), "stage_times")
        return dict(zip(self.STAGES, [float(x) for x in ms]))


class Rasterizer:
    """swr::Rasterizer: raster mode, scissor and pixel shader (Rasterizer.h:66-141)."""

    def __init__(self, ctx: Context = None):
        self.ctx = ctx or Context()
        self.last_stats = None

    def setRasterMode(self, mode):
        _lib.check(self.ctx.L.swr_set_raster_mode(self.ctx.h, int(RasterMode(mode))), "setRasterMode")

    def setScissorRect(self, x, y, width, height):
        _lib.check(self.ctx.L.swr_set_scissor_rect(self.ctx.h, x, y, width, height), "setScissorRect")

    def setPixelShader(self, ps_id, uniforms: SwrUniforms = None):
        _lib.check(self.ctx.L.swr_set_pixel_shader(self.ctx.h, int(ps_id)), "setPixelShader")
        if uniforms is not None:
            self.setUniforms(uniforms)

    def setUniforms(self, uniforms: SwrUniforms):
        self.ctx._keep["uniforms"] = uniforms
        _lib.check(self.ctx.L.swr_set_uniforms(self.ctx.h, ctypes.byref(uniforms)), "uniforms")

    def setTileSize(self, tile):
        _lib.check(self.ctx.L.swr_set_tile_size(self.ctx.h, int(tile)), "setTileSize")

    def _draw_list(self, mode, vertices, indices, sync):
        vertices = vertices.reshape(-1, RASTER_VERTEX_FLOATS)
        assert vertices.is_cuda and vertices.dtype == torch.float32 and vertices.is_contiguous()
        assert indices.is_cuda and indices.dtype == torch.int32 and indices.is_contiguous()
        for _ in range(4):
            rc = self.ctx.L.swr_draw_list(self.ctx.h, int(mode), ctypes.c_void_p(vertices.data_ptr()),
                                          vertices.shape[0], ctypes.c_void_p(indices.data_ptr()),
                                          indices.numel(), _stream())
            _lib.check(rc, "draw list")
            if not sync:
                return None
            rc, st = self.ctx.finish()
            self.last_stats = st
            if rc != _lib.SWR_EOVERFLOW:
                _lib.check(rc, "draw list")
                return st
        raise _lib.SwrError(_lib.SWR_EOVERFLOW, "draw list")

    def drawTriangleList(self, vertices, indices, sync=True):
        """IRasterizer::drawTriangleList (IRasterizer.h:70): RasterizerVertex records."""
        return self._draw_list(DrawMode.Triangle, vertices, indices, sync)

    def drawLineList(self, vertices, indices, sync=True):
        return self._draw_list(DrawMode.Line, vertices, indices, sync)

    def drawPointList(self, vertices, indices, sync=True):
        return self._draw_list(DrawMode.Point, vertices, indices, sync)

    def drawTriangle(self, v0, v1, v2, sync=True):
        """Rasterizer::drawTriangle (Rasterizer.h:111-114) with three RasterizerVertex rows."""
        v = torch.stack([torch.as_tensor(x, dtype=torch.float32) for x in (v0, v1, v2)]).cuda()
        return self.drawTriangleList(v, torch.tensor([0, 1, 2], dtype=torch.int32, device="cuda"), sync)


class VertexProcessor:
    """swr::VertexProcessor (VertexProcessor.h:56-151) bound to a Rasterizer."""

    def __init__(self, rasterizer: Rasterizer):
        self.setRasterizer(rasterizer)
        self._attribs = {}

    def setRasterizer(self, rasterizer: Rasterizer):
        self.r = rasterizer
        self.ctx = rasterizer.ctx

    def setViewport(self, x, y, width, height):
        _lib.check(self.ctx.L.swr_set_viewport(self.ctx.h, x, y, width, height), "setViewport")

    def setDepthRange(self, n, f):
        _lib.check(self.ctx.L.swr_set_depth_range(self.ctx.h, float(n), float(f)), "setDepthRange")

    def setCullMode(self, mode):
        _lib.check(self.ctx.L.swr_set_cull_mode(self.ctx.h, int(CullMode(mode))), "setCullMode")

    def setVertexShader(self, vs_id):
        _lib.check(self.ctx.L.swr_set_vertex_shader(self.ctx.h, int(vs_id)), "setVertexShader")

    def setVertexAttribPointer(self, index, stride, buffer: torch.Tensor):
        assert buffer.is_cuda and buffer.is_contiguous()
        self._attribs[index] = buffer
        nbytes = buffer.numel() * buffer.element_size()
        _lib.check(self.ctx.L.swr_set_vertex_attrib_pointer(self.ctx.h, index, stride,
                                                            ctypes.c_void_p(buffer.data_ptr()), nbytes),
                   "setVertexAttribPointer")

    def drawElements(self, mode, count, indices: torch.Tensor, sync=True):
        """VertexProcessor::drawElements (VertexProcessor.cpp:78-120)."""
        assert indices.is_cuda and indices.dtype in (torch.int32, torch.uint32) and indices.is_contiguous()
        assert count <= indices.numel()
        for _ in range(4):
            rc = self.ctx.L.swr_draw_elements(self.ctx.h, int(DrawMode(mode)), int(count),
                                              ctypes.c_void_p(indices.data_ptr()), _stream())
            _lib.check(rc, "drawElements")
            if not sync:
                return None
            rc, st = self.ctx.finish()
            self.r.last_stats = st
            if rc != _lib.SWR_EOVERFLOW:
                _lib.check(rc, "drawElements")
                return st
        raise _lib.SwrError(_lib.SWR_EOVERFLOW, "drawElements")
