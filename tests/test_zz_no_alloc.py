"""The allocation-free triangle-list draw against the context-based one.

swr_draw_triangle_list_noalloc exists for callers that cannot allocate device memory (an
application whose device memory is owned by another allocator, a frame loop that must not
stall in cudaMalloc, a plugin handed only a stream and buffers).  It must produce exactly
what swr_draw_list produces -- colour, depth, per-pixel fragment count and winning
primitive, bit for bit like every parity test here -- on consecutive calls that share its
one scratch array.  This file is collected last so a failure here cannot hide others.
"""
import ctypes

import numpy as np
import pytest

from softwarerenderer_gb300 import scenes
from softwarerenderer_gb300.abi import DrawMode, SwrUniforms

pytestmark = pytest.mark.gpu


def _entry(lib):
    f = lib.swr_draw_triangle_list_noalloc
    f.argtypes = [ctypes.POINTER(SwrUniforms), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                  ctypes.c_uint64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
    f.restype = ctypes.c_int
    return f


def _noalloc_render(fn, sc):
    import torch
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    ds = DeviceScene(sc)
    tg = DeviceTarget(sc)
    u = ds.uniforms(tg)
    frags = ctypes.c_uint64(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rv, idx = ds.raster_vertices, ds.indices
    rc = fn(ctypes.byref(u), int(sc.ps), int(sc.raster), *[int(v) for v in sc.scissor],
            ctypes.c_void_p(rv.data_ptr()), rv.shape[0], ctypes.c_void_p(idx.data_ptr()), idx.numel(),
            stream, ctypes.byref(frags))
    assert rc == 0, f"swr_draw_triangle_list_noalloc returned {rc}"
    return tg.to_host(), int(frags.value)


def _context_render(sc):
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    ds = DeviceScene(sc)
    tg = DeviceTarget(sc)
    st = ds.draw(tg)
    return tg.to_host(), int(st["fragments"])


def test_noalloc_matches_draw_list_on_consecutive_calls(gpu_lib):
    fn = _entry(gpu_lib)
    picked = [scenes.random_scene(s, direct=True, draw_mode=DrawMode.Triangle) for s in (5, 12, 5)]
    for sc in picked:  # three calls in a row share (and inherit) the scratch array
        got, gf = _noalloc_render(fn, sc)
        ref, rf = _context_render(sc)
        assert gf == rf and rf > 0, (sc.name, gf, rf)
        for k in ref:
            assert np.asarray(ref[k]).tobytes() == np.asarray(got[k]).tobytes(), (sc.name, k)


def test_noalloc_rejects_oversized_input(gpu_lib):
    fn = _entry(gpu_lib)
    sc = scenes.random_scene(5, direct=True, draw_mode=DrawMode.Triangle)
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    ds = DeviceScene(sc)
    tg = DeviceTarget(sc)
    u = ds.uniforms(tg)
    rc = fn(ctypes.byref(u), int(sc.ps), int(sc.raster), 0, 0, sc.width, sc.height,
            ctypes.c_void_p(ds.raster_vertices.data_ptr()), 12289, ctypes.c_void_p(ds.indices.data_ptr()),
            3 * 4097, None, None)
    assert rc == 1  # SWR_EINVAL: beyond the documented limits, nothing queued
