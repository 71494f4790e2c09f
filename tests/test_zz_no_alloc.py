"""The allocation-free triangle-list draw against the context-based one and the oracle.

swr_draw_triangle_list_noalloc exists for callers that cannot allocate device memory (an
application whose device memory is owned by another allocator, a frame loop that must not
stall in cudaMalloc, a plugin handed only a stream and buffers).  It must produce exactly
what swr_draw_list and the CPU oracle produce -- colour, depth, per-pixel fragment count
and winning primitive, bit for bit like every parity test here -- on consecutive calls that
share its one scratch array, and a draw with more bin entries than the array holds must
return SWR_EOVERFLOW with the target untouched and leave the next call correct.  This file
is collected last so a failure here cannot hide others.
"""
import ctypes

import numpy as np
import pytest

from softwarerenderer_gb300 import scenes
from softwarerenderer_gb300.abi import PS, RASTER_VERTEX_FLOATS, VS, CullMode, DrawMode, RasterMode, SwrUniforms

from .parity import diff, oracle_render

pytestmark = pytest.mark.gpu


def _entry(lib):
    f = lib.swr_draw_triangle_list_noalloc
    f.argtypes = [ctypes.POINTER(SwrUniforms), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                  ctypes.c_uint64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
    f.restype = ctypes.c_int
    return f


def _noalloc_call(fn, sc, tg=None):
    import torch
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    ds = DeviceScene(sc)
    tg = tg if tg is not None else DeviceTarget(sc)
    u = ds.uniforms(tg)
    frags = ctypes.c_uint64(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rv, idx = ds.raster_vertices, ds.indices
    rc = fn(ctypes.byref(u), int(sc.ps), int(sc.raster), *[int(v) for v in sc.scissor],
            ctypes.c_void_p(rv.data_ptr()), rv.shape[0], ctypes.c_void_p(idx.data_ptr()), idx.numel(),
            stream, ctypes.byref(frags))
    return rc, tg, int(frags.value)


def _noalloc_render(fn, sc):
    rc, tg, frags = _noalloc_call(fn, sc)
    assert rc == 0, f"swr_draw_triangle_list_noalloc returned {rc}"
    return tg.to_host(), frags


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


def test_noalloc_matches_oracle(gpu_lib, port):
    """Every call equals the CPU oracle; seeds repeat so later calls inherit the array."""
    fn = _entry(gpu_lib)
    for seed in (3, 8, 21, 3, 40, 8):
        sc = scenes.random_scene(seed, direct=True, draw_mode=DrawMode.Triangle)
        got, gf = _noalloc_render(fn, sc)
        ref, st = oracle_render(port, sc)
        assert gf == int(st["fragments"]), (sc.name, gf, st)
        assert not diff(ref, got), (sc.name, diff(ref, got))


def _many_big_triangles(n=160, side=2048, seed=9):
    """Direct-path triangles spanning most of a side x side target: each touches thousands
    of 16 x 16 tiles, so n of them need far more than 262144 (tile, triangle) bin entries."""
    rng = np.random.default_rng(seed)
    rv = np.zeros((3 * n, RASTER_VERTEX_FLOATS), np.float32)
    for t in range(n):
        c = rng.random(2) * 0.2 * side
        rv[3 * t + 0, 0:2] = c
        rv[3 * t + 1, 0:2] = (side - c[0], c[1] + 0.1 * side)
        rv[3 * t + 2, 0:2] = (c[0] + 0.1 * side, side - c[1])
    rv[:, 2] = rng.random(3 * n)
    rv[:, 3] = 1.0
    rv[:, 4:36] = rng.random((3 * n, 32))
    return scenes.Scene(name=f"big{n}", vs=VS.POS_RGB, ps=PS.VCOLOR, width=side, height=side,
                        draw_mode=DrawMode.Triangle, cull=CullMode.None_, raster=RasterMode.Block,
                        viewport=(0, 0, side, side), scissor=(0, 0, side, side),
                        indices=np.arange(3 * n, dtype=np.int32), raster_vertices=rv)


def test_noalloc_bin_overflow_leaves_target_untouched(gpu_lib, port):
    """More bin entries than the fixed array holds: SWR_EOVERFLOW (checked on the device),
    no pixel written; the next call on the same array is again exact."""
    import torch
    from softwarerenderer_gb300.device import DeviceTarget
    fn = _entry(gpu_lib)
    big = _many_big_triangles()
    tg = DeviceTarget(big)
    tg.color.fill_(0x01020304)
    tg.depth.fill_(0.75)
    before = tg.to_host()
    rc, tg, frags = _noalloc_call(fn, big, tg)
    torch.cuda.synchronize()
    assert rc == 3, f"expected SWR_EOVERFLOW, got {rc}"
    assert frags == 0
    after = tg.to_host()
    for k in before:
        assert np.asarray(before[k]).tobytes() == np.asarray(after[k]).tobytes(), k
    # the array keeps the overflowed call's contents: the next call must still be exact
    sc = scenes.random_scene(12, direct=True, draw_mode=DrawMode.Triangle)
    got, gf = _noalloc_render(fn, sc)
    ref, st = oracle_render(port, sc)
    assert not diff(ref, got), (sc.name, diff(ref, got))
    got2, rf = _context_render(sc)
    assert not diff(got2, got)
