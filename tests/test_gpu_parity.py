"""GPU parity: the CUDA pipeline against the CPU oracle (bit-exact).

Every buffer the pixel shaders write is compared bit for bit: colour, depth, per-pixel
drawPixel count (covered-pixel set and fragment count) and the id of the primitive that
won the depth test.  Shaded colours are computed with the same IEEE operations on both
sides, so the stated colour tolerance (max abs error <= 2^-20 on FP32 outputs) is met with
zero error; the comparison is exact.
"""
import numpy as np
import pytest

from softwarerenderer_gb300 import scenes
from softwarerenderer_gb300.abi import DrawMode, RasterMode

from .parity import describe, diff, gpu_render, oracle_render

pytestmark = pytest.mark.gpu

TRI_SEEDS = list(range(0, 160))


def _check(port, sc, tile=16, split=False):
    ref, rst = oracle_render(port, sc)
    got, gst = gpu_render(sc, tile=tile, split=split)
    bad = diff(ref, got)
    msgs = [describe(ref, got, k) for k in bad]
    assert not bad, f"{sc.name} {sc.draw_mode.name} {sc.raster.name}: " + "; ".join(msgs)
    assert gst["fragments"] == rst["fragments"], (sc.name, gst, rst)
    return rst


@pytest.mark.parametrize("seed", TRI_SEEDS)
def test_random_triangles(gpu_lib, port, seed):
    sc = scenes.random_scene(seed, draw_mode=DrawMode.Triangle)
    _check(port, sc)


@pytest.mark.parametrize("seed", range(0, 24))
def test_random_triangles_tile32(gpu_lib, port, seed):
    sc = scenes.random_scene(1000 + seed, draw_mode=DrawMode.Triangle)
    _check(port, sc, tile=32)


@pytest.mark.parametrize("seed", range(0, 24))
def test_random_triangles_tile8(gpu_lib, port, seed):
    """8-px raster tiles: 16-px bins, every tile rasterized as four 8 x 8 quadrant CTAs."""
    sc = scenes.random_scene(2000 + seed, draw_mode=DrawMode.Triangle)
    _check(port, sc, tile=8)


@pytest.mark.parametrize("tile,split", [(8, False), (16, True), (32, False)])
def test_heavy_tiles_split_or_whole(gpu_lib, port, tile, split):
    """The dense mesh's silhouette tiles (hundreds of bin entries) and the dense soup: by
    quadrant CTAs (tile 8; tile 16 with the heavy-tile split) and whole (tile 32)."""
    _check(port, scenes.sphere_scene(8), tile=tile, split=split)
    sc = scenes.soup_scene(1 << 14, width=320, height=240, seed=12, raster=RasterMode.Adaptive)
    _check(port, sc, tile=tile, split=split)


@pytest.mark.parametrize("frame", [0, 1, 17, 42, 99])
def test_cube_frames(gpu_lib, port, frame):
    st = _check(port, scenes.cube_scene(frame))
    assert st["fragments"] > 0


@pytest.mark.parametrize("pose", [0, 3, 8, 13, 25, 31])
def test_sphere7_poses(gpu_lib, port, pose):
    st = _check(port, scenes.sphere_scene(pose))
    assert st["fragments"] > 0


@pytest.mark.parametrize("mode", [RasterMode.Span, RasterMode.Block, RasterMode.Adaptive])
def test_sphere5_all_modes(gpu_lib, port, mode):
    _check(port, scenes.sphere_scene(4, level=5, width=640, height=360, raster=mode))


def test_soup_adaptive_64k(gpu_lib, port):
    st = _check(port, scenes.soup_scene(1 << 16))
    assert st["fragments"] > 1_000_000


def test_batch_boundary_clip_fans(gpu_lib, port):
    """Clip fans are appended after the whole 1024-primitive batch (VertexProcessor.cpp:254-260)."""
    # 3000 triangles crossing the near plane straddle two batch boundaries.
    for seed in (7, 8):
        sc = scenes.random_scene(seed, direct=False, draw_mode=DrawMode.Triangle, n_prims=3000)
        _check(port, sc)


@pytest.mark.parametrize("seed", range(0, 60))
@pytest.mark.parametrize("mode", [DrawMode.Line, DrawMode.Point])
def test_random_lines_points(gpu_lib, port, seed, mode):
    sc = scenes.random_scene(2000 + seed, draw_mode=mode)
    _check(port, sc)


@pytest.mark.parametrize("mode", [DrawMode.Line, DrawMode.Point])
def test_many_lines_points_multi_batch(gpu_lib, port, mode):
    sc = scenes.random_scene(77, direct=False, draw_mode=mode, n_prims=2600)
    _check(port, sc)


@pytest.mark.parametrize("shape", [(480, 640), (37, 5), (1, 3), (1080, 1920)])
@pytest.mark.parametrize("rgba32f", [False, True])
def test_clear_target(gpu_lib, shape, rgba32f):
    """swr_clear_target fills colour, depth, drawPixel counts and winners (odd sizes too)."""
    import torch
    from softwarerenderer_gb300.device import DeviceTarget
    sc = scenes.cube_scene(0)
    sc.height, sc.width = shape
    if rgba32f:
        sc.ps = scenes.PS.DIFF
    tg = DeviceTarget(sc, clear_color=0.25 if rgba32f else 0x11223344, clear_depth=0.5)
    for t in (tg.color, tg.depth, tg.frag_count, tg.winner):
        t.view(torch.uint8).fill_(0xAB) if t.dtype != torch.uint8 else t.fill_(0xAB)
    tg.clear()
    torch.cuda.synchronize()
    c = tg.color.cpu().numpy()
    if rgba32f:
        assert (c == np.float32(0.25)).all()
    else:
        assert (c.view(np.uint32) == 0x11223344).all()
    assert (tg.depth.cpu().numpy() == np.float32(0.5)).all()
    assert (tg.frag_count.cpu().numpy() == 0).all() and (tg.winner.cpu().numpy() == -1).all()


def _prefilled_depth(scene, ref_depth, seed):
    """A depth buffer holding, per 16 x 16 tile, one of the scene's own visible depths (so
    whole primitives fall behind a tile's largest depth), with exact ties, per-pixel noise,
    NaN and -inf pixels mixed in."""
    rng = np.random.default_rng(seed)
    h, w = ref_depth.shape
    fin = ref_depth[np.isfinite(ref_depth)]
    if fin.size == 0:
        fin = np.array([0.5], np.float32)
    d = np.empty((h, w), np.float32)
    for ty in range(0, h, 16):
        for tx in range(0, w, 16):
            d[ty:ty + 16, tx:tx + 16] = fin[int(rng.integers(0, fin.size))]
    noise = rng.random((h, w))
    d[noise < 0.05] = ref_depth[noise < 0.05]                       # exact ties with a fragment
    d[(noise >= 0.05) & (noise < 0.08)] = np.inf
    d[(noise >= 0.08) & (noise < 0.09)] = np.nan
    d[(noise >= 0.09) & (noise < 0.095)] = -np.inf
    jit = (noise >= 0.5) & (noise < 0.6)
    d[jit] = np.nextafter(d[jit], np.float32(np.inf) if seed & 1 else np.float32(-np.inf))
    return d


def _check_prefilled(port, sc, seed):
    import torch
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    first, _ = oracle_render(port, sc)
    d = _prefilled_depth(sc, first["depth"], seed)
    t = scenes.Target(sc)
    t.depth[...] = d
    rst = port.draw(sc, t)
    ds = DeviceScene(sc)
    tg = DeviceTarget(sc)
    tg.depth.copy_(torch.from_numpy(d.copy()))
    gst = ds.draw(tg)
    got, ref = tg.to_host(), t.arrays()
    bad = diff(ref, got)
    assert not bad, f"{sc.name} {sc.raster.name}: " + "; ".join(describe(ref, got, k) for k in bad)
    assert gst["fragments"] == rst["fragments"], (gst, rst)
    return rst


@pytest.mark.parametrize("seed", range(0, 48))
def test_prefilled_depth_random(gpu_lib, port, seed):
    """Depth-tested draws onto a target that already holds depths: whole primitives lie
    behind a tile's largest depth from the first chunk on (the raster's tile depth cull)."""
    sc = scenes.random_scene(3000 + seed, draw_mode=DrawMode.Triangle, n_prims=400)
    _check_prefilled(port, sc, seed)


@pytest.mark.parametrize("mode", [RasterMode.Span, RasterMode.Block, RasterMode.Adaptive])
def test_dense_soup_all_modes(gpu_lib, port, mode):
    """16k soup triangles on 320 x 240 (about 90 layers per pixel): many chunks per tile, most
    primitives behind the tile's depths; also drawn over a prefilled depth buffer."""
    sc = scenes.soup_scene(1 << 14, width=320, height=240, seed=11, raster=mode)
    st = _check(port, sc)
    assert st["fragments"] > 20 * 320 * 240
    _check_prefilled(port, sc, 5)


@pytest.mark.parametrize("n_tris", [1000, 3000, 8000])
@pytest.mark.parametrize("mode", [RasterMode.Span, RasterMode.Block, RasterMode.Adaptive])
def test_overwrite_sliced_tiles(gpu_lib, port, n_tris, mode):
    """Overwrite shader (no depth test) with hundreds to thousands of primitives per tile:
    tiles above the in-kernel sort limit are rasterized in ordered slices by separate CTAs
    and merged (last writer, summed counts); smaller tiles stay whole."""
    sc = scenes.benchmark_scene(n_tris, seed=7)
    sc.raster = mode
    st = _check(port, sc)
    assert st["fragments"] > 0
