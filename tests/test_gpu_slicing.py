"""GPU parity of heavy-tile slicing (swr_set_tile_slicing).

With the depth-min shaders (Lambert, Lambert-textured, vertex colour, nearest texture) a
tile of more than k raster chunks of bin entries (k = 1 here, the Lambert shader's default)
is rasterized by four CTAs, each over a run of whole chunks from the draw's starting
framebuffer, and the runs are merged in primitive order.  The piles of triangles here hold
tiles of 150 to 800 bin entries, at six constant depths, so equal depths in different runs
are common: the first fragment of the smallest depth must still win, as in the reference's
sequential drawPixel calls (PixelShaderBase.h:116 through Rasterizer.h:225-306).  Tiles of
more than 512 entries take the ordered-bin path, the others sort their own bin in each run.
"""
import numpy as np
import pytest

from softwarerenderer_gb300 import scenes
from softwarerenderer_gb300.abi import PS, RasterMode

from .parity import describe, diff, gpu_render, oracle_render

pytestmark = pytest.mark.gpu

DEPTH_MIN_SHADERS = [PS.VCOLOR, PS.LAMBERT, PS.LAMBERT_TEX, PS.TEX_NEAREST]


@pytest.mark.parametrize("n", [700, 2400])
@pytest.mark.parametrize("raster", [RasterMode.Block, RasterMode.Span, RasterMode.Adaptive])
@pytest.mark.parametrize("ps", DEPTH_MIN_SHADERS)
def test_sliced_pile_matches_oracle(gpu_lib, port, ps, raster, n):
    sc = scenes.stack_scene(int(ps) * 10 + int(raster), n, ps=ps, raster=raster)
    ref, rst = oracle_render(port, sc)
    got, gst = gpu_render(sc, slicing=1)
    bad = diff(ref, got)
    assert not bad, "; ".join(describe(ref, got, k) for k in bad)
    assert gst["fragments"] == rst["fragments"]
    # whole tiles (one CTA each) give the same buffers, and no fewer depth-test passes are
    # counted by the runs than by the sequential walk
    whole, wst = gpu_render(sc, slicing=0)
    assert not diff(whole, got)
    assert gst["passes"] >= wst["passes"]


@pytest.mark.parametrize("tile", [16, 32])
def test_sliced_dense_mesh_matches_whole_tiles(gpu_lib, port, tile):
    """The dense mesh's silhouette tiles (hundreds of bin entries) with and without slicing,
    and against the oracle."""
    sc = scenes.sphere_scene(11)
    ref, _ = oracle_render(port, sc)
    got, _ = gpu_render(sc, tile=tile, slicing=1)
    whole, _ = gpu_render(sc, tile=tile, slicing=0)
    assert not diff(ref, got), [describe(ref, got, k) for k in diff(ref, got)]
    assert not diff(whole, got)


@pytest.mark.parametrize("graph", [False, True])
def test_sliced_batch_of_dense_meshes(gpu_lib, port, graph):
    """A batch of three dense-mesh poses (the Lambert shader: heavy-tile runs on by default),
    one target each: runs of tiles of different targets in one raster launch, captured and
    replayed."""
    from softwarerenderer_gb300.batch import BatchRenderer
    scs = [scenes.sphere_scene(p, level=6, width=960, height=540) for p in (2, 9, 20)]
    br = BatchRenderer(scs, aux=True, graph=graph)
    refs = [oracle_render(port, sc)[0] for sc in scs]
    for rep in range(2):  # with graph mode the second pass replays the graph
        br.clear()
        br.draw()
        for sc, tg, ref in zip(scs, br.targets, refs):
            got = tg.to_host()
            assert not diff(ref, got), (rep, sc.name, [describe(ref, got, k) for k in diff(ref, got)])
