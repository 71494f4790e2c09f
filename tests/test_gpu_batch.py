"""Batched rendering (swr_draw_batch) against the CPU oracle, item by item.

A batch is one pass of the pipeline over all items; each item's target must equal what
the reference renders for that item alone (bit for bit), including items that share a
target (drawn in item order) and replays of the captured CUDA graph.
"""
import numpy as np
import pytest

from softwarerenderer_gb300 import scenes
from softwarerenderer_gb300.abi import DrawMode

from .parity import diff, oracle_render

pytestmark = pytest.mark.gpu


def _small_batch(n=10, seed=41):
    return scenes.batch_scenes(n, seed=seed, max_tris=3000, min_tris=20, sides=(48, 64, 96, 128),
                               texture_size=64)


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_oracle(gpu_lib, port, graph):
    from softwarerenderer_gb300.batch import BatchRenderer
    scs = _small_batch()
    br = BatchRenderer(scs, aux=True, graph=graph)
    for rep in range(2):  # second pass replays the graph
        br.clear()
        br.draw()
        for sc, tg in zip(scs, br.targets):
            ref, _ = oracle_render(port, sc)
            assert not diff(ref, tg.to_host()), (rep, sc.name)


def test_batch_shared_target_in_item_order(gpu_lib, port):
    """Items drawing into one colour buffer meet in one bin per tile, in item order."""
    from softwarerenderer_gb300.batch import BatchRenderer
    from softwarerenderer_gb300.device import DeviceTarget
    base = scenes.batch_scenes(4, seed=7, max_tris=2000, min_tris=200, sides=(96,), texture_size=64)
    shared = DeviceTarget(base[0], aux=True)
    br = BatchRenderer(base, aux=True, graph=False, targets=[shared] * len(base))
    br.clear()
    br.draw()
    # oracle: the same items drawn one after another into one host target
    t = scenes.Target(base[0])
    for sc in base:
        port.draw(sc, t)
    got = shared.to_host()
    # primitive ids restart per drawElements call, in the oracle and in the batch
    for k in ("color", "depth", "frag_count", "winner"):
        assert np.asarray(t.arrays()[k]).tobytes() == np.asarray(got[k]).tobytes(), k


@pytest.mark.parametrize("kind", ["cube", "sphere5", "sphere7"])
def test_graph_mode_single_draws(gpu_lib, port, kind):
    """Triangle drawElements in graph mode run as one-item batches: the first draw captures
    the graph, later draws (other poses, the other of two targets) replay it.  The dense
    1080p mesh (the bench's frame) also runs its heavy tiles as runs of chunks, whose
    completion counters must return to zero between replays."""
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    from .parity import diff, oracle_render
    mk = {"cube": lambda k: scenes.cube_scene(k),
          "sphere5": lambda k: scenes.sphere_scene(k, level=5, width=640, height=360),
          "sphere7": lambda k: scenes.sphere_scene(k)}[kind]
    sc0 = mk(0)
    ds = DeviceScene(sc0)
    ds.rast.ctx.set_graph_mode(True)
    tgs = [DeviceTarget(sc0), DeviceTarget(sc0)]
    for k in range(6):
        sc = mk(k)
        tg = tgs[k & 1]
        tg.clear()
        st = ds.draw(tg, mvp=sc.mvp)
        ref, rst = oracle_render(port, sc)
        got = tg.to_host()
        assert not diff(ref, got), (kind, k, diff(ref, got))
        assert st["fragments"] == rst["fragments"]


def test_full_batched_config_matches_oracle(gpu_lib, port):
    """The full batched workload exactly as bench.py builds it -- 256 deformed icospheres of
    100 to 200k triangles, targets of 256 to 1024 px, 512x512 RGBA8 textures -- in one
    swr_draw_batch captured as a CUDA graph and replayed: every item's colour, depth,
    per-pixel drawPixel count and winning primitive equal the oracle's, on the captured
    pass and on the replay (each item = one VertexProcessor::drawElements,
    VertexProcessor.cpp:78-120)."""
    from softwarerenderer_gb300.batch import BatchRenderer
    scs = scenes.batch_scenes(256)
    assert sum(len(sc.indices) // 3 for sc in scs) > 5_000_000
    refs = []
    for sc in scs:
        ref, st = oracle_render(port, sc)
        refs.append((ref, int(st["fragments"])))
    br = BatchRenderer(scs, aux=True, graph=True)
    total = sum(f for _, f in refs)
    for rep in range(2):  # capture, then replay
        br.clear()
        st = br.draw()
        assert int(st["fragments"]) == total, (rep, st["fragments"], total)
        for sc, tg, (ref, _) in zip(scs, br.targets, refs):
            assert not diff(ref, tg.to_host()), (rep, sc.name, diff(ref, tg.to_host()))


def test_autotuner_covers_tile_capacity_graph(gpu_lib, port):
    """The autotuner times tile x queue capacity x graph and its choice renders exactly."""
    from softwarerenderer_gb300 import autotune
    from softwarerenderer_gb300.batch import BatchRenderer
    scs = _small_batch(6, seed=45)
    best = autotune.tune(scs, reps=1, force=True)
    combos = {(t["tile"], t["capacity"], t["graph"]) for t in best["tried"] if t["geometry"] == "kernels"}
    assert combos == {(t, c, g) for t in autotune.TILES for c in autotune.CAPACITIES for g in autotune.GRAPHS}
    assert any(t["geometry"] == "persistent" for t in best["tried"])
    br = BatchRenderer(scs, aux=True, tile=best["tile"], graph=best["graph"])
    autotune.apply_config(br, best)
    br.clear()
    br.draw()
    for sc, tg in zip(scs, br.targets):
        ref, _ = oracle_render(port, sc)
        assert not diff(ref, tg.to_host()), sc.name


@pytest.mark.parametrize("graph", [False, True])
def test_persistent_geometry_matches_oracle(gpu_lib, port, graph):
    """Vertex shading and assembly as one cooperative launch with grid barriers
    (swr_set_persistent_geometry): a batch of meshes (captured and replayed) and single
    draws with near-plane clipping and several 1024-triangle batches render exactly."""
    from softwarerenderer_gb300.batch import BatchRenderer
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    scs = _small_batch(8, seed=47)
    br = BatchRenderer(scs, aux=True, graph=graph)
    br.ctx.set_persistent_geometry(True)
    for rep in range(2):
        br.clear()
        br.draw()
        for sc, tg in zip(scs, br.targets):
            ref, _ = oracle_render(port, sc)
            assert not diff(ref, tg.to_host()), (rep, sc.name)
    for sc in (scenes.sphere_scene(29), scenes.random_scene(5001, direct=False, draw_mode=DrawMode.Triangle, n_prims=3000)):
        ds = DeviceScene(sc)
        ds.rast.ctx.set_persistent_geometry(True)
        tg = DeviceTarget(sc)
        st = ds.draw(tg)
        ref, rst = oracle_render(port, sc)
        assert st["fragments"] == rst["fragments"]
        assert not diff(ref, tg.to_host()), sc.name
