"""Autotuner for batched rendering: times every configuration of a batch layout on the
current GPU and caches the fastest in softwarerenderer_gb300/_build/autotune.json, keyed by
the layout signature and the GPU name.

Axes (the full product is timed and reported in `tried`):
  tile      raster tile edge: 32 or 16 px (one CTA per tile) or 8 px (16-px bins, every tile
            rasterized as four 8 x 8 CTAs)
  graph     CUDA-graph capture and replay of the batch's kernel sequence, or plain launches
  capacity  how the primitive and bin-entry queues are sized:
              "grown"  automatically: sized from the submitted triangle count and grown
                       after a draw overflows them (one retried draw)
              "exact"  pre-sized once to what this batch needs (swr_set_queue_capacity)
              "2x"     pre-sized to twice that
            The primitive queue's size also sets the primitive segments of the binning
            (a segment spans capacity / 32 primitive ids), so it changes the sort work.
  geometry  the best of the above once more with vertex shading and assembly as one
            persistent cooperative launch ("persistent") instead of three kernels ("kernels")
"""
import hashlib
import json
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(HERE, "_build", "autotune.json")
TILES = (8, 16, 32)
GRAPHS = (True, False)
CAPACITIES = ("grown", "exact", "2x")


def signature(scenes):
    h = hashlib.sha256()
    for sc in scenes:
        h.update(repr((len(sc.indices), sc.width, sc.height, int(sc.raster), int(sc.vs), int(sc.ps))).encode())
    return h.hexdigest()[:24]


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def _time(br, reps):
    for _ in range(2):
        br.clear()
        br.draw()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        br.clear()
        br.draw(sync=False)
    e.record()
    torch.cuda.synchronize()
    rc, _ = br.ctx.finish()
    assert rc == 0, rc
    return s.elapsed_time(e) / reps


def needed_capacity(br):
    """Primitive and bin-entry counts of one draw of the batch (after any retry)."""
    br.clear()
    st = br.draw()
    return int(st["primitives"]), int(st["bin_pairs"])


def apply_config(br, best):
    """Configure a renderer built with best["tile"] / best["graph"] as tuned."""
    apply_capacity(br, best["capacity"], (best["need"]["primitives"], best["need"]["bin_entries"]))
    br.ctx.set_persistent_geometry(best.get("geometry") == "persistent")


def apply_capacity(br, capacity, need):
    """Configure a renderer's queues for one `capacity` setting (see the module doc)."""
    prims, pairs = need
    if capacity == "grown":
        br.ctx.set_queue_capacity(0, 0)
    else:
        k = 1 if capacity == "exact" else 2
        br.ctx.set_queue_capacity(max(1, k * prims), max(1, k * pairs))


def tune(scenes, reps=3, force=False):
    """Best configuration for this batch layout on this GPU (cached)."""
    from .batch import BatchRenderer
    key = f"{torch.cuda.get_device_name()}|{signature(scenes)}"
    cache = _load()
    if key in cache and not force:
        return cache[key]
    results = []
    need = None
    for tile in TILES:
        br = BatchRenderer(scenes, tile=tile, graph=True, pooled=True)
        if need is None:
            need = needed_capacity(br)
        for capacity in CAPACITIES:
            for graph in GRAPHS:
                br.ctx.set_graph_mode(graph)
                apply_capacity(br, capacity, need)
                ms = _time(br, reps)
                results.append((ms, {"tile": tile, "graph": graph, "capacity": capacity}))
        del br
    for _, c in results:
        c["geometry"] = "kernels"
    # the best configuration once more with the persistent geometry front end (vertex
    # shading and assembly as one cooperative launch instead of three kernels)
    ms, best = min(results, key=lambda r: r[0])
    br = BatchRenderer(scenes, tile=best["tile"], graph=best["graph"], pooled=True)
    apply_capacity(br, best["capacity"], need)
    br.ctx.set_persistent_geometry(True)
    results.append((_time(br, reps), dict(best, geometry="persistent")))
    del br
    ms, best = min(results, key=lambda r: r[0])
    entry = dict(best, ms=round(ms, 4), need={"primitives": need[0], "bin_entries": need[1]},
                 tried=[dict(c, ms=round(t, 4)) for t, c in results])
    cache[key] = entry
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    with open(CACHE, "w") as f:
        json.dump(cache, f, indent=1)
    return entry
