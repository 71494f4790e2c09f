"""Autotuner for batched rendering: times the candidate configurations of a batch layout
(screen tile edge 16 / 32 px, CUDA-graph replay on / off) on the current GPU and caches
the fastest in softwarerenderer_gb300/_build/autotune.json, keyed by the layout signature
and the GPU name.  Scratch-queue capacities are sized by the first (warm-up) draw of each
candidate, which grows the context's queues to exactly what the batch needs."""
import hashlib
import json
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(HERE, "_build", "autotune.json")
CANDIDATES = [{"tile": 16, "graph": True}, {"tile": 32, "graph": True}, {"tile": 16, "graph": False}]


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
    br.ctx.finish()
    return s.elapsed_time(e) / reps


def tune(scenes, reps=3, force=False):
    """Best configuration for this batch layout on this GPU (cached)."""
    from .batch import BatchRenderer
    key = f"{torch.cuda.get_device_name()}|{signature(scenes)}"
    cache = _load()
    if key in cache and not force:
        return cache[key]
    results = []
    for cand in CANDIDATES:
        br = BatchRenderer(scenes, tile=cand["tile"], graph=cand["graph"], pooled=True)
        ms = _time(br, reps)
        results.append((ms, cand))
        del br
    ms, best = min(results, key=lambda r: r[0])
    entry = dict(best, ms=round(ms, 4), tried=[dict(c, ms=round(t, 4)) for t, c in results])
    cache[key] = entry
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    with open(CACHE, "w") as f:
        json.dump(cache, f, indent=1)
    return entry
