"""Generate tests/golden/golden.json by running the reference library itself.

The reference's own sources (src/renderer of trenki2/SoftwareRenderer, and for the Box
example's frames the mip-mapped sampler of src/examples/Texture.h) are compiled unmodified
with oracle/ref_harness.cpp (make -C oracle ref; needs the reference checkout named by
SWR_REFERENCE).  For every scene spec below the harness renders the
seeded scene and the fixture records the reference's counters and a SHA-256 of each
buffer the pixel shader writes (colour, depth, per-pixel drawPixel count, winning
primitive).  Scenes are rebuilt from their specs by softwarerenderer_gb300.scenes, which is
bit-reproducible across platforms, so the fixture is small and checks full-size renders.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from softwarerenderer_gb300 import scenes  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")


def specs():
    out = [{"kind": "random", "seed": s} for s in range(300)]
    out += [{"kind": "random", "seed": 5000 + s, "direct": False, "draw_mode": 2, "n_prims": 3000}
            for s in range(4)]  # several 1024-primitive batches with clip fans
    out += [{"kind": "cube", "frame": f} for f in range(100)]
    out += [{"kind": "sphere", "pose": p} for p in range(32)]
    out += [{"kind": "sphere", "pose": 4, "level": 5, "width": 640, "height": 360, "raster": m}
            for m in (0, 1, 2)]
    out += [{"kind": "soup", "n": 1 << 16}, {"kind": "soup", "n": 1 << 20}]
    out += [{"kind": "benchmark"}]
    # the Box example's mip-mapped anisotropic sampler, and the perspective derivatives
    out += [{"kind": "box", "frame": f} for f in range(16)]
    out += [{"kind": "deriv", "frame": f, "raster": m} for f in range(8) for m in (0, 1, 2)]
    # items of the 256-mesh batched workload (scenes.batch_scenes(256)): the first four,
    # the three smallest (103-108 triangles) and the three largest (193k-198k triangles)
    out += [{"kind": "batch", "item": i} for i in (0, 1, 2, 3, 26, 98, 196, 79, 191, 69)]
    return out


def digest(arrays):
    return {k: hashlib.sha256(memoryview(v).cast("B")).hexdigest()[:32] for k, v in arrays.items()}


def main():
    ref = oracle.load("ref")
    res = []
    t0 = time.time()
    for sp in specs():
        sc = scenes.scene_from_spec(sp)
        tg = scenes.Target(sc)
        st = ref.draw(sc, tg)
        res.append({"spec": sp, "name": sc.name, "inputs": scenes.scene_digest(sc), "stats": {k: int(st[k]) for k in ("fragments", "outside", "primitives")},
                    "sha256": digest(tg.arrays())})
    with open(OUT, "w") as f:
        json.dump({"generator": "reference library (src/renderer; Box frames: src/examples/Texture.h) via "
                                "oracle/ref_harness.cpp",
                   "cases": res}, f, indent=0)
    print(f"{len(res)} cases in {time.time() - t0:.1f} s -> {OUT}")


if __name__ == "__main__":
    main()
