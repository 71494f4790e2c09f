"""Shared helpers of the parity tests: render a scene with the oracle and the GPU."""
import numpy as np

from softwarerenderer_gb300 import scenes


def oracle_render(port, scene, threads=0):
    t = scenes.Target(scene)
    st = port.draw(scene, t, threads=threads)
    return t.arrays(), st


def gpu_render(scene, tile=16, split=False, slicing=-1):
    """tile: 8, 16 or 32 (swr_set_tile_size); split: heavy 16-px tiles as quadrant CTAs (in
    place of the depth-min shaders' heavy-tile runs); slicing: swr_set_tile_slicing's chunk
    threshold for those runs (-1: the shader's default, 0: whole tiles)."""
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    ds = DeviceScene(scene, tile=tile)
    if split:
        slicing = 0
    if slicing != -1:
        ds.rast.ctx.set_tile_slicing(slicing)
    if split:
        ds.rast.ctx.set_tile_split(True)
    tg = DeviceTarget(scene)
    st = ds.draw(tg)
    return tg.to_host(), st


def diff(a, b):
    """Names of the buffers that differ bit for bit."""
    bad = []
    for k in a:
        if np.asarray(a[k]).tobytes() != np.asarray(b[k]).tobytes():
            bad.append(k)
    return bad


def describe(a, b, k):
    x, y = np.asarray(a[k]), np.asarray(b[k])
    if x.ndim == 3:
        m = np.any(x.view(np.uint32) != y.view(np.uint32), axis=-1)
    else:
        m = x.view(np.uint32) != y.view(np.uint32)
    ys, xs = np.nonzero(m)
    return f"{k}: {m.sum()} pixels differ, first at {list(zip(xs[:5].tolist(), ys[:5].tolist()))}"
