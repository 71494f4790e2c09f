"""Error paths of the C ABI: queue overflow and allocation failure.

The reference has only asserts here (VertexProcessor.cpp:39, :69) and grows std::vectors
without limit; the GPU pipeline sizes device queues ahead of a draw instead.  A draw that
needs more than a queue holds is skipped on the device: swr_finish reports SWR_EOVERFLOW,
the targets keep every byte they had, the queue is grown, and the retried draw must equal
the CPU oracle bit for bit.  A device allocation that fails (simulated with the context's
memory budget, swr_set_memory_limit) returns SWR_ENOMEM before anything is queued.
"""
import numpy as np
import pytest

from softwarerenderer_gb300 import scenes

from .parity import diff

pytestmark = pytest.mark.gpu

CLEAR_COLOR, CLEAR_DEPTH = 0x01020304, 0.97


def _scene():
    # level-5 icosphere, 640x360, Block: ~5k primitives and ~15k bin entries after culling
    return scenes.sphere_scene(4, level=5, width=640, height=360)


def _oracle(port, sc):
    t = scenes.Target(sc, clear_color=CLEAR_COLOR, clear_depth=CLEAR_DEPTH)
    st = port.draw(sc, t)
    return t.arrays(), st


def _target(sc):
    from softwarerenderer_gb300.device import DeviceTarget
    return DeviceTarget(sc, clear_color=CLEAR_COLOR, clear_depth=CLEAR_DEPTH)


@pytest.mark.parametrize("which", ["bin_entries", "primitives"])
def test_overflow_leaves_target_untouched_then_retry_matches_oracle(gpu_lib, port, which):
    from softwarerenderer_gb300 import _lib
    from softwarerenderer_gb300.device import DeviceScene
    sc = _scene()
    ds = DeviceScene(sc)
    ctx = ds.rast.ctx
    if which == "bin_entries":
        ctx.set_queue_capacity(0, 1000)
    else:
        ctx.set_queue_capacity(100, 0)
    tg = _target(sc)
    before = tg.to_host()
    ds.draw(tg, sync=False)
    rc, st = ctx.finish()
    assert rc == _lib.SWR_EOVERFLOW, (which, rc, st)
    assert st["fragments"] == 0
    after = tg.to_host()
    assert not diff(before, after), diff(before, after)
    prims, pairs = ctx.queue_capacity()
    assert (pairs if which == "bin_entries" else prims) > (1000 if which == "bin_entries" else 100)
    st2 = ds.draw(tg)  # grown queue: the retry succeeds
    ref, rst = _oracle(port, sc)
    assert st2["fragments"] == rst["fragments"]
    assert not diff(ref, tg.to_host()), diff(ref, tg.to_host())


def test_batch_overflow_then_retry_matches_oracle(gpu_lib, port):
    """The same through swr_draw_batch (graph mode): the overflowed layout is recaptured."""
    from softwarerenderer_gb300 import _lib
    from softwarerenderer_gb300.batch import BatchRenderer
    from .parity import oracle_render
    scs = scenes.batch_scenes(6, seed=43, max_tris=3000, min_tris=200, sides=(64, 96), texture_size=64)
    br = BatchRenderer(scs, aux=True, graph=True)
    br.ctx.set_queue_capacity(0, 512)
    br.clear()
    before = [tg.to_host() for tg in br.targets]
    rc = br.ctx.L.swr_draw_batch(br.ctx.h, br.items, len(scs), ctypes_stream())
    assert rc == 0
    rc, st = br.ctx.finish()
    assert rc == _lib.SWR_EOVERFLOW, rc
    for b, tg in zip(before, br.targets):
        assert not diff(b, tg.to_host())
    br.draw()
    for rep in range(2):
        if rep:
            br.clear()
            br.draw()
        for sc, tg in zip(scs, br.targets):
            ref, _ = oracle_render(port, sc)
            assert not diff(ref, tg.to_host()), (rep, sc.name)


def ctypes_stream():
    from softwarerenderer_gb300.renderer import _stream
    return _stream()


def test_memory_limit_returns_enomem_and_queues_nothing(gpu_lib, port):
    from softwarerenderer_gb300 import _lib
    from softwarerenderer_gb300.device import DeviceScene
    sc = _scene()
    ds = DeviceScene(sc)
    ctx = ds.rast.ctx
    held = ctx.memory_used()
    ctx.set_memory_limit(held + 64 * 1024)  # far below what the draw's queues need
    tg = _target(sc)
    before = tg.to_host()
    with pytest.raises(_lib.SwrError) as e:
        ds.draw(tg)
    assert e.value.code == _lib.SWR_ENOMEM
    assert ctx.memory_used() <= held + 64 * 1024
    rc, st = ctx.finish()  # nothing was queued: no fragments, no error bits
    assert rc == 0 and st["fragments"] == 0
    assert not diff(before, tg.to_host())
    ctx.set_memory_limit(0)
    st = ds.draw(tg)
    ref, rst = _oracle(port, sc)
    assert st["fragments"] == rst["fragments"]
    assert not diff(ref, tg.to_host())
    assert ctx.memory_used() > held + 64 * 1024


def test_persistent_geometry_barrier_wait_runs_out(gpu_lib, port):
    """The persistent geometry launch's grid barriers wait a bounded time: started from an
    arrival count that can never complete (a test hook, no GPU fault), every CTA gives up
    after about a second and the draw reports SWR_ECUDA with its target untouched; the same
    context then draws exactly."""
    import ctypes
    from softwarerenderer_gb300 import _lib
    from softwarerenderer_gb300.device import DeviceScene
    sc = _scene()
    ds = DeviceScene(sc)
    ctx = ds.rast.ctx
    ctx.set_persistent_geometry(True)
    ctx.L.swr_test_stall_geometry_barrier.argtypes = [ctypes.c_void_p, ctypes.c_int]
    ctx.L.swr_test_stall_geometry_barrier.restype = ctypes.c_int
    assert ctx.L.swr_test_stall_geometry_barrier(ctx.h, 1) == 0
    tg = _target(sc)
    before = tg.to_host()
    ds.draw(tg, sync=False)
    rc, st = ctx.finish()
    assert rc == _lib.SWR_ECUDA, rc
    assert st["flags"] & 256  # SWR_F_BARRIER_TIMEOUT
    assert st["fragments"] == 0
    assert not diff(before, tg.to_host())
    assert ctx.L.swr_test_stall_geometry_barrier(ctx.h, 0) == 0
    st2 = ds.draw(tg)
    ref, rst = _oracle(port, sc)
    assert st2["fragments"] == rst["fragments"]
    assert not diff(ref, tg.to_host())
