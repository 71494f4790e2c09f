"""Host-side checks that need no GPU: the C ABI library exports what its header declares,
product code never reaches the oracle, scenes are deterministic, and the replica reduction
of the benchmark works across two gloo ranks."""
import ctypes
import os
import re
import shutil
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "swr_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:SWR_API\s+)?(?:int|const char\*)\s+(swr_\w+)\s*\(", txt, re.M)))


def test_header_declares_the_reference_api():
    names = declared_symbols()
    for n in ("swr_create", "swr_destroy", "swr_set_viewport", "swr_set_depth_range", "swr_set_cull_mode",
              "swr_set_vertex_shader", "swr_set_vertex_attrib_pointer", "swr_draw_elements",
              "swr_set_raster_mode", "swr_set_scissor_rect", "swr_set_pixel_shader", "swr_draw_list",
              "swr_finish"):
        assert n in names


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="needs nvcc to build the library")
def test_library_exports_every_declared_symbol():
    from softwarerenderer_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)  # loading needs no GPU; nothing is called
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_product_code_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "softwarerenderer_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in txt and "from oracle" not in txt, f
                assert "oracle_abi" not in txt and "liboracle" not in txt, f


def test_scene_generation_is_deterministic():
    from softwarerenderer_gb300 import scenes
    a = scenes.scene_digest(scenes.sphere_scene(3, level=4))
    b = scenes.scene_digest(scenes.sphere_scene(3, level=4))
    assert a == b
    assert scenes.scene_digest(scenes.random_scene(1)) != scenes.scene_digest(scenes.random_scene(2))


def test_icosphere_counts():
    from softwarerenderer_gb300 import scenes
    p, f = scenes.icosphere(7)
    assert p.shape == (163842, 3) and f.shape == (327680, 3)
    n = np.sqrt((p * p).sum(1))
    assert np.allclose(n, 1.0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _replica_worker(rank, world, port, out):
    import torch.distributed as dist
    import sys
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ms, frags = [10.0, 12.5][rank], [1000, 3000][rank]
    res = bench.reduce_replicas(ms, frags, dist, "cpu")
    out.put((rank, res))
    dist.destroy_process_group()


def test_replica_reduction_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == (12.5, 4000.0)
