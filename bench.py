#!/usr/bin/env python
"""Benchmark of the GB300 rasterization pipeline on the dense-mesh workload.

Workload: icosphere subdivision 7 (163,842 vertices / 327,680 triangles; position+normal
24 B and uv 8 B per vertex, uint32 indices), 1920x1080 target, RasterMode Block, CullMode
CW, Lambert + procedural checker pixel shader with FP32 depth test, 32 seeded camera poses
of which 3 put the near plane through the mesh.  One step = one frame: clear colour and
depth, set the pose, VertexProcessor::drawElements over all 983,040 indices.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

`value` is shaded fragments per second over the K timed frames (device time from CUDA
events around each frame, L2 flushed with a 256 MiB write before every frame); Mtris/s is
reported beside it.  `e2e` repeats the measurement through the public API with the
step's vertex/index buffers copied host->device from pinned memory and the colour buffer
copied back inside the timed region.  `--impl reference` times the reference algorithm on
the host cores instead: the reference library compiled from its own sources where that
build exists on the machine (oracle/_ref), else the CPU oracle port (the same OpenMP placement; at one
thread it skips OpenMP's team fork per triangle and runs as fast as the reference built
without OpenMP).  With N > 1 (torchrun) every rank renders the same frames on its own
GPU: replicas, no collective on the data path.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gfrags/s & Mtris/s at 1080p on 1 GB300; batched views/s, fwd+bwd/s vs plain"
WORKLOAD = ("icosphere subdivision 7 (163,842 v / 327,680 t, pos+normal 24 B + uv 8 B, uint32 "
            "indices), 1920x1080, RasterMode Block, CullMode CW, Lambert + checker, FP32 depth "
            "test, 32 seeded poses (3 near-plane clipped), 1 frame per step")


# Means over the headline k_raster launches of the 32 timed poses, from ncu captures of
# `python bench.py --steps 32 --warmup 3 --no-...` (profiles/k_raster_lambert_sphere7_1080p.md):
# dram__bytes_read.sum + dram__bytes_write.sum with the L2 as the frame's earlier kernels
# leave it (--cache-control none: the setup records and the cleared target are still in L2;
# the writes are dirty lines of the L2 flush buffer that the launch's own stores evict) and
# with the L2 flushed before every launch (ncu's default), and smsp__inst_executed.sum (warp
# instructions) per launch.
NCU_DRAM_BYTES_PER_LAUNCH = {"raster": 7464800}
NCU_DRAM_BYTES_COLD = {"raster": 19747224}
NCU_WARP_INST_PER_LAUNCH = {"raster": 35816046}
SMS = 152


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def frame_bytes(n_idx, vertex_bytes, pixels, frags, passes, texel_bytes=0):
    """Algorithmic bytes of one frame (index + vertex streams read once, colour+depth
    clear/store per target pixel, depth read per fragment, depth+RGBA8 write per pass)."""
    return 4 * n_idx + vertex_bytes + 8 * pixels + 4 * frags + 8 * passes + texel_bytes * frags


def cpu_engine():
    """The CPU implementation timed as the reference: the reference library itself
    (oracle/_ref, compiled from its own sources with OpenMP) where it was built on this
    machine, else the oracle port (its operation-for-operation restatement, same OpenMP
    placement).  The reference's sources are not on every benchmark machine."""
    from oracle import oracle
    if os.path.exists(oracle.PATHS["ref"]):
        try:
            return oracle.load("ref"), "reference"
        except OSError:
            pass
    return oracle.load("port"), "port"


def cpu_baseline(min_seconds=10.0, max_frames=32):
    """The reference algorithm on host cores, best of 1 thread and all."""
    from softwarerenderer_gb300 import scenes
    port, kind = cpu_engine()
    ncores = os.cpu_count() or 1
    results = {}
    for threads in sorted({1, ncores}):
        frags, t_tot, n = 0, 0.0, 0
        while n < max_frames and (t_tot < min_seconds / 2 or n < 2):
            sc = scenes.sphere_scene(n % 32)
            tg = scenes.Target(sc, aux=False)
            t0 = time.perf_counter()
            st = port.draw(sc, tg, threads=threads)
            t_tot += time.perf_counter() - t0
            frags += st["fragments"]
            n += 1
        results[threads] = (frags / t_tot / 1e9, n, t_tot, 327680 * n / t_tot / 1e6)
    best = max(results, key=lambda k: results[k][0])
    v, n, t, mtris = results[best]
    # the reference's Benchmark.cpp program: one drawElements of its scene, wall time, the
    # better of 1 thread and every thread (Span mode gains nothing from OpenMP)
    bsc = scenes.benchmark_scene()
    bres = {}
    for threads in sorted({1, ncores}):
        btg = scenes.Target(bsc, aux=False)
        t0 = time.perf_counter()
        bst = port.draw(bsc, btg, threads=threads)
        bres[threads] = ((time.perf_counter() - t0) * 1e3, int(bst["fragments"]))
    bth = min(bres, key=lambda k: bres[k][0])
    bms, bfr = bres[bth]
    return {"value": v, "unit": "Gfrags/s", "cores": best, "kind": kind,
            "sample": f"{n} of the 32 poses, {t:.1f} s of CPU time at {best} thread(s) "
                      f"(best of 1 and {ncores} threads; OpenMP as in the reference)",
            "mtris_per_s": mtris,
            "by_threads": {str(k): round(r[0], 4) for k, r in results.items()},
            "benchmark_program": {"ms": round(bms, 1), "threads": bth, "fragments": bfr,
                                  "gfrags_per_s": round(bfr / (bms / 1e3) / 1e9, 4),
                                  "ms_by_threads": {str(k): round(r[0], 1) for k, r in bres.items()}}}


def run_reference(args, rank):
    """Reference arm: the reference algorithm (CPU oracle port, OpenMP where the reference
    has it) on the host's cores, W warm-up and K timed frames of the same workload.  The
    warm-up frames time both 1 thread and every host thread and the faster count is used
    (the reference forks its OpenMP team per triangle half, which on this mesh of 2-pixel
    triangles makes every-thread runs slower than one thread)."""
    if rank != 0:
        return
    from softwarerenderer_gb300 import scenes
    port, kind = cpu_engine()
    allc = os.cpu_count() or 1
    # the first warm-up frame (cold caches, thread-pool start) is not compared; the order of
    # the thread counts alternates so neither always follows the other's idle spin-wait
    spent = {}
    counts = sorted({1, allc})
    for k in range(args.warmup):
        sc = scenes.sphere_scene(k % 32)
        for th in (counts if k % 2 == 0 else counts[::-1]):
            t0 = time.perf_counter()
            port.draw(sc, scenes.Target(sc, aux=False), threads=th)
            if k > 0:
                spent[th] = spent.get(th, 0.0) + time.perf_counter() - t0
    ncores = min(spent, key=spent.get) if spent else 1
    frags, t_tot = 0, 0.0
    for k in range(args.steps):
        sc = scenes.sphere_scene(k % 32)
        tg = scenes.Target(sc, aux=False)
        t0 = time.perf_counter()
        st = port.draw(sc, tg, threads=ncores)
        t_tot += time.perf_counter() - t0
        frags += st["fragments"]
    value = frags / t_tot / 1e9
    cb = {"value": value, "unit": "Gfrags/s", "cores": ncores, "kind": kind,
          "sample": f"{args.steps} frames (poses 0..{min(args.steps, 32) - 1}), {t_tot:.1f} s"}
    line = {"metric": METRIC, "value": value, "unit": "Gfrags/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_tot / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded icosphere and poses)", "impl": "reference",
            "config": {"workload": WORKLOAD,
                       "engine": ("the reference library (VertexProcessor+Rasterizer) compiled with OpenMP"
                                  if kind == "reference" else "CPU oracle port of VertexProcessor+Rasterizer"),
                       "threads": ncores, "threads_tried": counts},
            "mtris_per_s": 327680 * args.steps / t_tot / 1e6,
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "Gfrags/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def reduce_replicas(ms, frags, dist=None, device="cpu"):
    """Whole-job timing of independent replicas: the slowest rank's time and the fragments
    of all ranks (no collective touches the rendering itself)."""
    if dist is None:
        return float(ms), float(frags)
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    f = torch.tensor([frags], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(f, op=dist.ReduceOp.SUM)
    return float(t[0]), float(f[0])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--tile", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-rendering section")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiable-rendering section")
    ap.add_argument("--no-program", action="store_true", help="skip the Benchmark.cpp program section")
    ap.add_argument("--no-soup", action="store_true", help="skip the 4K triangle-soup section")
    ap.add_argument("--no-graph", action="store_true", help="time the frames without CUDA graph replay")
    ap.add_argument("--section", default="all", choices=["all", "batch", "diff", "benchmark_program", "soup"],
                    help="run one side section alone and print its JSON (profiling); 'all' is the bench line")
    args = ap.parse_args()
    assert args.warmup >= 3, "at least 3 warm-up steps"
    if args.section != "all":
        import torch
        from softwarerenderer_gb300 import build
        if not os.path.exists(build.LIB):
            build.build()
        fn = {"batch": run_batched, "diff": run_diff, "benchmark_program": run_benchmark_program,
              "soup": run_soup}[args.section]
        print(json.dumps(fn(torch, steps=args.steps)))
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(local)

    from softwarerenderer_gb300 import build, scenes
    if not os.path.exists(build.LIB):
        build.build()
    from softwarerenderer_gb300.abi import make_uniforms
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget

    sc = scenes.sphere_scene(0)
    poses = [scenes.sphere_scene(p).mvp for p in range(scenes.SPHERE_POSES)]
    ds = DeviceScene(sc, tile=args.tile)
    tg = DeviceTarget(sc, aux=False)
    ctx = ds.rast.ctx
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")  # 256 MiB > L2
    stream = torch.cuda.current_stream()
    ds.bind(tg)

    def frame(k):
        tg.clear()
        ds.rast.setUniforms(ds.uniforms(tg, poses[k % len(poses)]))
        ds.vp.drawElements(sc.draw_mode, ds.indices.numel(), ds.indices, sync=False)

    # warm-up (also grows the scratch queues to their steady-state size), then the same
    # frames with graph mode on: the first one captures the draw's CUDA graph
    for k in range(args.warmup):
        frame(k)
        rc, _ = ctx.finish()
        if rc == 3:  # overflow: queues grown, run again
            frame(k)
            ctx.finish()
    ctx.set_graph_mode(not args.no_graph)
    for k in range(args.warmup):
        frame(k)
        ctx.finish()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.fill_(k)
            starts[k].record(stream)
            frame(k)
            ends[k].record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    rc, st = ctx.finish()
    assert rc == 0, f"draw status {rc}"
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    # Stage times: the same frames again, launch by launch with the library's per-stage
    # CUDA events on the draw's stream (profiling bypasses graph replay).
    ctx.set_profiling(True)
    ctx.stage_times()
    ps0, ps1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ps0.record(stream)
    for k in range(args.steps):
        flush.fill_(k)
        frame(k)
    ps1.record(stream)
    torch.cuda.synchronize()
    rc2, _ = ctx.finish()
    assert rc2 == 0, f"draw status {rc2}"
    stages = ctx.stage_times()
    ctx.set_profiling(False)
    ms_max = ms
    frags, passes = st["fragments"], st["passes"]
    ms_max, frags_all = reduce_replicas(ms, frags, dist, "cuda")
    value = frags_all / (ms_max / 1e3) / 1e9
    mtris = 327680 * args.steps * world / (ms_max / 1e3) / 1e6

    # roofline of the dominant kernel (by stage time)
    hbm, peak_kind = peaks()
    dom = max(stages, key=stages.get)
    n_idx = ds.indices.numel()
    vbytes = sum(b.numel() for b, _ in ds.attribs)
    pixels = sc.width * sc.height
    per_launch = {
        # fragment terms: depth read per drawPixel call, depth + RGBA8 write per colour write
        "raster": (4 * frags + 8 * passes) / args.steps,
        "vertex": vbytes + sc.vertex_count() * 64,   # attribute streams read + post-transform records written
        "assemble": 4 * n_idx,
        "setup": 0, "bin": 0,
    }
    alg = per_launch.get(dom, 0)
    t_launch = stages[dom] / args.steps / 1e3
    achieved = alg / t_launch / 1e9 if t_launch > 0 else 0.0
    # DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the dominant
    # kernel on this workload, from an ncu capture of the pose-0 frame (tile 16)
    traffic = NCU_DRAM_BYTES_PER_LAUNCH.get(dom) if args.tile == 16 else None
    roofline = {"bound": "hbm", "kernel": f"k_raster<PsLambert,{args.tile}>" if dom == "raster" else dom,
                "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 5), "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6.8 TB/s",
                "traffic": traffic, "traffic_l2_flushed": NCU_DRAM_BYTES_COLD.get(dom) if args.tile == 16 else None,
                "traffic_over_algorithmic": round(traffic / alg, 3) if traffic and alg else None,
                "algorithmic_bytes_per_launch": alg,
                "launch_ms": round(stages[dom] / args.steps, 4)}
    fb = frame_bytes(n_idx, vbytes, pixels, frags / args.steps, passes / args.steps)
    frame_roof = {"bytes_per_frame": fb, "achieved_gbs": round(fb / (ms / args.steps / 1e3) / 1e9, 2),
                  "frac": round(fb / (ms / args.steps / 1e3) / 1e9 / hbm, 5)}

    # e2e through the public API with host buffers
    e2e = run_e2e(ds, tg, sc, poses, args, torch)
    batched = None
    if not args.no_batch:
        batched = run_batched(torch)
    diffr = None
    if not args.no_diff:
        diffr = run_diff(torch)
    bprog = None if args.no_program else run_benchmark_program(torch)
    soup = None if args.no_soup else run_soup(torch)

    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cb = cpu_baseline()
        except Exception as ex:  # pragma: no cover
            cb = {"error": str(ex)}
    # issue roofline of the same kernel: its warp instructions per launch (ncu, mean over the
    # 32 poses) over what 152 SMs x 4 schedulers issue at the clock sampled during the frames
    clocks = clk.summary()
    inst = NCU_WARP_INST_PER_LAUNCH.get(dom)
    issue_roof = None
    if inst and clocks.get("sm_mhz") and args.tile == 16:
        rate = SMS * 4 * clocks["sm_mhz"] * 1e6
        ideal_ms = inst / rate * 1e3
        issue_roof = {"bound": "issue", "kernel": roofline["kernel"],
                      "warp_inst_per_fragment": round(inst / (frags / args.steps), 2),
                      "warp_inst_per_launch": inst, "issue_slots_per_s": rate,
                      "ideal_ms": round(ideal_ms, 4), "launch_ms": roofline["launch_ms"],
                      "frac": round(ideal_ms / roofline["launch_ms"], 4) if roofline["launch_ms"] else None}
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 4), "unit": "Gfrags/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded icosphere and poses)",
                "config": {"workload": WORKLOAD, "tile": args.tile, "parallelism": f"replicas x{world}",
                           "l2": "flushed before every timed frame (256 MiB write)",
                           "cuda_graph": not args.no_graph},
                "mtris_per_s": round(mtris, 2),
                "fragments_per_frame": frags / args.steps, "depth_passes_per_frame": passes / args.steps,
                "stage_ms_per_frame": {k: round(v / args.steps, 4) for k, v in stages.items()},
                "stage_pass_ms_per_frame": round(ps0.elapsed_time(ps1) / args.steps, 4),
                "gpu_launches": int(st["launches"]),
                "roofline": roofline, "issue_roofline": issue_roof, "frame_roofline": frame_roof,
                "clocks": clocks, "e2e": e2e, "cpu_baseline": cb, "batched": batched,
                "differentiable": diffr, "benchmark_program": bprog, "soup_4k": soup}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def run_batched(torch, n=256, steps=10):
    """Batched views/s: 256 seeded meshes (100 to 200k triangles each, piecewise-log-uniform;
    targets 256..1024 px square; own camera and 512x512 RGBA8 texture) rendered by one
    swr_draw_batch per step (configuration from the autotuner, CUDA graph replay) against
    the same views as 256 separate drawElements calls per step.  Targets total ~1 GB, larger
    than L2."""
    from softwarerenderer_gb300 import autotune, scenes
    from softwarerenderer_gb300.batch import BatchRenderer
    scs = scenes.batch_scenes(n)
    best = autotune.tune(scs)
    br = BatchRenderer(scs, tile=best["tile"], graph=best["graph"], pooled=True)
    autotune.apply_config(br, best)
    res = {"n_views": n, "triangles_per_step": int(sum(len(x.indices) // 3 for x in scs)),
           "pixels_per_step": int(sum(x.width * x.height for x in scs)), "autotune": best}
    for mode in ("batch", "loop"):
        fn = br.draw if mode == "batch" else br.draw_loop
        for _ in range(3):
            br.clear()
            fn()
        s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s0.record()
        for _ in range(steps):
            br.clear()
            fn(sync=False)
        e0.record()
        torch.cuda.synchronize()
        if mode == "batch":
            rc, st = br.ctx.finish()
            assert rc == 0, rc
        else:
            for ds in br.dev:
                rc, _ = ds.rast.ctx.finish()
                assert rc == 0, rc
        ms = s0.elapsed_time(e0) / steps
        res[f"{mode}_ms_per_step"] = round(ms, 4)
        res[f"{mode}_views_per_s"] = round(n / (ms / 1e3), 1)
    res["speedup_vs_loop"] = round(res["batch_views_per_s"] / res["loop_views_per_s"], 3)
    res["batch_mtris_per_s"] = round(res["triangles_per_step"] / (res["batch_ms_per_step"] / 1e3) / 1e6, 1)
    return res


def run_soup(torch, steps=5, warmup=3):
    """The triangle-soup stress configuration: 1,048,576 independent triangles at 3840x2160,
    Adaptive mode, per-vertex RGB with depth test; about a third cross the near, far or
    guard planes and half are culled by winding.  One drawElements per step, CUDA events,
    256 MiB L2 flush before each step."""
    from softwarerenderer_gb300 import scenes
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    sc = scenes.soup_scene()
    ds, tg = DeviceScene(sc), DeviceTarget(sc, aux=False)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")
    st = None
    for _ in range(warmup):
        tg.clear()
        st = ds.draw(tg)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        tg.clear()
        flush.fill_(k)
        ev[k][0].record()
        ds.draw(tg, sync=False)
        ev[k][1].record()
    torch.cuda.synchronize()
    rc, st2 = ds.rast.ctx.finish()
    assert rc == 0, rc
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    frags, passes = st2["fragments"] / steps, st2["passes"] / steps
    n_idx = len(sc.indices)
    algo = frame_bytes(n_idx, 24 * n_idx, sc.width * sc.height, frags, passes)
    hbm, _ = peaks()
    return {"workload": "1,048,576-triangle soup, 3840x2160, Adaptive, depth-tested vertex colour",
            "fragments": int(frags), "depth_passes": int(passes), "primitives": int(st["primitives"]),
            "ms": round(ms, 4), "gfrags_per_s": round(frags / (ms / 1e3) / 1e9, 2),
            "mtris_per_s": round(1048576 / (ms / 1e3) / 1e6, 1),
            "frame_roofline": {"bytes_per_frame": int(algo), "achieved_gbs": round(algo / (ms / 1e3) / 1e9, 1),
                               "peak": hbm, "frac": round(algo / (ms / 1e3) / 1e9 / hbm, 4)}}


def run_benchmark_program(torch, steps=10, warmup=3):
    """The reference's Benchmark.cpp program on the GPU: its scene (40,960 triangles of
    vertices from Random(0), CullMode None, Span, 640x480, affine colour without depth test;
    240 M fragments) drawn by one drawElements per step, each step timed with CUDA events
    after a 256 MiB L2 flush.  Algorithmic bytes per step: indices, vertex stream, the RGBA8
    target store and one 4-byte colour write per fragment (no depth test)."""
    from softwarerenderer_gb300 import scenes
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    sc = scenes.benchmark_scene()
    ds, tg = DeviceScene(sc), DeviceTarget(sc, aux=False)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")
    frags = 0
    for _ in range(warmup):
        tg.clear()
        frags = ds.draw(tg)["fragments"]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        tg.clear()
        flush.fill_(k)
        ev[k][0].record()
        ds.draw(tg, sync=False)
        ev[k][1].record()
    torch.cuda.synchronize()
    rc, st = ds.rast.ctx.finish()
    assert rc == 0, rc
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    n_idx = len(sc.indices)
    algo = 4 * n_idx + 24 * n_idx + 4 * sc.width * sc.height + 4 * frags
    hbm, _ = peaks()
    return {"workload": "Benchmark.cpp scene: 40,960 triangles, Random(0) vertices, 640x480, Span, CullMode None",
            "fragments": int(frags), "ms": round(ms, 4), "gfrags_per_s": round(frags / (ms / 1e3) / 1e9, 2),
            "mtris_per_s": round(40960 / (ms / 1e3) / 1e6, 1),
            "roofline": {"bound": "hbm", "algorithmic_bytes": algo, "achieved": round(algo / (ms / 1e3) / 1e9, 1),
                         "peak": hbm, "unit": "GB/s", "frac": round(algo / (ms / 1e3) / 1e9 / hbm, 4)}}


def run_diff(torch, steps=20, warmup=3):
    """Differentiable rendering: 16 views of the level-6 icosphere (40,962 vertices, 81,920
    triangles) at 512x512, per-vertex RGB and uv sampling a 1024x1024 RGBA32F texture
    bilinearly, L2 loss against seeded targets.  `fwd` = clearing the 16 targets + one
    swr_draw_batch (CUDA graph replay); `fwd_bwd` = fwd + zeroing the gradient buffers +
    swr_backward with the fused L2 loss (dL/d vertex records, dL/d texels, loss).  L2 is
    flushed (256 MiB write) before every step; every step is timed with CUDA events."""
    from softwarerenderer_gb300 import scenes
    from softwarerenderer_gb300.diff import DiffRenderer
    P = scenes.diff_problem()
    dr = DiffRenderer(P.indices, P.vertices.shape[0], P.texture.shape[1], P.texture.shape[0], P.mvps,
                      P.width, P.height, cull=P.cull, raster=P.raster)
    v = torch.from_numpy(P.vertices).cuda()
    t = torch.from_numpy(P.texture).cuda()
    tg = torch.from_numpy(P.targets).cuda()
    gv, gt = torch.zeros_like(v), torch.zeros_like(t)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")
    for _ in range(warmup):
        dr.forward(v, t)
        gv.zero_()
        gt.zero_()
        dr.backward(v, t, target=tg, grad_vertices=gv, grad_texture=gt)
    res = {"workload": "16 views of icosphere-6 (81,920 triangles) at 512x512, 1024x1024 RGBA32F texture, L2 loss",
           "views": P.n_views, "triangles_per_view": len(P.indices) // 3}
    for mode in ("fwd", "fwd_bwd"):
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
        torch.cuda.synchronize()
        for k in range(steps):
            flush.fill_(k)
            ev[k][0].record()
            dr.forward(v, t, sync=False)
            ev[k][1].record()
            if mode == "fwd_bwd":
                gv.zero_()
                gt.zero_()
                dr.backward(v, t, target=tg, grad_vertices=gv, grad_texture=gt, sync=False)
            ev[k][2].record()
        torch.cuda.synchronize()
        rc, st = dr.ctx.finish()
        assert rc == 0, rc
        res[f"{mode}_ms"] = round(sum(e[0].elapsed_time(e[2]) for e in ev) / steps, 4)
        if mode == "fwd_bwd":
            res["bwd_ms"] = round(sum(e[1].elapsed_time(e[2]) for e in ev) / steps, 4)
    res["fwd_views_per_s"] = round(P.n_views / (res["fwd_ms"] / 1e3), 1)
    res["fwd_bwd_views_per_s"] = round(P.n_views / (res["fwd_bwd_ms"] / 1e3), 1)
    res["fwd_bwd_over_fwd"] = round(res["fwd_bwd_ms"] / res["fwd_ms"], 3)
    res["covered_pixels"] = int((dr.winner >= 0).sum())
    # how the gradients are checked (tests/test_gpu_diff.py, tests/test_diff_oracle.py)
    res["gradient_checks"] = {
        "vs_cpu_reference": "all parameters, relative 2-norm error <= 1e-3 per group (rgb, uv, position, texels)",
        "vs_central_fd_h1e-3": "vertex rgb, uv and texels: plain central differences at h = 1e-3, 256 "
                               "sampled parameters per group, within 1e-3",
        "positions": "plain central FD at h = 1e-3 meets 1e-3 only on a coarser mesh (icosphere-4, 27-px "
                     "triangles: 6e-4); on this level-6 mesh (1.7-px triangles) its O(h^2) curvature term "
                     "leaves ~7e-3, so positions are checked against Richardson-extrapolated differences "
                     "(h and h/2; 4e-5) on vertices whose visible triangles have >= 1 px altitude"}
    return res


def run_e2e(ds, tg, sc, poses, args, torch):
    """Same frames through VertexProcessor.drawElements with host (pinned) inputs: every step
    copies the vertex streams and indices host->device and reads the colour buffer back.
    Steps are pipelined the usual way for a GPU frame loop: device inputs and targets are
    double-buffered and three streams overlap step k+1's input copy and step k-1's image
    read-back with step k's draw.  The timed region spans all K steps on all streams."""
    from softwarerenderer_gb300.device import DeviceTarget
    hv = [torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).pin_memory() for a, _ in sc.attribs]
    hi = torch.from_numpy(np.asarray(sc.indices, np.int32)).pin_memory()
    tgs = [tg, DeviceTarget(sc, aux=False)]
    hout = [torch.empty(tg.color.shape, dtype=tg.color.dtype).pin_memory() for _ in range(2)]
    dv = [[torch.empty_like(d) for d, _ in ds.attribs] for _ in range(2)]
    di = [torch.empty_like(ds.indices) for _ in range(2)]
    strides = [st for _, st in ds.attribs]
    comp, cin, cout = torch.cuda.current_stream(), torch.cuda.Stream(), torch.cuda.Stream()
    h2d = sum(t.numel() for t in hv) + hi.numel() * 4
    d2h = hout[0].numel() * 4
    unis = {(p, j): ds.uniforms(tgs[j], poses[p]) for p in range(len(poses)) for j in range(2)}
    ev = {name: [torch.cuda.Event() for _ in range(2)] for name in ("in_ready", "in_free", "out_ready", "out_done")}
    for j in range(2):
        ev["in_free"][j].record(comp)
        ev["out_done"][j].record(comp)

    def step(k):
        j = k & 1
        cin.wait_event(ev["in_free"][j])
        with torch.cuda.stream(cin):
            for d, h in zip(dv[j], hv):
                d.copy_(h, non_blocking=True)
            di[j].copy_(hi, non_blocking=True)
        ev["in_ready"][j].record(cin)
        comp.wait_event(ev["in_ready"][j])
        comp.wait_event(ev["out_done"][j])
        tgs[j].clear()
        for i, d in enumerate(dv[j]):
            ds.vp.setVertexAttribPointer(i, strides[i], d)
        ds.rast.setUniforms(unis[(k % len(poses), j)])
        ds.vp.drawElements(sc.draw_mode, di[j].numel(), di[j], sync=False)
        ev["in_free"][j].record(comp)
        ev["out_ready"][j].record(comp)
        cout.wait_event(ev["out_ready"][j])
        with torch.cuda.stream(cout):
            hout[j].copy_(tgs[j].color, non_blocking=True)
        ev["out_done"][j].record(cout)

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    ds.rast.ctx.finish()
    ds.rast.ctx.stage_times()
    s0 = torch.cuda.Event(enable_timing=True)
    e0 = torch.cuda.Event(enable_timing=True)
    s0.record(comp)
    cin.wait_event(s0)
    cout.wait_event(s0)
    for k in range(args.steps):
        step(k)
    comp.wait_stream(cin)
    comp.wait_stream(cout)
    e0.record(comp)
    torch.cuda.synchronize()
    rc, st = ds.rast.ctx.finish()
    assert rc == 0
    # the last image read back equals the frame the pipeline drew for it
    assert hout[(args.steps - 1) & 1].numpy().tobytes() == tgs[(args.steps - 1) & 1].color.cpu().numpy().tobytes()
    ds.bind(tg)  # restore the single-buffer binding for later users of ds
    ms = s0.elapsed_time(e0)
    return {"value": round(st["fragments"] / (ms / 1e3) / 1e9, 4), "unit": "Gfrags/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": round(ms / args.steps, 4),
            "mtris_per_s": round(327680 * args.steps / (ms / 1e3) / 1e6, 2),
            "pipeline": "double-buffered inputs and targets, copy-in / draw / read-back streams"}


if __name__ == "__main__":
    main()
