"""Benchmark of the GB300 meshlet visibility-buffer path.

Metric: views/s at 1920x1080 on the 82M-triangle torus-grid scene (2048
instances of a 40,000-triangle displaced torus, 843,776 meshlet draws) with
two-pass frustum + HiZ occlusion culling, visibility-buffer rasterisation,
HiZ pyramid and textured resolve, one step = one frame through a captured
CUDA graph.  The batched leg renders 256 views of uneven resolution in one
graph launch.  Inputs are synthetic (seeded procedural scene and cameras).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank renders its own views (weak scaling, no
collective on the data path); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "views/s at 1080p, 82M-tri scene: batched vs single-view CUDA; adjoint ms/view"
WORKLOAD = ("torus grid: 2048 instances x 40,000 tris = 81.92M tris, 843,776 meshlet draws (<=64 verts/"
            "<=124 tris), 1920x1080, two-pass frustum+cone+HiZ culling (with the fine footprint test), HiZ "
            "pyramid, textured resolve, steady state (previous frame's pyramid)")
W1080, H1080 = 1920, 1080
FLAGS_NAMES = ("CULL_FRUSTUM|CULL_CONE|CULL_OCCLUSION|CULL_OCCLUSION_FINE|CULL_TWO_PASS|BUILD_PYRAMID|"
               "RESOLVE_TEXTURED|WRITE_IDS")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--batch-views", type=int, default=256)
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--batched-only", action="store_true",
                   help="run only the batched leg (for profiling); prints its own JSON line")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--no-c1", action="store_true", help="skip the icosphere (C1) single-view leg")
    p.add_argument("--no-fine", action="store_true",
                   help="leave out the fine occlusion test (CULL_OCCLUSION_FINE) of the C2 and batched frames")
    p.add_argument("--no-motion", action="store_true", help="skip the motion-vector frame")
    p.add_argument("--no-world", action="store_true", help="skip the node-tree transform and draw-list leg")
    p.add_argument("--no-texture", action="store_true", help="skip the texture decode leg")
    p.add_argument("--world-only", action="store_true",
                   help="run only the node-tree transform and draw-list leg (for profiling); prints its own JSON line")
    p.add_argument("--adjoint-only", action="store_true",
                   help="run only the adjoint legs (for profiling); prints their own JSON line")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.lines: list[str] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------- reference

def bench_config(draws: int, triangles: int, world: int) -> dict:
    """The workload description both arms print."""
    return {"workload": WORKLOAD, "flags": FLAGS_NAMES, "width": W1080, "height": H1080,
            "draws": draws, "triangles": triangles,
            "l2": "256 MiB buffer written between timed steps (outside the events)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def run_reference(args, rank, world):
    """The reference's path on the host cores: the CPU restatement of the
    shader math (the Vulkan renderer itself cannot run here), same workload,
    all host threads, steady state.  Its scene and camera come from the
    oracle's own producers (byte-identical to the product's, checked by
    tests/test_oracle_scene.py), so this arm never loads the product library."""
    if rank != 0:
        return
    from oracle import binding as ob
    from oracle import scene as oscene

    threads = os.cpu_count() or 1
    ob.set_threads(threads)
    host = oscene.scene_torus_grid()
    cam = oscene.grid_camera(W1080, H1080)
    osc = ob.OracleScene(host)
    # the same frame flags as the CUDA arm (its cone and fine occlusion
    # tests are restated in the oracle; the ids are the same either way)
    flags = (ob.CULL_FRUSTUM | ob.CULL_CONE | ob.CULL_OCCLUSION | ob.CULL_OCCLUSION_FINE | ob.CULL_TWO_PASS
             | ob.BUILD_PYRAMID | ob.RESOLVE_TEXTURED)
    prev = ob.frame(osc, cam, W1080, H1080, flags)["pyramid"]
    for _ in range(max(0, args.warmup)):
        prev = ob.frame(osc, cam, W1080, H1080, flags, prev_pyramid=prev)["pyramid"]
    t0 = time.perf_counter()
    for _ in range(args.steps):
        prev = ob.frame(osc, cam, W1080, H1080, flags, prev_pyramid=prev)["pyramid"]
    dt = time.perf_counter() - t0
    v = args.steps / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "views/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64",
        "data": "synthetic",
        "config": bench_config(host.draw_count, host.triangle_count, world),
        "cpu_baseline": {"value": v, "unit": "views/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} steady-state frames of the workload on {threads} host threads"},
        "e2e": {"value": v, "unit": "views/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the Vulkan renderer needs a mesh-shader graphics device (none on this box); its CPU "
                "restatement (oracle/oracle.c) is timed instead",
    }), flush=True)


def run_batched(r, dev, host, flags, args, local, world, pg, stream, barrier):
    """Batched leg: the uneven views rendered in one captured graph launch,
    steady state (each view reads its own previous pyramid).  Under N ranks
    the views are sharded by pixel count (sharding.shard_views), so every
    view is rendered once across the ranks; the value is all views over the
    slowest rank's time."""
    import numpy as np
    import torch

    from vk_gltf_viewer_gb300 import scene, sharding
    from vk_gltf_viewer_gb300.renderer import ViewBuffers

    rank = int(os.environ.get("RANK", "0"))
    poses = scene.batch_views(args.batch_views)
    mine = sharding.shard_views([w * h for _, w, h in poses], world, rank)
    bv = []
    for i in mine:
        bcam, w, h = poses[i]
        vb = ViewBuffers.allocate(w, h, bcam, host.draw_count, device=f"cuda:{local}", prev_pyramid="alias",
                                  survivors=False)
        bv.append(vb)
    for vb in bv:
        vb.use_prev = False
    r.frame(dev, bv, flags)
    for vb in bv:
        vb.use_prev = True
    r.frame(dev, bv, flags)
    # launch shape from the autotuner (bin size x meshlets per CTA), then a
    # context with that shape for everything below
    from vk_gltf_viewer_gb300 import autotune
    r, tune = autotune.tuned_renderer(r, dev, bv, flags, launches=2)
    r.frame(dev, bv, flags)
    r.set_profiling(True)
    r.frame(dev, bv, flags)
    stages = r.stage_times()
    r.set_profiling(False)
    bgraph = r.capture(dev, bv, flags)
    for _ in range(2):
        bgraph.launch()
    torch.cuda.synchronize()
    bsteps = max(2, min(args.steps, 5))
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    b0.record(stream)
    for _ in range(bsteps):
        bgraph.launch()
    b1.record(stream)
    torch.cuda.synchronize()
    tb = torch.tensor([b0.elapsed_time(b1) / 1000.0], device=f"cuda:{local}")
    if pg:
        pg.all_reduce(tb, op=pg.ReduceOp.MAX)
    bval = bsteps * len(poses) / float(tb.item())
    kernels_per_launch = bgraph.kernel_count()
    bgraph.close()

    # The same poses through the plain single-view path: one captured
    # single-view frame per pose, replayed back to back on the stream.
    singles = [r.capture(dev, [vb], flags) for vb in bv]
    for g in singles:
        g.launch()
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    s0.record(stream)
    for _ in range(bsteps):
        for g in singles:
            g.launch()
    s1.record(stream)
    torch.cuda.synchronize()
    ts = torch.tensor([s0.elapsed_time(s1) / 1000.0], device=f"cuda:{local}")
    if pg:
        pg.all_reduce(ts, op=pg.ReduceOp.MAX)
    sval = bsteps * len(poses) / float(ts.item())
    for g in singles:
        g.close()
    r.close()
    out = {"value": bval, "unit": "views/s", "views_per_launch": len(poses), "views_this_rank": len(bv),
           "steps": bsteps,
           "single_view_same_poses": {"value": sval, "unit": "views/s",
                                      "ms_per_pass": 1000.0 * float(ts.item()) / bsteps},
           "speedup_vs_single_view_same_poses": bval / sval,
           "autotune": {"bin_size": tune["bin_size"], "meshlets_per_cta": tune["meshlets_per_cta"],
                        "cached": tune["cached"], "table": tune["table"]},
           "ms_per_launch": 1000.0 * float(tb.item()) / bsteps, "kernels_per_launch": kernels_per_launch,
           "mean_pixels_per_view": float(np.mean([w * h for _, w, h in poses])),
           "stages_ms": stages,
           "sharding": f"{len(bv)} of {len(poses)} views on rank {rank} of {world} (pixel-balanced)",
           "config": f"{len(poses)} poses on a radius-30 sphere around the grid centre, sizes uniform over "
                     "256^2, 512x384, 1024x576, 1280x720, 1920x1080"}
    return out


def run_c1(local, args, stream, flush, cpu: bool):
    """C1: the level-6 icosphere (81,920 triangles) at 1280x720, camera at
    (0, 0, 3) with a 60 degree field of view, frustum + cone culling, no HiZ,
    flat resolve; one captured single-view frame per step, L2 flushed between
    steps; beside it the oracle on all host threads."""
    import torch

    from vk_gltf_viewer_gb300 import abi, scene
    from vk_gltf_viewer_gb300.renderer import DeviceScene, Renderer, ViewBuffers

    w, h = 1280, 720
    host = scene.scene_icosphere(6)
    cam = scene.camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, w / h)
    flags = abi.CULL_FRUSTUM | abi.CULL_CONE | abi.RESOLVE_FLAT | abi.WRITE_IDS
    r = Renderer(local)
    dev = DeviceScene(host, f"cuda:{local}")
    v = ViewBuffers.allocate(w, h, cam, host.draw_count, device=f"cuda:{local}", pyramid=False)
    r.frame(dev, [v], flags)
    g = r.capture(dev, [v], flags)
    for _ in range(max(3, args.warmup)):
        g.launch()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.fill_(float(i))
        starts[i].record(stream)
        g.launch()
        ends[i].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / args.steps
    out = {"value": 1000.0 / ms, "unit": "views/s", "ms_per_view": ms, "triangles": host.triangle_count,
           "draws": host.draw_count, "survivors": int(v.survivor_count.item()), "kernels_per_frame": g.kernel_count(),
           "config": "icosphere level 6 (81,920 tris), 1280x720, eye (0,0,3), 60 deg, frustum + cone, no HiZ, "
                     "flat resolve, L2 flushed between steps"}
    g.close()
    r.close()
    if cpu:
        from oracle import binding as ob
        threads = os.cpu_count() or 1
        ob.set_threads(threads)
        osc = ob.OracleScene(host)
        n, t0 = 0, time.perf_counter()
        while n < 5 or (time.perf_counter() - t0 < 3.0 and n < 200):
            ob.frame(osc, cam, w, h, ob.CULL_FRUSTUM | ob.CULL_CONE | ob.RESOLVE_FLAT)
            n += 1
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / tc, "unit": "views/s", "cores": threads, "kind": "port",
                               "sample": f"{n} frames of the same view (oracle/oracle.c, {threads} threads)"}
    return out


def sphere_poses(rng, n, radius=3.0):
    """n eye points uniform on a sphere, aimed at the origin."""
    import numpy as np
    v = rng.normal(size=(n, 3))
    return radius * v / np.linalg.norm(v, axis=1, keepdims=True)


def run_adjoint_case(r, local, level, displace, tex_size, sizes, seed, steps, warmup, stream, pg=None):
    """One adjoint workload: zero + forward + backward (MSE against target
    renders) over all views in one captured graph; returns ms/view and the
    device memory the workload holds.  Under N ranks each rank steps the
    views of its pixel-balanced shard and the position, colour and texel
    gradients are summed with one all-reduce per step (inside the timed
    region); ms/view is over all views."""
    import numpy as np
    import torch

    from vk_gltf_viewer_gb300 import diff, scene

    dev = torch.device("cuda", local)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    torch.cuda.reset_peak_memory_stats(dev)
    alloc0 = torch.cuda.memory_allocated(dev)
    free0, total = torch.cuda.mem_get_info(dev)
    rng = np.random.default_rng(seed)
    mesh = scene.icosphere(level, displace=displace, seed=seed)
    nv = mesh.positions.shape[0]
    colors = rng.uniform(0, 1, size=(nv, 3)).astype(np.float32)
    texture = rng.uniform(0, 1, size=(tex_size, tex_size, 3)).astype(np.float32)
    ds = diff.DiffScene.create(mesh, colors, texture, device=dev)
    trng = np.random.default_rng(seed + 1000)
    pos_t = mesh.positions + trng.normal(0, 0.01, size=mesh.positions.shape).astype(np.float32)
    tex_t = trng.uniform(0, 1, size=texture.shape).astype(np.float32)
    dt = diff.DiffScene.create(mesh, colors, tex_t, device=dev, positions=pos_t)
    from vk_gltf_viewer_gb300 import sharding

    world = pg.get_world_size() if pg else 1
    rank = pg.get_rank() if pg else 0
    eyes = sphere_poses(rng, len(sizes))
    mine = sharding.shard_views([w * h for w, h in sizes], world, rank)
    views, targets, rgb = [], [], []
    for i in mine:
        w, h = sizes[i]
        eye = eyes[i]
        cam = scene.camera(tuple(eye), (0, 0, 0), scene.safe_up(eye, (0, 0, 0)), 60.0, w / h)
        views.append(diff.DiffViewBuffers.allocate(w, h, cam, device=dev))
        targets.append(torch.empty(w * h * 3, device=dev))
        rgb.append(torch.empty(w * h * 3, device=dev))
    diff.forward(r, dt, views, targets)
    gp, gc, gt = torch.empty_like(ds.positions), torch.empty_like(ds.colors), torch.empty_like(ds.texture)
    loss = torch.zeros(1, device=dev)
    px = sum(w * h for w, h in sizes)
    g = diff.capture_step(r, ds, views, rgb_out=rgb, targets=targets, grad_positions=gp, grad_colors=gc,
                          grad_texture=gt, scale=1.0 / (3 * px), loss=loss)

    def step():
        g.launch()
        if world > 1:
            sharding.allreduce_gradients([gp, gc, gt, loss])

    for _ in range(max(3, warmup)):
        step()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if pg:
        pg.barrier()
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    tm = torch.tensor([e0.elapsed_time(e1) / steps], device=dev)
    if pg:
        pg.all_reduce(tm, op=pg.ReduceOp.MAX)
    ms = float(tm.item())
    out = {"ms_per_view": ms / len(sizes), "ms_per_step": ms, "views": len(sizes), "views_this_rank": len(views),
           "pixels_per_step": px,
           "triangles": mesh.triangle_count, "vertices": nv, "texture": f"{tex_size}x{tex_size} fp32 RGB",
           "kernels_per_step": g.kernel_count(), "loss": float(loss.item()),
           "device_bytes_held": int(free0 - free1),
           "peak_tensor_bytes": int(torch.cuda.max_memory_allocated(dev) - alloc0)}
    g.close()
    del ds, dt, views, targets, rgb, gp, gc, gt
    torch.cuda.empty_cache()
    return out


def _meshopt_throughput() -> dict:
    """EXT_meshopt_compression ATTRIBUTES decode on the host: 1M vertex
    records of 16 bytes (slowly varying, like quantised positions), written
    by the package's encoder, decoded through the C ABI."""
    import ctypes

    import numpy as np

    from vk_gltf_viewer_gb300 import abi
    from vk_gltf_viewer_gb300.gltf_export import meshopt_encode_attributes
    rng = np.random.default_rng(17)
    count, stride = 1 << 20, 16
    data = (np.cumsum(rng.integers(-2, 3, (count, stride), dtype=np.int16), 0, dtype=np.int16) & 0xFF).astype(np.uint8)
    stream = meshopt_encode_attributes(data)
    out = np.empty(count * stride, np.uint8)
    lib = abi.load()
    times = []
    for _ in range(5):
        t0 = time.perf_counter()
        abi.check(lib.vkgv_meshopt_decode(out.ctypes.data, count, stride, ctypes.c_char_p(stream), len(stream),
                                          abi.MESHOPT_ATTRIBUTES, abi.MESHOPT_FILTER_NONE))
        times.append(time.perf_counter() - t0)
    assert out.tobytes() == data.tobytes()
    t = statistics.median(times)
    return {"decoded_bytes": int(out.size), "stream_bytes": len(stream), "ms": 1000.0 * t,
            "gb_per_s": out.size / t / 1e9, "threads": min(16, os.cpu_count() or 1),
            "note": "host, blocks split over threads after a serial scan of block starts"}


def run_world(r, host, local, args, stream, peak):
    """World::updateTransformBuffer and World::rebuildDrawBuffer of the torus
    grid as a node tree (root, 8 layers, 2,048 animated tori, 1,098 channels;
    843,776 draws) on the device, and the oracle's restatement of the
    reference's host walk timed beside it."""
    import numpy as np
    import torch

    from vk_gltf_viewer_gb300.world import DeviceWorld, grid_world

    mesh = host.meshes[0]
    wh = grid_world(mesh.meshlet_count, mesh.position_scale)
    dw = DeviceWorld(r, wh)
    dev = f"cuda:{local}"
    transforms = torch.empty(16 * dw.transform_count, dtype=torch.float32, device=dev)
    draws = torch.empty(3 * dw.draw_count, dtype=torch.int32, device=dev)
    reps, replays = 50, 4

    def timed(fn):
        # the calls are captured into one CUDA graph so that the device time,
        # not the Python launch rate, is measured
        side = torch.cuda.Stream()
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            for i in range(3):
                fn(i)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            for i in range(reps):
                fn(i)
        g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(replays):
            g.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / (reps * replays)

    ms_t = timed(lambda i: dw.update_transforms(0.01 * i, transforms))
    ms_d = timed(lambda i: dw.build_draws(draws))
    status = r.device_status()
    draw_bytes = 12 * dw.draw_count + 12 * (len(wh.mesh_primitives) + dw.transform_count)
    achieved = draw_bytes / (ms_d / 1000.0) / 1e9
    out = {
        "config": "torus grid as a node tree: 2,057 nodes (root, 8 layers, 2,048 tori), 1,098 channels (LINEAR, "
                  "STEP, CUBICSPLINE; translation, rotation, scale), 843,776 MeshletDraw records",
        "transforms_ms": ms_t, "transforms_per_s": dw.transform_count / (ms_t / 1000.0),
        "draws_ms": ms_d, "draws_per_s": dw.draw_count / (ms_d / 1000.0),
        "draws_roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                           "frac": achieved / peak, "algorithmic_bytes": draw_bytes,
                           "note": "12 B per draw written + 8 B per (primitive, slot) segment and its offset read; "
                                   "50 launches per CUDA graph, so the 10 MB list stays L2-resident"},
        "gpu_launches_per_update": 2, "gpu_launches_per_draw_build": 1,
        "device_status": list(status),
    }
    # the same scene as a .glb (1 primitive, 2,057 nodes, 1,098 channels)
    # read back through the importer: parse, accessors, meshlets, node tree
    import tempfile

    from vk_gltf_viewer_gb300 import gltf
    from vk_gltf_viewer_gb300.gltf_export import write_world
    with tempfile.TemporaryDirectory() as tmp:
        path = write_world(Path(tmp) / "grid.glb", [mesh], wh)
        loads = []
        for _ in range(3):
            t0 = time.perf_counter()
            ih, iw = gltf.load(path)
            loads.append(1000.0 * (time.perf_counter() - t0))
        out["gltf_import"] = {"ms": statistics.median(loads), "bytes": path.stat().st_size,
                              "draws": int(ih.draws.shape[0]), "nodes": int(iw.nodes.size),
                              "note": "host: JSON + GLB parse, accessors, meshlets of the 40k-triangle torus, "
                                      "node tree, samplers, host draw list"}
        # the same asset with EXT_meshopt_compression vertex and index views
        cpath = write_world(Path(tmp) / "grid_meshopt.glb", [mesh], wh, meshopt=True)
        loads = []
        for _ in range(3):
            t0 = time.perf_counter()
            ch, _ = gltf.load(cpath)
            loads.append(1000.0 * (time.perf_counter() - t0))
        assert np.array_equal(ch.meshes[0].positions, ih.meshes[0].positions)
        out["gltf_import"]["meshopt"] = {"ms": statistics.median(loads), "bytes": cpath.stat().st_size}
    out["meshopt_decode"] = _meshopt_throughput()
    if not args.no_cpu_baseline:
        from oracle import binding as ob
        n_t = n_d = 0
        t0 = time.perf_counter()
        while n_t < 3 or time.perf_counter() - t0 < 2.0:
            ob.world_transforms(wh, 0.01 * n_t)
            n_t += 1
        tt = (time.perf_counter() - t0) / n_t
        t0 = time.perf_counter()
        while n_d < 3 or time.perf_counter() - t0 < 2.0:
            ob.world_draws(wh)
            n_d += 1
        td = (time.perf_counter() - t0) / n_d
        out["cpu_baseline"] = {"transforms_ms": 1000.0 * tt, "draws_ms": 1000.0 * td, "cores": 1, "kind": "port",
                               "sample": f"{n_t} transform updates and {n_d} draw builds of the same world "
                                         "(oracle/world.c, the reference's recursive walk, one thread)"}
    dw.close()
    return out


def run_texture(r, local, args, stream, peak):
    """Base-colour texture decode: BC1, BC3 and BC7 blocks of an 8192^2
    texture into RGBA8 on the device (k_decode_bc; the BC7 blocks take the
    eight modes equally often), BC6H UF16 blocks (the fourteen modes equally
    often) into float32 RGB (k_decode_bc6h), and a 2048^2 RGBA8 PNG on the
    host (the C2 texture size)."""
    import zlib

    import numpy as np
    import torch

    from vk_gltf_viewer_gb300 import abi, texture

    out = {}
    rng = np.random.default_rng(3)
    w = h = 8192
    bc6h_modes = np.array([0x00, 0x01, 0x02, 0x06, 0x0A, 0x0E, 0x12, 0x16, 0x1A, 0x1E, 0x03, 0x07, 0x0B, 0x0F],
                          np.uint8)
    for name, fmt, bsize in (("bc1", abi.BC1, 8), ("bc3", abi.BC3, 16), ("bc7", abi.BC7, 16),
                             ("bc6h", abi.BC6H_UF16, 16)):
        host_blocks = rng.integers(0, 256, size=((w // 4) * (h // 4), bsize), dtype=np.uint8)
        if fmt == abi.BC7:  # mode m: the lowest set bit of the first byte is bit m
            modes = np.arange(host_blocks.shape[0]) % 8
            first = host_blocks[:, 0].astype(np.uint32)
            host_blocks[:, 0] = (((first >> (modes + 1)) << (modes + 1)) | (1 << modes)).astype(np.uint8)
        if fmt == abi.BC6H_UF16:  # a 2-bit (0, 1) or 5-bit mode field
            modes = bc6h_modes[np.arange(host_blocks.shape[0]) % bc6h_modes.size]
            keep = np.where(modes < 2, 0xFC, 0xE0).astype(np.uint8)
            host_blocks[:, 0] = (host_blocks[:, 0] & keep) | modes
        blocks = torch.from_numpy(host_blocks.reshape(-1)).cuda(local)
        hdr = fmt == abi.BC6H_UF16
        rgba = torch.empty((h, w, 3) if hdr else (h, w, 4), dtype=torch.float32 if hdr else torch.uint8,
                           device=f"cuda:{local}")
        lib = abi.load()
        decode = lib.vkgv_decode_bc6h if hdr else lib.vkgv_decode_bc
        for _ in range(3):
            abi.check(decode(r.ctx, fmt, blocks.data_ptr(), w, h, rgba.data_ptr(), stream.cuda_stream), r.ctx)
        torch.cuda.synchronize()
        ts = []
        for _ in range(10):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            decode(r.ctx, fmt, blocks.data_ptr(), w, h, rgba.data_ptr(), stream.cuda_stream)
            e1.record(stream)
            ts.append((e0, e1))
        torch.cuda.synchronize()
        ms = statistics.median(a.elapsed_time(b) for a, b in ts)
        nbytes = blocks.numel() + rgba.numel() * rgba.element_size()
        gbs = nbytes / (ms / 1000.0) / 1e9
        out[name + "_8192"] = {"ms": ms, "bytes": nbytes, "achieved_gbs": gbs, "frac": gbs / peak,
                               "texels_per_s": w * h / (ms / 1000.0)}
        del blocks, rgba
    # a 2048^2 RGBA8 PNG (dynamic DEFLATE, Paeth-filtered rows) on the host
    px = rng.integers(0, 256, size=(2048, 2048, 4), dtype=np.uint8)
    px[:, 1::2] = px[:, ::2]  # some redundancy for the compressor
    raw = bytearray()
    for row in px:
        raw += b"\x00" + row.tobytes()
    import struct
    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)
    png = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 2048, 2048, 8, 6, 0, 0, 0))
           + chunk(b"IDAT", zlib.compress(bytes(raw), 6)) + chunk(b"IEND", b""))
    t0 = time.perf_counter()
    img = texture.decode_png(png)
    png_ms = 1000.0 * (time.perf_counter() - t0)
    assert img.shape == (2048, 2048, 4)
    out["png_2048_host_ms"] = png_ms
    out["png_bytes"] = len(png)
    # a 2048^2 4:2:0 JPEG: entropy decode on the host, pixels on the device
    jpg = _synthetic_jpeg(2048, 2048, rng)
    t0 = time.perf_counter()
    j = texture.Jpeg(jpg)
    host_ms = 1000.0 * (time.perf_counter() - t0)
    for _ in range(3):
        j.to_rgba(r, stream)
    torch.cuda.synchronize()
    ts = []
    for _ in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        j.to_rgba(r, stream)
        e1.record(stream)
        ts.append((e0, e1))
    torch.cuda.synchronize()
    dev_ms = statistics.median(a.elapsed_time(b) for a, b in ts)
    coef_bytes = sum(p.nbytes for p in j.planes)
    # the same image with a restart marker every 16 MCUs: intervals on host threads
    jr = _synthetic_jpeg(2048, 2048, np.random.default_rng(3), restart=16)
    t0 = time.perf_counter()
    texture.Jpeg(jr).close()
    restart_ms = 1000.0 * (time.perf_counter() - t0)
    out["jpeg_2048"] = {"bytes": len(jpg), "host_entropy_ms": host_ms, "device_ms": dev_ms,
                        "host_entropy_ms_restart_16": restart_ms,
                        "coefficient_bytes": int(coef_bytes),
                        "note": "4:2:0, blocks from 256 random coefficient sets, 8-bit AC codes; device time "
                                "includes the pageable copy of the coefficient planes, the IDCT and the colour pass"}
    j.close()
    return out


def _synthetic_jpeg(w: int, h: int, rng, restart: int = 0) -> bytes:
    """A valid baseline 4:2:0 JPEG of w x h (multiples of 16): every block one
    of 256 random coefficient sets (magnitudes falling with frequency, DC
    differences 0), coded with one 1-bit DC code and 8-bit AC codes; with
    `restart`, a restart marker every `restart` MCUs."""
    import struct

    import numpy as np

    sym_index = {}
    pool = []
    for _ in range(256):
        bits = [0]  # DC: size 0
        k = 1
        while k < 64:
            run = int(rng.integers(0, 4))
            if k + run >= 64 or rng.random() < 0.04 * k ** 0.5:
                break
            k += run
            v = int(rng.integers(1, max(2, 200 // (k + 2)) + 1)) * (1 if rng.random() < 0.5 else -1)
            size = abs(v).bit_length()
            sym = (run << 4) | size
            code = sym_index.setdefault(sym, len(sym_index))
            bits += [(code >> i) & 1 for i in range(7, -1, -1)]
            bits += [((v if v > 0 else v + (1 << size) - 1) >> i) & 1 for i in range(size - 1, -1, -1)]
            k += 1
        if k < 64:
            code = sym_index.setdefault(0x00, len(sym_index))
            bits += [(code >> i) & 1 for i in range(7, -1, -1)]
        pool.append(np.array(bits, np.uint8))
    mcus = (w // 16) * (h // 16)
    choice = rng.integers(0, 256, mcus * 6)
    step = restart or mcus
    data = b""
    for k, first in enumerate(range(0, mcus, step)):
        bits = np.concatenate([pool[c] for c in choice[6 * first:6 * min(first + step, mcus)]])
        bits = np.concatenate([bits, np.ones(-len(bits) % 8, np.uint8)])  # pad with 1-bits
        data += np.packbits(bits).tobytes().replace(b"\xff", b"\xff\x00")
        if first + step < mcus:
            data += bytes([0xFF, 0xD0 + (k & 7)])
    values = sorted(sym_index, key=sym_index.get)
    seg = lambda m, body: struct.pack(">BBH", 0xFF, m, len(body) + 2) + body
    q = bytes([4] * 64)
    out = b"\xff\xd8" + seg(0xDB, b"\x00" + q) + seg(0xDB, b"\x01" + q)
    out += seg(0xC0, struct.pack(">BHHB", 8, h, w, 3) + bytes([1, 0x22, 0, 2, 0x11, 1, 3, 0x11, 1]))
    dc = bytes([0x00, 1] + [0] * 15 + [0])
    ac = bytes([0x10] + [0] * 7 + [len(values)] + [0] * 8) + bytes(values)
    out += seg(0xC4, dc) + seg(0xC4, ac)
    if restart:
        out += seg(0xDD, struct.pack(">H", restart))
    out += seg(0xDA, bytes([3, 1, 0x00, 2, 0x00, 3, 0x00, 0, 63, 0])) + data + b"\xff\xd9"
    return out


def run_adjoint(r, local, args, stream, pg=None):
    """Adjoint legs: the 64-view 512^2 icosphere-5 case and the batched
    512-view uneven-resolution icosphere-8 case (one graph per step)."""
    import numpy as np

    steps = max(3, min(args.steps, 10))
    c4 = run_adjoint_case(r, local, 5, 0.0, 1024, [(512, 512)] * 64, 41, steps, args.warmup, stream, pg)
    c4["config"] = ("icosphere level 5 (20,480 tris), per-vertex colours U(0,1), 1024^2 fp32 texture, 64 views "
                    "512^2 on a radius-3 sphere, MSE vs renders of N(0,0.01^2)-perturbed positions and a "
                    "separately seeded texture; step = zero + forward + backward in one graph")
    rng = np.random.default_rng(77)
    sides = rng.integers(256, 1025, size=512)
    c5 = run_adjoint_case(r, local, 8, 0.02, 2048, [(int(s), int(s)) for s in sides], 43, max(2, steps // 3),
                          args.warmup, stream, pg)
    c5["config"] = ("icosphere level 8 (1,310,720 tris) with seeded normal displacement 0.02, 2048^2 fp32 "
                    "texture, 512 square views with sides uniform in [256, 1024] on a radius-3 sphere; "
                    "zero + forward + backward (visibility recomputed) in one graph")
    return {"c4": c4, "c5": c5}


# ------------------------------------------------------------------- ours

def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import numpy as np
    import torch

    from vk_gltf_viewer_gb300 import abi, scene
    from vk_gltf_viewer_gb300 import build as vbuild
    from vk_gltf_viewer_gb300.renderer import DeviceScene, Renderer, ViewBuffers

    if not vbuild.LIB.exists():
        vbuild.build()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    r = Renderer(local)
    host = scene.scene_torus_grid()
    dev = DeviceScene(host, f"cuda:{local}")
    flags = (abi.CULL_FRUSTUM | abi.CULL_CONE | abi.CULL_OCCLUSION | abi.CULL_TWO_PASS | abi.BUILD_PYRAMID
             | abi.RESOLVE_TEXTURED | abi.WRITE_IDS)
    if not args.no_fine:
        flags |= abi.CULL_OCCLUSION_FINE
    stream = torch.cuda.current_stream()
    if args.batched_only:
        out = run_batched(r, dev, host, flags, args, local, world, pg, stream, barrier)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "batched": out}), flush=True)
        r.close()
        return
    if args.world_only:
        peaks_path = ROOT / "MEASURED_PEAKS.json"
        peak = float(json.loads(peaks_path.read_text())["hbm_gbs"]) if peaks_path.exists() else 6800.0
        out = run_world(r, host, local, args, stream, peak)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "world": out}), flush=True)
        r.close()
        return
    if args.adjoint_only:
        out = run_adjoint(r, local, args, stream, pg)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "adjoint": out}), flush=True)
        r.close()
        return
    cam = scene.grid_camera(W1080, H1080)
    view = ViewBuffers.allocate(W1080, H1080, cam, host.draw_count, device=f"cuda:{local}", prev_pyramid="alias")
    # first frame without history, then steady state
    view.use_prev = False
    r.frame(dev, [view], flags)
    view.use_prev = True
    for _ in range(2):
        r.frame(dev, [view], flags)
    torch.cuda.synchronize()
    from vk_gltf_viewer_gb300 import autotune
    rs, tune1 = autotune.tuned_renderer(r, dev, [view], flags, launches=5)
    rs.frame(dev, [view], flags)

    # per-stage zones of one steady-state frame (outside the timed region)
    rs.set_profiling(True)
    stage_runs = []
    for _ in range(5):
        rs.frame(dev, [view], flags)
        stage_runs.append(rs.stage_times())
    rs.set_profiling(False)
    stages = {k: statistics.median([s[k] for s in stage_runs]) for k in stage_runs[0]}

    graph = rs.capture(dev, [view], flags)
    kernels_per_frame = graph.kernel_count()
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    for _ in range(max(3, args.warmup)):
        graph.launch()
    torch.cuda.synchronize()

    # ---- timed: single view, device-resident inputs, L2 flushed between steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            flush.fill_(float(i))
            starts[i].record(stream)
            graph.launch()
            ends[i].record(stream)
        torch.cuda.synchronize()
        # The timed region is far shorter than the 200 ms sampling period:
        # keep the same frame running for ~1.5 s so the clock record has
        # samples under this load.
        t_load = time.perf_counter()
        while time.perf_counter() - t_load < 1.5:
            for _ in range(50):
                graph.launch()
            torch.cuda.synchronize()
    per_step = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    t_local = sum(per_step) / 1000.0
    t = torch.tensor([t_local], device=f"cuda:{local}")
    if pg:
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
    t_max = float(t.item())
    value = world * args.steps / t_max
    ms_per_step = 1000.0 * t_max / args.steps
    status = rs.device_status()

    # ---- e2e through the C ABI with host buffers: camera in, RGBA8 out.
    # Two colour images alternate, so the device-to-host read of frame i
    # (on a copy stream) overlaps frame i+1; every step still copies its
    # camera in and its image out inside the timed region.
    import dataclasses
    view_b = dataclasses.replace(view, color=torch.empty_like(view.color))
    graphs = [graph, rs.capture(dev, [view_b], flags)]
    colors = [view.color, view_b.color]
    cam_host = torch.from_numpy(scene.camera_bytes(cam)).pin_memory()
    rgba_host = [torch.empty(W1080 * H1080, dtype=torch.int32).pin_memory() for _ in range(2)]
    copy_stream = torch.cuda.Stream()
    rendered = [torch.cuda.Event() for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]
    for g in graphs:
        g.launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    for i in range(args.steps):
        s = i % 2
        if i >= 2:
            stream.wait_event(copied[s])
        view.camera.copy_(cam_host, non_blocking=True)
        graphs[s].launch()
        rendered[s].record(stream)
        copy_stream.wait_event(rendered[s])
        with torch.cuda.stream(copy_stream):
            rgba_host[s].copy_(colors[s], non_blocking=True)
        copied[s].record(copy_stream)
    stream.wait_stream(copy_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    graphs[1].close()
    te = torch.tensor([e0.elapsed_time(e1) / 1000.0], device=f"cuda:{local}")
    if pg:
        pg.all_reduce(te, op=pg.ReduceOp.MAX)
    e2e_value = world * args.steps / float(te.item())

    # ---- the same frame with the motion-vector image as well (the
    # reference's visibility pass writes it every frame), seen from a camera
    # that moved 0.1 units since the previous frame; L2 flushed between steps
    motion = None
    if not args.no_motion:
        # the moved camera also changes the pass-1 occlusion test (last
        # frame's pyramid seen through prevOcclusionViewProjection), so the
        # frame without motion vectors is timed on the same camera
        ms_pair = {}
        for name, mflags in (("plain", flags), ("motion", flags | abi.WRITE_MOTION)):
            view_m = ViewBuffers.allocate(W1080, H1080, scene.grid_camera(W1080, H1080, moved=0.1), host.draw_count,
                                          device=f"cuda:{local}", prev_pyramid="alias", motion=True)
            view_m.use_prev = False
            rs.frame(dev, [view_m], mflags)
            view_m.use_prev = True
            for _ in range(2):
                rs.frame(dev, [view_m], mflags)
            gm = rs.capture(dev, [view_m], mflags)
            for _ in range(max(3, args.warmup)):
                gm.launch()
            torch.cuda.synchronize()
            for i in range(args.steps):
                flush.fill_(float(i))
                starts[i].record(stream)
                gm.launch()
                ends[i].record(stream)
            torch.cuda.synchronize()
            ms_pair[name] = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / args.steps
            if name == "motion":
                mv_abs = float(np.abs(view_m.motion_vectors()).mean())
            gm.close()
            del view_m
        ms_m = ms_pair["motion"]
        motion = {"value": 1000.0 / ms_m, "unit": "views/s", "ms_per_view": ms_m,
                  "flags": FLAGS_NAMES + "|WRITE_MOTION", "ms_per_view_without_motion": ms_pair["plain"],
                  "time_vs_without": ms_m / ms_pair["plain"], "mean_abs_motion": mv_abs,
                  "camera": "grid camera, moved 0.1 units along +x since the previous frame"}
    graph.close()
    rs.close()

    # ---- roofline of the dominant kernel (meshlet raster, pass 1)
    dominant = max(("raster1", "big1", "cull1", "cull2", "hiz", "resolve", "clear"), key=lambda k: stages[k])
    surv = int(view.survivor_count.item())
    mesh = host.meshes[0]
    g_unique = (36 * mesh.meshlet_count + 4 * mesh.vertex_indices.size + 24 * mesh.vertices.size
                + mesh.primitive_indices.size)
    px = W1080 * H1080
    alg_bytes = {
        # survivor entry + draw record per meshlet, unique geometry, transforms,
        # one 8-byte depth|id write-back per pixel
        "raster1": 16 * surv + g_unique + 64 * host.transforms.shape[0] + 8 * px,
        # draw list + transforms + meshlet bounds read, survivor/reject lists written
        "cull1": 12 * host.draw_count + 64 * host.transforms.shape[0] + 36 * mesh.meshlet_count + 8 * surv,
        "resolve": 8 * px + 4 * px + 4 * px,
        "hiz": 8 * px + 4 * sum(max(1, (W1080 >> 1) >> k) * max(1, (H1080 >> 1) >> k) for k in range(10)),
        "clear": 8 * px,
    }
    dom_bytes = alg_bytes.get(dominant, alg_bytes["raster1"])
    dom_ms = stages[dominant]
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    peak, peak_src = 6800.0, "fallback"
    if peaks_path.exists():
        peak, peak_src = float(json.loads(peaks_path.read_text())["hbm_gbs"]), "measured"
    achieved = dom_bytes / (dom_ms / 1000.0) / 1e9
    traffic = None
    prof_instr = prof_meshlets = prof_atom = prof_atom_busy = prof_ncu_us = None
    prof = ROOT / "profiles" / "raster_meshlets_c2_1080p.md"
    if prof.exists():
        for line in prof.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch:"):
                traffic = int(line.split(":")[1].strip())
            elif line.startswith("warp_instructions_per_launch:"):
                prof_instr = int(line.split(":")[1].strip())
            elif line.startswith("meshlets_per_launch:"):
                prof_meshlets = int(line.split(":")[1].strip())
            elif line.startswith("atomic_sectors_per_launch:"):
                prof_atom = int(line.split(":")[1].strip())
            elif line.startswith("l2_atomic_unit_busy_pct:"):
                prof_atom_busy = float(line.split(":")[1].strip())
            elif line.startswith("ncu_duration_us:"):
                prof_ncu_us = float(line.split(":")[1].strip())

    # ---- batched leg: 256 uneven views in one graph launch
    batched = None
    if not args.no_batched and args.batch_views > 0:
        batched = run_batched(r, dev, host, flags, args, local, world, pg, stream, barrier)
        batched["speedup_vs_single_view"] = batched["value"] / value

    # ---- C1: the icosphere single view
    c1 = None
    if not args.no_c1:
        c1 = run_c1(local, args, stream, flush, cpu=rank == 0 and not args.no_cpu_baseline)

    # ---- node tree: animated transforms and the draw list on the device
    tree = None
    if not args.no_world:
        tree = run_world(r, host, local, args, stream, peak)

    # ---- texture decode (device BC blocks, host PNG)
    tex = None
    if not args.no_texture:
        tex = run_texture(r, local, args, stream, peak)

    # ---- adjoint legs (ms/view)
    adjoint = None
    if not args.no_adjoint:
        adjoint = run_adjoint(r, local, args, stream, pg)

    # ---- CPU baseline: the oracle on the host cores, bounded sample
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import binding as ob
        threads = os.cpu_count() or 1
        ob.set_threads(threads)
        osc = ob.OracleScene(host)
        of = (ob.CULL_FRUSTUM | ob.CULL_CONE | ob.CULL_OCCLUSION | ob.CULL_OCCLUSION_FINE | ob.CULL_TWO_PASS
              | ob.BUILD_PYRAMID | ob.RESOLVE_TEXTURED)
        prev = ob.frame(osc, cam, W1080, H1080, of)["pyramid"]
        n_cpu = 0
        tc0 = time.perf_counter()
        while n_cpu < 3 or (time.perf_counter() - tc0 < 10.0 and n_cpu < 30):
            prev = ob.frame(osc, cam, W1080, H1080, of, prev_pyramid=prev)["pyramid"]
            n_cpu += 1
        tc = time.perf_counter() - tc0
        cpu = {"value": n_cpu / tc, "unit": "views/s", "cores": threads, "kind": "port",
               "sample": f"{n_cpu} steady-state frames of the same workload (oracle/oracle.c, {threads} threads)"}

    # The raster is bound by instruction issue, not HBM: its warp
    # instructions per launch (the ncu count per meshlet, scaled to this
    # run's survivors) against the SMs' issue rate at the sampled clock.
    issue = None
    if dominant == "raster1" and prof_instr and prof_meshlets and dom_ms > 0:
        csum = clocks.summary()
        mhz = csum.get("sm_mhz") or 2070.0
        instr = prof_instr / prof_meshlets * surv
        peak_issue = 152 * 4 * mhz * 1e6
        issue = {"warp_instructions": instr, "achieved": instr / (dom_ms / 1000.0), "peak": peak_issue,
                 "unit": "warp instructions/s", "frac": instr / (dom_ms / 1000.0) / peak_issue,
                 "note": "152 SMs x 4 schedulers x 1 warp instruction per cycle at the sampled SM clock; "
                         "instruction count from the ncu capture of profiles/raster_meshlets_c2_1080p.md"}
    # The L2 atomic bound of the same launch: its 64-bit atomicMax count and
    # the L2 atomic units' busy fraction from the ncu capture, rescaled from
    # the capture's duration to this run's.
    # Whole-frame algorithmic bytes (12 B per draw, 4 B per survivor, the
    # unique geometry and transforms once, per pixel 8 B clear + 8 B raster
    # write-back + 8 B HiZ read + 8 B resolve read + 4 B RGBA8 write, and the
    # pyramid) over the frame time.
    frame_bytes = (12 * host.draw_count + 4 * surv + g_unique + 64 * host.transforms.shape[0] + 36 * px
                   + 4 * sum(max(1, (W1080 >> 1) >> k) * max(1, (H1080 >> 1) >> k) for k in range(10)))
    frame_roof = {"algorithmic_bytes": frame_bytes, "achieved": frame_bytes / (ms_per_step / 1000.0) / 1e9,
                  "unit": "GB/s", "frac": frame_bytes / (ms_per_step / 1000.0) / 1e9 / peak}
    atomic = None
    if dominant == "raster1" and prof_atom and prof_atom_busy is not None and prof_ncu_us and dom_ms > 0:
        atomic = {"atomics": prof_atom / (prof_meshlets or surv) * surv, "unit": "64-bit atomicMax/s",
                  "achieved": prof_atom / (prof_meshlets or surv) * surv / (dom_ms / 1000.0),
                  "frac": prof_atom_busy / 100.0 * prof_ncu_us / (dom_ms * 1000.0),
                  "note": "L2 atomic-unit busy fraction (lts__d_atomic_input_cycles_active) from the ncu capture "
                          "of profiles/raster_meshlets_c2_1080p.md, scaled by its duration over this run's"}
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "views/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic",
            "config": bench_config(host.draw_count, host.triangle_count, world),
            "e2e": {"value": e2e_value, "unit": "views/s", "h2d_bytes_per_step": 352,
                    "d2h_bytes_per_step": W1080 * H1080 * 4,
                    "note": "camera H2D + frame + RGBA8 D2H per step; the D2H of step i overlaps step i+1 "
                            "(two colour images, copy stream); a continuous loop, so no L2 flush between "
                            "steps (the device-only value flushes L2 before every step)"},
            "gpu_launches": kernels_per_frame * args.steps,
            "autotune": {"bin_size": tune1["bin_size"], "meshlets_per_cta": tune1["meshlets_per_cta"],
                         "cached": tune1["cached"], "table": tune1["table"]},
            "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                         "algorithmic_bytes": dom_bytes, "kernel_ms": dom_ms,
                         "issue": issue, "atomic": atomic, "frame": frame_roof},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "stages_ms": stages,
            "survivors": surv,
            "device_status": list(status),
        }
        if batched:
            # the metric's own comparison at the top level: batched views/s
            # and its ratio to the same poses through the single-view path
            out["batched_value"] = batched["value"]
            out["batched_speedup_same_poses"] = batched["speedup_vs_single_view_same_poses"]
            out["batched_speedup_vs_c2_single_view"] = batched["speedup_vs_single_view"]
            out["batched"] = batched
        if c1:
            out["c1_value"] = c1["value"]
            out["c1_cpu_value"] = (c1.get("cpu_baseline") or {}).get("value")
            out["c1"] = c1
        if adjoint:
            out["adjoint"] = adjoint
        if motion:
            out["motion"] = motion
        if tree:
            out["world"] = tree
        if tex:
            out["texture"] = tex
        print(json.dumps(out), flush=True)
    if pg:
        pg.destroy_process_group()
    r.close()


if __name__ == "__main__":
    main()
