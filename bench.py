"""Throughput benchmark of the GB300 wavefront path tracer (Msamples/s).

Workload (default): the mesh-heavy frame, 1920x1080 with 8x8 stratified samples (64 spp),
max depth 8, 2,355,202 triangles (a 1024x1024 Perlin height field and 64 tori) under a
2048x1024 f32 sky with a sun, sampled by next-event estimation — one step is one full
frame.  `--config cornell` runs the Cornell box of cornell_box_world
(raytracing/scenes.rs:226-294) with a GGX box and a glass sphere (600x600, 256 spp, depth
50), `--config final` the reference's final scene (400x225, 32 spp), `--config batch` 64
adaptive animation frames, `--config smoke` a world with two media, `--config denoise` the
denoiser's time to a relMSE; `--rng substreams` the throughput mode.

Arms:
  default          : this library (f32 wavefront) through the C ABI.
  --impl reference : the reference's CPU path.  The Rust crate cannot be built here, so
                     this times the C++ restatement of it (oracle/, "port") with every
                     host thread, on a bounded band of rows of the same frame.

One JSON line is printed by rank 0.  Multi-GPU runs (torchrun) render one independent
frame per GPU (replicas; there is no exchange step), so `scaling` is "weak".
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Msamples/s"
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="mesh", choices=["cornell", "final", "mesh", "batch", "smoke", "denoise"])
    ap.add_argument("--target-spp", type=int, default=4096, help="denoise config: samples of the reference image")
    ap.add_argument("--max-spp", type=int, default=1024, help="denoise config: largest plain sample count")
    ap.add_argument("--scene", default="mesh", choices=["mesh", "cornell"],
                    help="denoise config: the mesh-heavy workload or the Cornell box, both at 1920x1080")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target length of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--schedule", default="auto", choices=["auto", "wavefront", "persistent"])
    ap.add_argument("--tail-slots", type=int, default=0,
                    help="auto schedule: unfinished pixels at which the persistent kernel takes over (0 = library)")
    ap.add_argument("--stripes", type=int, default=0, help="wavefront stripes (0 = library default)")
    ap.add_argument("--rng", default="pixel", choices=["pixel", "substreams"],
                    help="per-sample random streams: the reference's (one per pixel) or the throughput mode's "
                         "(one per pixel and sample)")
    ap.add_argument("--migrate", default="default", choices=["default", "on", "off"],
                    help="auto schedule: move slow pixels to a concurrent persistent kernel (default: library rule)")
    ap.add_argument("--f32-tree", default="wide", choices=["wide", "binary"],
                    help="tree the f32 path traverses: the eight-wide compressed tree or the reference binary tree")
    ap.add_argument("--gpu-bvh", action="store_true",
                    help="the f32 path traverses a linear BVH built on the GPU (GT_BVH_GPU_LBVH)")
    ap.add_argument("--autotune", action="store_true",
                    help="pick stripes, tail size and blocks per SM with gt_autotune before the warm-up")
    ap.add_argument("--width", type=int, default=0, help="smaller image for profiling runs (0 = the workload's)")
    ap.add_argument("--grid", type=int, default=0, help="stratified grid width for profiling runs (0 = 16)")
    ap.add_argument("--profile-run", action="store_true",
                    help="render warmup+steps frames and print nothing else (for ncu captures)")
    return ap.parse_args()


def workload(name, width=0, grid=0):
    from gartus_gb300 import scenes
    if name == "cornell":
        scene, lights = scenes.cornell_scene()
        width, grid = width or 600, grid or 16
        cam = scenes.cornell_camera(width, grid, 50)
        cfg = {"workload": "cornell_box_ggx_glass", "width": width, "height": width, "spp": grid * grid,
               "max_depth": 50,
               "sampling": f"stratified {grid}x{grid}", "lights": "SamplingTargetList mixture (weight 0.5)",
               "primitives": len(scene), "precision": "f32"}
        return scene, lights, None, cam, cfg
    if name == "mesh":
        scene, env = scenes.mesh_heavy_scene()
        width = width or 1920
        grid = grid or 8
        cam = scenes.mesh_heavy_camera(width, width * 1080 // 1920, grid, 8)
        w, h, spp = width, width * 1080 // 1920, grid * grid
        cfg = {"workload": "mesh_heavy_perlin_tori_sun", "width": w, "height": h, "spp": spp, "max_depth": 8,
               "sampling": f"stratified {grid}x{grid}", "lights": "HDR environment 2048x1024 f32 with sun (NEE)",
               "primitives": len(scene), "precision": "f32"}
        return scene, None, env, cam, cfg
    if name == "smoke":  # participating media: the persistent kernel's world variant
        scene, _ = scenes.cornell_smoke_scene()
        width, grid = width or 600, grid or 8
        cam = scenes.cornell_camera(width, grid, 50)
        cfg = {"workload": "cornell_smoke_media", "width": width, "height": width, "spp": grid * grid,
               "max_depth": 50, "sampling": f"stratified {grid}x{grid}", "lights": "none (material sampling)",
               "primitives": len(scene), "media": 2, "precision": "f32"}
        return scene, None, None, cam, cfg
    if name == "batch":
        scene, lights = scenes.batch_scene()
        width = width or 512
        cams = scenes.batch_cameras(64, width)
        cfg = {"workload": "batch_64_frames_orbit_moving_spheres", "frames": len(cams), "width": width,
               "height": width, "spp": "adaptive, minimum cycling 4/8/16/32/64, cap 256, threshold 0.02",
               "max_depth": 50, "sampling": "random (adaptive)", "lights": "SamplingTargetList mixture (weight 0.5)",
               "primitives": len(scene), "precision": "f32", "shutter": "[0, 1), two moving spheres"}
        return scene, lights, None, cams, cfg
    scene = scenes.final_scene_ray_scene()
    width = width or 400
    cam = scenes.final_scene_camera(width, 32)
    cfg = {"workload": "final_scene_spheres", "width": width, "height": max(int(width / (16.0 / 9.0)), 1), "spp": 32,
           "max_depth": 10,
           "sampling": "random", "lights": "none (sky gradient)", "primitives": len(scene), "precision": "f32"}
    return scene, None, None, cam, cfg


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r.split(",") for r in self.path.read_text().strip().splitlines() if r.count(",") >= 8]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes per unit of work of each wavefront kernel on the mesh-heavy workload, from
# the ncu launch list of one 1920x1080 frame at 1 sample per pixel (four stripes, 12
# iterations each): dram__bytes_read.sum + dram__bytes_write.sum summed over the kernel's
# 48 launches, divided by the frame's units (4,272,505 closest-hit queries for k_trace and
# k_shade, 1,753,633 shadow queries for k_shadow, 2,073,600 samples for k_generate).  ncu
# empties the caches before every launch, so these are upper bounds on what the timed
# frame moves.  `roofline.traffic` scales them by the units of the dominant kernel's
# average launch.
DRAM_BYTES_PER_UNIT = {
    "mesh_heavy_perlin_tori_sun": {"trace": 473.0, "shadow": 825.1, "shade": 537.6, "generate": 304.3},
}
# Issue ceiling of k_trace on the same workload (one 912-block launch of that frame, all
# sections): the warp schedulers issue in 41.3% of their active cycles, and on average
# 9.80 of a warp's 32 lanes execute each instruction (rays of a warp visit different
# numbers of nodes and triangles).  The traversal kernels are bound by dependent loads and
# this divergence, not by HBM bandwidth.
ISSUE_PROFILE = {
    "mesh_heavy_perlin_tori_sun": {"kernel": "k_trace", "issue_active": 0.413, "lanes_per_instruction": 9.80,
                                   "warp_stall_long_scoreboard_per_issue": 6.91},
}


# ----------------------------------------------------------------------------------
def cpu_baseline(scene, lights, env, cam, seconds: float):
    """The oracle (C++ restatement of the reference's rayon renderer) on a band of rows
    of the same frame (of the middle frame for a batch), with every host thread; returns
    (Msamples/s, threads, sample)."""
    import oracle
    if isinstance(cam, list):
        cam = cam[len(cam) // 2]
    o = oracle.OracleScene.from_ray_scene(scene)
    la = lights.to_array() if lights is not None else None
    w, h, spp = oracle.camera_size(cam.desc())
    threads = os.cpu_count() or 1
    rows = 1
    t0 = time.perf_counter()
    o.render(cam.desc(), la, env, precision=1, threads=threads, window=(0, h // 2, w, rows))
    dt = max(time.perf_counter() - t0, 1e-3)
    rows = max(1, min(h, int(rows * seconds / dt)))
    y0 = max(0, h // 2 - rows // 2)
    t0 = time.perf_counter()
    _, acc = o.render(cam.desc(), la, env, precision=1, threads=threads, window=(0, y0, w, rows))
    dt = time.perf_counter() - t0
    samples = float(acc.sum())
    return samples / dt / 1e6, threads, f"rows {y0}..{y0 + rows} of {h} ({w * rows} pixels x {spp} spp), f64", dt


def run_denoise(args):
    """Time to relMSE 1e-3 on the mesh-heavy workload at 1920x1080 (random sampling, depth
    8): plain accumulation against the learned denoiser with its per-tile fallback."""
    import numpy as np
    import torch

    from gartus_gb300 import abi, scenes
    from gartus_gb300 import build as gbuild
    from gartus_gb300.denoiser import Denoiser, convergence_sweep
    from gartus_gb300.raytracing import Context

    gbuild.build()
    world, rank, local = dist_env()
    if world > 1 and rank != 0:  # one GPU measures; replicas would repeat the same curve
        return
    ctx = Context(local if world > 1 else 0)
    width = args.width or 1920
    height = width * 1080 // 1920
    den = Denoiser.pretrained(context=ctx)
    gen = torch.Generator(device="cpu").manual_seed(5)
    frame = [torch.rand((height, width, 3), generator=gen).cuda() for _ in range(3)]
    half = (frame[0] * 0.9).contiguous()
    if args.profile_run:  # denoise warmup+steps frames for an ncu capture; no timing, no output
        for _ in range(args.warmup + args.steps):
            den.denoise(frame[0], frame[1], frame[2], beauty_half=half)
        torch.cuda.synchronize()
        return
    # Inference roofline: tensor-core FLOPs of one frame (2 * pixels * 9 * cin * cout per
    # layer, padded channels included) over its time with device buffers.
    for _ in range(3):
        den.denoise(frame[0], frame[1], frame[2], beauty_half=half)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 10
    for _ in range(reps):
        den.denoise(frame[0], frame[1], frame[2], beauty_half=half)
    torch.cuda.synchronize()
    infer_s = (time.perf_counter() - t0) / reps
    from gartus_gb300.denoiser import layer_shapes
    hp, wp = (height + 15) // 16 * 16, (width + 15) // 16 * 16
    lv = [0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 3, 3, 2, 2, 1, 1, 0, 0, 0]
    flops = sum(2.0 * (hp >> l) * (wp >> l) * 9 * ((cin + 15) // 16 * 16) * ((cout + 7) // 8 * 8)
                for l, (cin, cout, _) in zip(lv, layer_shapes()))
    pk = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    bf16_peak = float(pk.get("bf16_tflops", 1900.0))
    achieved = flops / infer_s / 1e12
    if args.scene == "mesh":
        scene, env = scenes.mesh_heavy_scene()
        lights = None
        cam = scenes.mesh_heavy_camera(width, width * 1080 // 1920, 1, 8)
        wl = {"workload": "mesh_heavy_perlin_tori_sun", "max_depth": 8}
    else:
        scene, lights = scenes.cornell_scene()
        env = None
        cam = scenes.cornell_camera(width, 1, 50)._with(aspect_ratio=1920.0 / 1080.0)
        wl = {"workload": "cornell_box_ggx_glass_1080p", "max_depth": 50}
    cam = cam.with_pixel_sample_mode(abi.GT_SAMPLE_RANDOM).with_samples_per_pixel(1)
    w, h, _ = cam.image_size()
    log = (lambda m: print(m, file=sys.stderr, flush=True))
    with ClockSampler(ctx.device) as clocks:
        r = convergence_sweep(den, scene, cam, lights, env, target_spp=args.target_spp, max_spp=args.max_spp,
                              context=ctx, log=log)
    value = r["denoised"]["time_s"] if r["denoised"] else None
    line = {
        "metric": "time-to-relMSE 1e-3", "value": value, "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 0,
        "ms_per_step": value * 1e3 if value else None, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 render, bf16 network (fp32 accumulate)",
        "data": "synthetic (seeded procedural scene)",
        "config": {**wl, "width": w, "height": h, "sampling": "random", "reference_spp": args.target_spp,
                   "reference": "two independent f32 renders of half the samples each (Kahan-compensated "
                                "accumulation), their difference estimating the reference's own error",
                   "plain_sweep_spp": f"1..{args.max_spp} doubling", "denoiser": "committed U-Net weights",
                   "relmse": "mean over pixels of mean_c (x - T)^2 / (T^2 + 0.01), less the reference's own "
                             "error, over all but the 0.1% of pixels with the largest error (raw values in curve)",
                   "tile": 16, "threshold": 3.0},
        "plain_time_s": r["plain"]["time_s"] if r["plain"] else None,
        "plain_spp": r["plain"]["spp"] if r["plain"] else None,
        "plain_extrapolated": r["plain"]["extrapolated"] if r["plain"] else None,
        "goals": r["goals"], "plain_relmse_times_spp": r["plain_c"],
        "denoised_spp": r["denoised"]["spp"] if r["denoised"] else None,
        "speedup": r["speedup"], "best_denoised_relmse": r["best_denoised"],
        "reference_error": r["reference_error"], "clocks": clocks.summary(),
        "roofline": {"bound": "tensor", "kernel": "denoiser inference (19 k_conv_fwd + elementwise)",
                     "achieved": achieved, "peak": bf16_peak,
                     "peak_kind": "measured" if pk else "fallback", "unit": "TFLOP/s",
                     "frac": achieved / bf16_peak, "traffic": None, "flops_per_frame": flops,
                     "frame_ms": infer_s * 1e3, "frame": f"{width}x{height} (padded {wp}x{hp})"},
        "gpu_launches": None,
        "curve": r["curve"],
    }
    print(json.dumps(line))


def run_reference_arm(args):
    world, rank, _ = dist_env()
    if args.config == "denoise":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no denoiser, and its CPU path "
                              "cannot render the 1080p reference image of this experiment within minutes"}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        if rank != 0:
            dist.barrier()
            return
    scene, lights, env, cam, cfg = workload(args.config, args.width, args.grid)
    per_step = max(args.cpu_seconds / 3.0, 2.0)
    for _ in range(args.warmup):
        cpu_baseline(scene, lights, env, cam, 0.5)
    vals, dts = [], []
    sample = ""
    threads = 1
    for _ in range(args.steps):
        v, threads, sample, dt = cpu_baseline(scene, lights, env, cam, per_step)
        vals.append(v)
        dts.append(dt)
    value = statistics.median(vals)
    cfg = dict(cfg, precision="f64", implementation="C++ restatement of the reference (oracle/)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(dts), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded procedural scene)",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_ours(args):
    import ctypes as C

    import numpy as np
    import torch

    from gartus_gb300 import abi
    from gartus_gb300 import build as gbuild
    from gartus_gb300._lib import check, lib
    from gartus_gb300.raytracing import Context, PathTracer

    gbuild.build()
    world, rank, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local if world > 1 else 0
    torch.cuda.set_device(device)
    ctx = Context(device)
    scene, lights, env, cam, cfg = workload(args.config, args.width, args.grid)
    if args.gpu_bvh:
        scene.use_gpu_bvh()
        cfg = dict(cfg, bvh="linear BVH built on the GPU at upload (GT_BVH_GPU_LBVH)")
    if args.f32_tree == "binary":
        scene.use_binary_f32_tree()
    cfg = dict(cfg, f32_tree=("binary reference SAH tree" if args.f32_tree == "binary" or args.gpu_bvh
                              else "eight-wide compressed tree collapsed from the reference SAH tree"))
    cams = cam if isinstance(cam, list) else None
    if cams is not None:
        cam = cams[0]
    pt = PathTracer(cam, context=ctx, schedule=args.schedule, tail_slots=args.tail_slots, stripes=args.stripes,
                    migrate=args.migrate, rng=args.rng)
    tuned = None
    if args.autotune:  # a batch tunes on its first 16 frames
        tuned = pt.autotune(scene, lights, env, cameras=cams[:16] if cams is not None else None)
        print(f"autotune: {tuned}", file=sys.stderr, flush=True)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")

    def render():
        if cams is not None:
            return pt.render_batch_hdr_images(scene, cams, lights=lights, environment=env)[-1]
        if env is not None:
            return pt.render_with_environment_hdr_image(scene, env)
        if lights is not None:
            return pt.render_with_lights_hdr_image(scene, lights)
        return pt.render_hdr_image(scene)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(device)

    if args.profile_run:  # a fixed number of frames for an ncu capture; no timing, no bench line
        for _ in range(args.warmup + args.steps):
            render()
        torch.cuda.synchronize(device)
        # the last frame's counts (rays per kernel), to turn a capture's bytes into bytes per ray
        print(json.dumps({"profile_run_stats": pt.last_stats, "config": cfg}), file=sys.stderr)
        return
    for _ in range(max(args.warmup, 3)):
        render()
    dev_ms, samples, rays, launches = 0.0, 0, 0, 0
    barrier()
    wall0 = time.perf_counter()
    with ClockSampler(device) as clocks:
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between timed iterations (outside the device-timed region)
            torch.cuda.synchronize(device)
            img = render()
            st = pt.last_stats
            dev_ms += st["gpu_ms"]
            samples += st["samples"]
            rays += st["rays"] + st["shadow_rays"]
            launches += sum(st["kernel_launches"].values())
    barrier()
    wall_s = time.perf_counter() - wall0
    clock = clocks.summary()
    assert np.isfinite(img.pixels).all()

    # Max over ranks of the device time; the aggregate counts every rank's samples.
    t = torch.tensor([dev_ms, float(samples)], dtype=torch.float64, device=f"cuda:{device}")
    if dist is not None:
        tmax = t.clone()
        dist.all_reduce(tmax[0:1], op=dist.ReduceOp.MAX)
        dist.all_reduce(tmax[1:2], op=dist.ReduceOp.SUM)
        t = tmax
    dev_ms_max, total_samples = float(t[0]), float(t[1])
    value = total_samples / (dev_ms_max / 1e3) / 1e6

    # End to end through the C ABI with host buffers.  The metric leaves the scene upload out
    # and reports the BVH build on its own, as a renderer that keeps its scene resident works:
    # gt_scene_create (host SAH build) and the first render (upload of primitives, tree,
    # materials, lights and environment) are timed once, separately; every timed step is then
    # one gt_render (gt_render_batch) call with the camera descriptions in host memory and the
    # images and accepted-sample counts read back into host memory.
    prims = np.ascontiguousarray(scene.primitives_array())
    mats = np.ascontiguousarray(scene.materials_array())
    d = abi.gt_scene_desc()
    d.struct_size = C.sizeof(abi.gt_scene_desc)
    d.num_primitives, d.num_materials, d.bvh_leaf_size = len(prims), len(mats), scene.leaf_size
    d.bvh_builder = scene._bvh_builder
    d.f32_tree = scene._f32_tree
    d.primitives = prims.ctypes.data_as(C.POINTER(abi.gt_primitive))
    d.materials = mats.ctypes.data_as(C.POINTER(abi.gt_material))
    sh, lh, eh = C.c_void_p(), C.c_void_p(), C.c_void_p()
    t0 = time.perf_counter()
    check(lib().gt_scene_create(ctx.handle, C.byref(d), C.byref(sh)))
    bvh_build_s = time.perf_counter() - t0
    la = lights.to_array() if lights is not None else None
    if la is not None:
        check(lib().gt_lights_create(ctx.handle, la.ctypes.data_as(C.c_void_p), len(la), C.byref(lh)))
    if env is not None:
        check(lib().gt_environment_create(ctx.handle, C.byref(env.desc()), C.byref(eh)))
    outs, frames, descs = [], [], []
    for c in (cams or [cam]):
        w, h, _ = c.image_size()
        rgb = np.empty((h, w, 3), dtype=np.float32)
        acc = np.empty((h, w), dtype=np.uint32)
        f = abi.gt_frame()
        f.struct_size = C.sizeof(abi.gt_frame)
        f.width, f.height, f.device_buffers = w, h, 0
        f.rgb, f.accepted = rgb.ctypes.data, acc.ctypes.data
        outs += [rgb, acc]
        frames.append(f)
        descs.append(c.desc())
    o = abi.gt_render_opts()
    o.struct_size = C.sizeof(abi.gt_render_opts)
    pt._launch_opts(o)  # the same schedule and launch shapes as the timed leg
    stt = abi.gt_render_stats()
    o.stats = C.pointer(stt)
    jobs = None
    if cams is not None:
        jobs = (abi.gt_frame_job * len(cams))()
        for i in range(len(cams)):
            jobs[i].camera = C.pointer(descs[i])
            jobs[i].frame = C.pointer(frames[i])

    def abi_render():
        if jobs is not None:
            check(lib().gt_render_batch(sh, lh if la is not None else None, eh if env is not None else None,
                                        jobs, len(cams), C.byref(o)))
        else:
            check(lib().gt_render(sh, lh if la is not None else None, eh if env is not None else None,
                                  C.byref(descs[0]), C.byref(o), C.byref(frames[0])))

    t0 = time.perf_counter()
    abi_render()  # uploads the scene, then renders
    first_s = time.perf_counter() - t0
    abi_render()  # captures this call's graphs
    e2e_vals = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        abi_render()
        dt = time.perf_counter() - t0
        e2e_vals.append(stt.samples / dt / 1e6)
    steady_s = stt.samples / statistics.median(e2e_vals) / 1e6
    lib().gt_scene_destroy(sh)
    if la is not None:
        lib().gt_lights_destroy(lh)
    if env is not None:
        lib().gt_environment_destroy(eh)
    h2d = len(descs) * C.sizeof(abi.gt_camera_desc)
    d2h = sum(x.nbytes for x in outs)
    scene_setup = {"bvh_build_s": bvh_build_s, "upload_s": max(first_s - steady_s, 0.0),
                   "bvh": "reference SAH on the host (gt_scene_create)" if scene._bvh_builder == abi.GT_BVH_REFERENCE_SAH
                   else "linear BVH on the GPU (first render)",
                   "upload_bytes": len(prims) * 64 + len(prims) * 8 + max(len(prims) - 1, 1) * 64 + len(mats) * 64
                   + (len(la) * 128 if la is not None else 0) + (env.texels.nbytes if env is not None else 0)}
    e2e = statistics.median(e2e_vals) * world

    # Roofline of the dominant kernel from one profiled frame (events around every launch).
    prof = PathTracer(cam, context=ctx, profile=True, **pt._launch_kw())
    if cams is not None:
        prof.render_batch_hdr_images(scene, cams, lights=lights, environment=env)
    elif env is not None:
        prof.render_with_environment_hdr_image(scene, env)
    elif lights is not None:
        prof.render_with_lights_hdr_image(scene, lights)
    else:
        prof.render_hdr_image(scene)
    ps = prof.last_stats
    kms = ps["kernel_ms"]
    dom = max(("trace", "shade", "generate", "shadow", "persistent"), key=lambda k: kms[k])
    ids, _, bstats = PathTracer(cam.with_samples_per_pixel(1), context=ctx).trace_primary(scene, 1)
    per_ray_nodes = bstats["node_bounds_tests"] / max(bstats["rays"], 1)
    per_ray_prims = bstats["primitive_candidates"] / max(bstats["rays"], 1)
    kinds = scene.primitives_array()["geometry"]["kind"]
    s_by_kind = {0: 16, 1: 28, 2: 36, 3: 48}
    s_prim = float(np.mean([s_by_kind[int(k)] for k in kinds])) if len(kinds) else 0.0
    b_ray = 32.0 * per_ray_nodes + s_prim * per_ray_prims + 64.0
    b_state = 2 * (32 + 12 + 8 + 4 + 4) + 8
    bytes_per_unit = {"trace": b_ray, "shade": float(b_state), "generate": float(b_state), "shadow": b_ray,
                      "persistent": b_ray}
    # closest-hit queries of the wavefront kernels: all of them less those traced inside
    # k_persistent (exact without next-event shadow rays, which k_persistent also counts)
    wave_rays = max(ps["rays"] - ps["persistent_rays"], 0)
    units = {"trace": wave_rays, "shade": wave_rays, "generate": ps["samples_started"], "shadow": ps["shadow_rays"],
             "persistent": ps["persistent_rays"]}
    launches_dom = max(ps["kernel_launches"][dom], 1)
    avg_ms = kms[dom] / launches_dom
    algo_bytes = units[dom] * bytes_per_unit[dom] / launches_dom
    peak, peak_kind = measured_peaks()
    achieved = algo_bytes / (avg_ms / 1e3) / 1e9 if avg_ms > 0 else 0.0
    per_unit = DRAM_BYTES_PER_UNIT.get(cfg["workload"], {}).get(dom)
    traffic = per_unit * units[dom] / launches_dom if per_unit is not None else None
    issue = ISSUE_PROFILE.get(cfg["workload"])
    if issue is not None:
        issue = dict(issue, simt_efficiency=issue["lanes_per_instruction"] / 32.0,
                     issue_ceiling=issue["issue_active"] * issue["lanes_per_instruction"] / 32.0)
    # every kernel's own roofline point from the same profiled frame
    per_kernel = {}
    for k in ("generate", "trace", "shade", "shadow", "persistent"):
        nl = ps["kernel_launches"][k]
        if nl == 0 or kms[k] <= 0:
            continue
        gbs = units[k] * bytes_per_unit[k] / nl / (kms[k] / nl / 1e3) / 1e9
        per_kernel[f"k_{k}"] = {"achieved": gbs, "frac": gbs / peak, "avg_launch_ms": kms[k] / nl, "launches": nl,
                                "bytes_per_unit": bytes_per_unit[k], "units_per_launch": units[k] / nl}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, threads, sample, _ = cpu_baseline(scene, lights, env, cam, args.cpu_seconds)
        cpu = {"value": v, "unit": METRIC, "cores": threads, "kind": "port", "sample": sample}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "rng": pt.rng,
            "config": dict(cfg, l2="flushed between timed steps (512 MiB write)", schedule=pt.schedule, rng=pt.rng,
                           parallelism=f"replicas x{world}" if world > 1 else "single GPU",
                           launch={"stripes": pt.stripes, "tail_slots": pt.tail_slots,
                                   "generate_blocks_per_sm": pt.generate_blocks_per_sm,
                                   "trace_blocks_per_sm": pt.trace_blocks_per_sm,
                                   "migrate": pt.migrate,
                                   "from": "gt_autotune" if tuned else "library defaults"}),
            "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "call": "gt_render_batch" if cams is not None else "gt_render",
                    "scene": "resident (created and uploaded once, outside the timed steps)"},
            "scene_setup": scene_setup,
            "gpu_launches": launches,
            "clocks": clock,
            "roofline": {"bound": "hbm", "kernel": f"k_{dom}", "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "traffic_source": "DRAM bytes per unit from the ncu launch list of the "
                                                               "1-spp frame, times this run's units per launch"
                         if traffic is not None else None,
                         "issue": issue, "algorithmic_bytes_per_launch": algo_bytes,
                         "avg_launch_ms": avg_ms, "bytes_per_unit": bytes_per_unit[dom],
                         "units_per_launch": units[dom] / launches_dom, "per_kernel": per_kernel},
            "cpu_baseline": cpu,
            "detail": {"wall_s_timed": wall_s, "rays_per_s": rays / (dev_ms / 1e3), "kernel_ms_profiled": kms,
                       "kernel_launches_profiled": ps["kernel_launches"], "iterations_per_frame": ps["iterations"],
                       "migrated_pixels_profiled": ps["migrated_pixels"], "tail_pixels_profiled": ps["tail_pixels"],
                       "bvh_per_ray": {"node_tests": per_ray_nodes, "prim_candidates": per_ray_prims}},
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_arm(args)
    elif args.config == "denoise":
        run_denoise(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
