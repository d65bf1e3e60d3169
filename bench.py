#!/usr/bin/env python
"""Benchmark of Pike's wavefront path tracer on one GB300 (or N replicas).

Workload: the incoherent 1080p scene -- an icosphere subdivided 8 times
(1,310,720 triangles) displaced by value noise inside an open 10x10x10 box
(10 triangles), 256 GGX/Lambert material groups, a 2048x1024 log-normal HDR
environment with a sun -- rendered at 1920x1080 with 8 bounces.  One step is
one PikeRenderer.tick(): one sample per pixel, camera rays, 8 x (closest-hit
trace, shade, shadow trace), accumulate and tonemap.  The 64-spp job is 64
steps.  Inputs are synthetic (seeded generators of that shape).

Metric: Mrays/s (closest-hit + shadow rays traced per second, whole job),
with spp*Mpix/s alongside.  `value` is device time (CUDA events on the
library's API stream, which waits for every frame in flight) with the scene
resident in HBM; `e2e` runs the same steps through the C ABI with the
per-step render state and camera (56 bytes, handed to the device as launch
parameters of the frame's state kernel) and every frame's 8-bit image read
back asynchronously into pinned host memory, timed by the host clock from the
first call to the return of the final pk_sync.  Frames render eight at a
time in flight (pk_set_frames_in_flight), bit-identical to one at a time.  The
roofline line adds an L2 fraction against an L2 read peak measured in the
same run (pk_probe_read_bandwidth).  The `forms` block includes the
8,388,608-triangle soup (the precision workload) unless --no-precision.

--impl reference times the CPU restatement of the reference path (the oracle;
the reference itself is JavaScript + WGSL on WebGPU and cannot run here) on
the host cores, on a bounded band of the same frame.

Multi-GPU: the path shards by sample, so N ranks render N independent
replicas (rank r renders samples r, r+N, ...); no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s, spp/s @1080p"
UNIT = "Mrays/s"
WORKLOAD = "icosphere8+openbox 1920x1080, 8 bounces, 1 spp per step (64-spp job = 64 steps)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--bounces", type=int, default=8)
    ap.add_argument("--subdivisions", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--trace-mode", default="persistent", choices=["persistent", "chunked", "wide"],
                    help="traversal scheduling (identical results): persistent lanes with refill, or 32-ray chunks")
    ap.add_argument("--no-forms", action="store_true", help="skip the forms blocks (wide BVH, adjoint, batching)")
    ap.add_argument("--profile-case", choices=["wide", "wide_soup", "adjoint", "batch"],
                    help="run one small case of a form kernel (for ncu captures) and exit")
    ap.add_argument("--frames-in-flight", type=int, default=8, choices=list(range(1, 17)),
                    help="frames of pk_render_frame rendered concurrently (accumulation stays in order); "
                         "8 measured 1-2%% above 4 at 1080p, 12 and 16 no faster than 8")
    ap.add_argument("--overlap", choices=["auto", "on", "off"], default="auto",
                    help="shadow traversal beside the next bounce's closest-hit traversal "
                         "(auto: with one frame in flight or below 2^20 pixels)")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip form (1)'s 8.4M-triangle soup workload (part of the default run)")
    ap.add_argument("--node-records", type=int, default=64, choices=[32, 64],
                    help="inner-node record size (identical results): decoded float boxes (64) or snorm16 (32)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Dist:
    """Barrier and max-over-ranks for the replica runs (torch.distributed when world > 1)."""

    def __init__(self, world: int, local: int):
        self.world = world
        self.dist = None
        if world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(local)
            dist.init_process_group(backend=backend)
            self.dist, self.torch = dist, torch
            self.dev = torch.device("cuda", local) if backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.dist:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def replica_throughput(D: Dist, rays_local: float, ms_local: float):
    """Whole-job Mrays/s of N replicas: every rank's rays over the slowest
    rank's time (max over ranks); returns (value, ms_max) on every rank."""
    ms_max = D.max(ms_local)
    rays_total = D.sum(float(rays_local))
    return rays_total / (ms_max / 1000.0) / 1e6, ms_max


class Clocks:
    """nvidia-smi samples (every 200 ms) while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self) -> dict | None:
        if not self.p:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """Per-launch DRAM bytes of the closest-hit kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "trace_closest_dram.txt")
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("dram_bytes_per_launch_full_frame:"):
                    return float(line.split(":", 1)[1].split()[0])
    except (OSError, ValueError):
        pass
    return None


def l2_peak(ctx) -> dict:
    """L2 read-bandwidth peak from the library's probe kernel
    (pk_probe_read_bandwidth): 128-bit L2-only loads from every SM over a
    buffer read 40 times, at 32 and 64 MB (both inside the 129 MB L2); the
    larger rate is the denominator."""
    import ctypes as C
    rates = {}
    for mb in (32, 64):
        g = C.c_float(0.0)
        ctx.call("pk_probe_read_bandwidth", mb << 20, 40, C.byref(g))
        rates[f"{mb}MB"] = float(g.value)
    return {"gbs": max(rates.values()), "rates": rates,
            "source": "measured in this run: pk_probe_read_bandwidth (L2-resident read, 32/64 MB x 40)"}


def make_scene(args):
    from pike_gb300 import synth
    return synth.displaced_sphere_scene(subdivisions=args.subdivisions, width=args.width, height=args.height,
                                        bounces=args.bounces)


# ---------------------------------------------------------------- CPU (oracle)
def cpu_band_rows(src) -> int:
    """Rows of the CPU sample's band: a tenth of the image, in its middle."""
    return max(1, src.height // 10)


def cpu_run(src, bounces: int, seconds: float, threads: int, warmup: int = 1):
    """The CPU restatement on a bounded band of the frame: frames of a batch of
    rows in the middle of the image (the reference's BATCH_SIZE/invocationOffset
    mechanism, pike.js:133-147), `warmup` untimed band frames, then repeated
    until `seconds` of rendering."""
    from oracle import pyoracle
    t0 = time.perf_counter()
    pos, attrs = pyoracle.flatten(src)
    idx, layers = pyoracle.materials(src.materials)
    bvh = pyoracle.BVH(pos, src.tris)
    bvh_s = time.perf_counter() - t0
    env = pyoracle.Env(src.env_rgbe)
    rows = cpu_band_rows(src)
    batch = src.width * rows
    r = pyoracle.Renderer(src.width, src.height, batch=batch, threads=threads)
    r.set_scene(bvh, attrs, idx, layers)
    r.set_env(env)
    r.set_camera(src.camera_state(invocation_offset=(src.height // 2 - rows // 2) * src.width))
    for w in range(max(warmup, 0)):  # untimed: pages in the tables, spins up the worker threads
        r.set_render_state(1_000_000 + w)
        r.tick_batch(bounces)
    frames, rays, elapsed = 0, 0, 0.0
    while elapsed < seconds or frames == 0:
        r.reset_stats()
        r.set_render_state(frames)
        t = time.perf_counter()
        r.tick_batch(bounces)  # the band only
        elapsed += time.perf_counter() - t
        s = r.stats()
        rays += s["trace_rays"] + s["shadow_rays"]
        frames += 1
    return {"mrays": rays / elapsed / 1e6, "frames": frames, "rays": rays, "seconds": elapsed, "bvh_s": bvh_s,
            "sample": f"{frames} frame(s) of a {src.width}x{rows}-pixel band ({batch} pixels, {bounces} bounces)"}


def bench_config(args, src, world: int) -> dict:
    """The workload description both arms print (identical keys and values):
    what is rendered, how the GPU arm schedules it, and which band the CPU
    sample renders."""
    rows = cpu_band_rows(src)
    return {"workload": WORKLOAD, "triangles": src.n_tris, "resolution": f"{src.width}x{src.height}",
            "bounces": args.bounces, "env": "2048x1024 RGBE8", "parallelism": f"replicas{world}",
            "trace_mode": args.trace_mode, "node_record_bytes": args.node_records,
            "frame_overlap": args.trace_mode != "chunked" and (
                args.overlap == "on" or (args.overlap == "auto" and (
                    args.frames_in_flight == 1 or src.width * src.height < (1 << 20)))),
            "frames_in_flight": args.frames_in_flight,
            "l2": "working set > L2 (BVH+triangles 150 MB, ray queues 400 MB); no flush between steps",
            "cpu_sample": f"CPU arm and cpu_baseline: band of {rows} rows x {src.width} (rows "
                          f"{src.height // 2 - rows // 2}..{src.height // 2 - rows // 2 + rows - 1}) per frame, "
                          f"same scene, camera and bounces; Mrays/s is per ray traced"}


def reference_arm(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    src = make_scene(args)
    threads = os.cpu_count() or 1
    per_step = max(args.cpu_seconds / max(args.steps, 1), 0.5)
    res = cpu_run(src, args.bounces, per_step * args.steps, threads, warmup=max(args.warmup, 1))
    value = res["mrays"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * res["seconds"] / res["frames"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(args, src, dist_env()[1]),
        "measured": {"bvh_build_s": res["bvh_s"], "band_frames": res["frames"], "warmup_band_frames": max(args.warmup, 1),
                     "note": "CPU restatement of the reference path (oracle); the reference is JavaScript+WGSL "
                             "on WebGPU, which cannot run on this machine"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": res["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- GPU
def setup_context(src, local: int):
    import numpy as np
    from pike_gb300 import _lib
    from pike_gb300._lib import Context, ptr
    from pike_gb300.passes import CameraPass  # noqa: F401  (API mirror; the bench drives the C ABI directly)
    ctx = Context(local)
    ctx.call("pk_configure", src.width, src.height, src.width * src.height)
    tr = np.zeros(3)
    ctx.call("pk_scene_flatten", ptr(src.pos), ptr(src.normal), ptr(src.tangent), ptr(src.uv), src.pos.shape[0],
             ptr(src.tris), src.tris.shape[0], 1.0, ptr(tr))
    ctx.call("pk_materials_set", ptr(src.materials), src.materials.shape[0])
    ctx.call("pk_sync")
    ctx.timer_start()
    ctx.call("pk_bvh_build", _lib.PK_BVH_SWEEP)
    bvh_ms = ctx.timer_stop()
    env = np.ascontiguousarray(src.env_rgbe)
    ctx.call("pk_env_build", ptr(env), env.shape[1], env.shape[0])
    return ctx, bvh_ms


def camera_struct(src):
    from pike_gb300._lib import CameraState
    st = src.camera_state()
    cs = CameraState()
    cs.pos[:] = st["pos"]
    cs.dir[:] = st["dir"]
    cs.fov, cs.focal_depth, cs.aperture_size = st["fov"], st["focalDepth"], st["apertureSize"]
    cs.distortion, cs.bokeh, cs.invocation_offset = st["distortion"], st["bokeh"], 0
    return cs


def read_stats(ctx):
    import numpy as np
    from pike_gb300._lib import ptr
    s = np.zeros(10, np.uint64)
    ctx.call("pk_read_stats", ptr(s))
    keys = ["closest_fetch", "closest_tests", "shadow_fetch", "shadow_tests", "closest_rays", "shadow_rays",
            "closest_hits", "shadow_hits", "rays_traced", "frames"]
    return {k: int(v) for k, v in zip(keys, s)}


def read_timing(ctx):
    import numpy as np
    from pike_gb300._lib import ptr
    t = np.zeros(16, np.float32)
    ctx.call("pk_read_timing", ptr(t))
    kinds = ["camera", "trace", "compact", "shade", "shadow", "accumulate", "postprocess", "other"]
    return {k: {"ms": float(t[i]), "launches": int(t[8 + i])} for i, k in enumerate(kinds)}


def hit_agreement(ctx, mode_a: int, mode_b: int, bounces: int = 2, full: bool = True):
    """Per-ray closest-hit agreement of two traversal modes on the pass path
    (camera rays, then bounce rays shaded from mode_b's hits): rays whose
    {t, slot, barycentrics} differ (full) or whose hit triangle id differs,
    out of all rays traced."""
    import numpy as np
    from pike_gb300 import _lib
    from pike_gb300._lib import ptr

    def counters():
        c = np.zeros(8, np.uint32)
        ctx.call("pk_read_counters", ptr(c))
        return c

    def hit_rows(mode):
        ctx.call("pk_set_trace_mode", mode)
        ctx.call("pk_clear_hits_misses")
        ctx.call("pk_trace")
        k = int(counters()[1])
        out = np.zeros((k, 16), np.uint32)
        if k:
            ctx.call("pk_read_hits", 0, k, ptr(out))
        keys = np.ascontiguousarray(out[:, 4:16]).view(np.dtype((np.void, 48))).ravel()
        return keys, out[:, :3]

    ctx.call("pk_set_render_state", 0, 0.0)
    for name in ("clear_color", "clear_hits_misses", "clear_rays", "camera"):
        ctx.call("pk_" + name)
    total = differ = 0
    for _ in range(bounces):
        total += int(counters()[3])
        ka, va = hit_rows(mode_a)
        kb, vb = hit_rows(mode_b)
        common, ia, ib = np.intersect1d(ka, kb, assume_unique=True, return_indices=True)
        cols = slice(0, 3) if full else slice(1, 2)
        differ += (ka.size - common.size) + (kb.size - common.size) + int((va[ia, cols] != vb[ib, cols]).any(axis=1).sum())
        for name in ("shade_hit", "trace_shadow", "shade_miss"):
            ctx.call("pk_" + name)
    return total, differ


def warm_graphs(ctx, first_sample: int, B: int):
    """Replays every frame slot once (a counting or timing frame re-captures a
    slot's graph), so no capture falls inside a timed region."""
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_render_frames", 8, B)  # up to eight slots
    ctx.call("pk_sync")


def profile_case(name: str, local: int = 0):
    """One small invocation of a form kernel, for ncu captures (a few seconds,
    well under a GB on the device): `wide` = icosphere7 + box (327,690
    triangles) at 480x270, 8 bounces, 8-wide traversal; `adjoint` = icosphere6
    + box at 256x256, 4 spp, depth 4, one render and one adjoint; `batch` = 16
    requests over 2 scenes (9,998 / 327,690 triangles), half the batching
    workload's resolutions, <= 4 spp, block 128, stack 16, chunk 4, rendered
    twice (the second launch is the one to capture); `wide_soup` = the
    8,388,608-triangle soup at 480x270 through the 8-wide traversal."""
    from pike_gb300 import _lib, synth
    if name in ("wide", "wide_soup"):
        if name == "wide":
            src = synth.displaced_sphere_scene(subdivisions=7, width=480, height=270)
        else:
            src = synth.triangle_soup_scene(width=480, height=270)
        ctx, _ = setup_context(src, local)
        ctx.call("pk_set_trace_mode", _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_WIDE)
        ctx.call("pk_set_camera", camera_struct(src))
        ctx.call("pk_set_render_state", 0, 0.0)
        ctx.call("pk_render_frames", 1, 8)
        ctx.call("pk_sync")
    elif name == "adjoint":
        import torch
        from pike_gb300.diff import DiffScene
        src = synth.displaced_sphere_scene(subdivisions=6, width=256, height=256, env_size=(64, 32))
        scene = DiffScene(src, 256, 256, spp=4, depth=4, device=local)
        albedo, rough, env = scene.source_params(env_size=(256, 128), sun=20.0)
        scene.set_env_sampling(env)
        img = scene.render(albedo, rough, env, seed=0)
        scene.backward(albedo, rough, env, torch.ones_like(img), seed=0)
        torch.cuda.synchronize()
    else:
        from pike_gb300.batch import Batch, random_requests, scene_context
        srcs = [synth.small_scene(n_boxes=833), synth.displaced_sphere_scene(subdivisions=7, width=16, height=16)]
        ctxs = [scene_context(x, local) for x in srcs]
        reqs = random_requests(16, 2, seed=7)
        for r in reqs:
            r.width, r.height, r.spp = max(64, r.width // 2), max(64, r.height // 2), min(r.spp, 4)
        b = Batch(ctxs)
        b.set_requests(reqs)
        b.set_config(128, 16, 4)
        b.render(1)
        b.reset()
        b.render(1)
    print(json.dumps({"profile_case": name, "ok": True}))


def wide_form(ctx, args, B: int, first_sample: int, plain_mode: int):
    """Form (1): the 8-wide compressed BVH traced through the same frame
    pipeline; throughput, work per ray and closest-hit agreement with the
    drop-in traversal."""
    from pike_gb300 import _lib
    wide_mode = _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_WIDE
    ctx.call("pk_sync")
    ctx.timer_start()
    ctx.call("pk_set_trace_mode", wide_mode)
    build_ms = ctx.timer_stop()
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_render_frames", max(args.warmup, 1), B)
    ctx.call("pk_reset_stats")
    ctx.call("pk_set_counting", 1)
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_render_frames", 1, B)
    ctx.call("pk_sync")
    counts = read_stats(ctx)
    ctx.call("pk_set_counting", 0)
    ctx.call("pk_set_timing", 1)
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_render_frames", 4, B)
    ctx.call("pk_sync")
    kt = read_timing(ctx)
    ctx.call("pk_set_timing", 0)
    warm_graphs(ctx, first_sample, B)
    steps = max(1, min(args.steps, 32))
    ctx.call("pk_reset_stats")
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_sync")
    ctx.timer_start()
    ctx.call("pk_render_frames", steps, B)
    ms = ctx.timer_stop()
    rays = read_stats(ctx)["rays_traced"]
    total, differ = hit_agreement(ctx, plain_mode, wide_mode, full=False)
    # the FP32 binary reference of form (1): same tree, outward-rounded FP32 boxes, (t, slot) ties
    exact_mode = _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_EXACT
    etotal, ediffer = hit_agreement(ctx, exact_mode, wide_mode)
    ctx.call("pk_set_trace_mode", exact_mode)
    ctx.call("pk_reset_stats")
    ctx.call("pk_set_counting", 1)
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_render_frames", 1, B)
    ctx.call("pk_sync")
    ecounts = read_stats(ctx)
    ctx.call("pk_set_counting", 0)
    warm_graphs(ctx, first_sample, B)
    ctx.call("pk_reset_stats")
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_sync")
    ctx.timer_start()
    ctx.call("pk_render_frames", steps, B)
    ems = ctx.timer_stop()
    erays = read_stats(ctx)["rays_traced"]
    # the plain schedule of the drop-in: each warp takes 32 consecutive rays
    # and traces them to the end (one ray per lane, as trace.wgsl runs one
    # invocation per ray), no refill or bounded inner loop
    ctx.call("pk_set_trace_mode", _lib.PK_TRACE_CHUNKED)
    warm_graphs(ctx, first_sample, B)
    ctx.call("pk_reset_stats")
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_sync")
    ctx.timer_start()
    ctx.call("pk_render_frames", steps, B)
    cms = ctx.timer_stop()
    crays = read_stats(ctx)["rays_traced"]
    ctx.call("pk_set_trace_mode", plain_mode)
    tr = kt["trace"]
    R = max(counts["closest_rays"], 1)
    return {"value": rays / (ms / 1000.0) / 1e6, "unit": UNIT, "steps": steps, "ms_per_step": ms / steps,
            "closest_hit_launch_ms": tr["ms"] / max(tr["launches"], 1), "wide_build_ms": build_ms,
            "wide_nodes_per_ray": counts["closest_fetch"] / R, "tri_tests_per_ray": counts["closest_tests"] / R,
            "shadow_wide_nodes_per_ray": counts["shadow_fetch"] / max(counts["shadow_rays"], 1),
            "node_bytes": 80,
            "closest_hit_agreement": {"rays": total, "differ": differ, "fraction_equal": 1.0 - differ / max(total, 1),
                                      "compared": "hit triangle id (the drop-in uses Moller-Trumbore, form (1) "
                                                  "the watertight test)",
                                      "note": "camera + first bounce rays, pass path; differing rays are the "
                                              "drop-in's truncated-box misses, t ties and edge hits where the "
                                              "two triangle tests disagree (the wide result equals brute "
                                              "force, tests/test_gpu_wide.py)"},
            "fp32_binary": {"value": erays / (ems / 1000.0) / 1e6, "unit": UNIT, "ms_per_step": ems / steps,
                            "node_bytes": 64,
                            "fetch_units_per_ray": ecounts["closest_fetch"] / max(ecounts["closest_rays"], 1),
                            "closest_hit_agreement_with_wide": {"rays": etotal, "differ": ediffer,
                                                                "fraction_equal": 1.0 - ediffer / max(etotal, 1)}},
            "chunked_dropin": {"value": crays / (cms / 1000.0) / 1e6, "unit": UNIT, "ms_per_step": cms / steps,
                               "wide_over_chunked": (rays / ms) / max(crays / cms, 1e-9),
                               "schedule": "the drop-in's kernels with 32 consecutive rays per warp traced to the "
                                           "end (one ray per lane, no refill, no bounded inner loop); same "
                                           "frame pipeline"}}


def adjoint_form(args, local: int):
    """Form (3), the differentiation workload: the 1.31M-triangle scene at
    512x512, 16 spp, depth 4; parameters = 256 group albedos (RGB), 256
    roughness values and a 256x128 RGB environment; the drop-in's estimator
    (GGX VNDF sampling, lobe choice, env NEE with MIS) with detached sampling.
    Forward and adjoint throughput (rays/s, full gradients/s), 32 central
    differences (h = 1e-3, common random numbers, sampling roughness and
    environment tables held) against the adjoint, and Adam inverse rendering
    with the recovery error of every parameter kind."""
    import numpy as np
    import torch
    from pike_gb300 import synth
    from pike_gb300.diff import DiffScene, inverse_render, l2_loss
    src = synth.displaced_sphere_scene(subdivisions=args.subdivisions, width=512, height=512, env_size=(64, 32))
    scene = DiffScene(src, 512, 512, spp=16, depth=4, device=local)
    albedo, rough, env = scene.source_params(env_size=(256, 128), sun=20.0)
    n_free = src.materials.shape[0] - 1
    scene.set_env_sampling(env)
    target = scene.render(albedo, rough, env, seed=12345)
    a0 = torch.full_like(albedo, 0.5)
    a0[n_free:] = albedo[n_free:]
    r0 = torch.full_like(rough, 0.5)
    r0[n_free:] = rough[n_free:]
    e0 = torch.full_like(env, float(env.mean()))
    scene.set_env_sampling(e0)
    for _ in range(2):  # warm-up
        img = scene.render(a0, r0, e0, seed=0)
        d = 2.0 * (img - target) / (3 * 512 * 512)
        scene.backward(a0, r0, e0, d, seed=0)
    reps = 5
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fwd_rays = 0
    for k in range(reps):
        img = scene.render(a0, r0, e0, seed=k)
        fwd_rays += scene.rays()
    fwd_s = time.perf_counter() - t0
    d = 2.0 * (img - target) / (3 * 512 * 512)
    d[..., 3] = 0
    t0 = time.perf_counter()
    adj_rays = 0
    for k in range(reps):
        ga, gr, ge = scene.backward(a0, r0, e0, d, seed=reps - 1)
        adj_rays += scene.rays()
    adj_s = time.perf_counter() - t0
    # central differences at 32 parameters drawn among those whose gradient is
    # at least 1% of the largest of its kind; criterion |g - fd| <= 1% |fd|
    rng = np.random.default_rng(2024)
    img = scene.render(a0, r0, e0, seed=7)
    d = 2.0 * (img - target) / (3 * 512 * 512)
    d[..., 3] = 0
    ga, gr, ge = scene.backward(a0, r0, e0, d, seed=7)
    grads, base = {"albedo": ga, "rough": gr, "env": ge}, {"albedo": a0, "rough": r0, "env": e0}

    def pick(name, k):
        g = grads[name].abs()
        if name != "env":
            g = g[:n_free]
        cand = torch.nonzero(g >= 0.01 * g.max()).cpu().numpy()
        return [(name, tuple(int(x) for x in cand[i])) for i in rng.choice(cand.shape[0], k, replace=False)]

    picks = pick("albedo", 12) + pick("rough", 10) + pick("env", 10)
    worst, within = 0.0, 0
    for name, idx in picks:
        vals = []
        for sgn in (1.0, -1.0):
            p = {k: v.clone() for k, v in base.items()}
            p[name][idx] += sgn * 1e-3
            vals.append(float(l2_loss(scene.render(p["albedo"], p["rough"], p["env"], seed=7,
                                                   rough_sampling=r0).double(), target.double())))
        fd = (vals[0] - vals[1]) / 2e-3
        g = float(grads[name][idx])
        rel = abs(g - fd) / abs(fd)
        worst = max(worst, rel)
        within += rel <= 0.01
    # inverse rendering: a target with 8x the samples, Adam with fresh samples
    # every step, the sampling tables and roughness following the current
    # parameters; the loss evaluated at a fixed seed against that target
    scene.set_env_sampling(env)
    target_hq = sum(scene.render(albedo, rough, env, seed=50000 + k) for k in range(8)) / 8
    steps = 200
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    a, r, e, hist = inverse_render(scene, target_hq, a0, r0, e0, steps=steps, lr=0.02, n_free=n_free,
                                   seed_per_step=True, seed=0)
    torch.cuda.synchronize()
    opt_s = time.perf_counter() - t0

    def eval_loss(A, R, E):  # L2 error of the expected image, estimated from 8 renders
        scene.set_env_sampling(E)
        return float(l2_loss(sum(scene.render(A, R, E, seed=90000 + k) for k in range(8)) / 8, target_hq))

    # the same with the environment known (materials only): how well the
    # gradients recover what the image constrains without the map's ambiguity
    a_k, r_k, _, hist_k = inverse_render(scene, target_hq, a0, r0, env, steps=steps, lr=0.02, n_free=n_free,
                                         seed_per_step=True, seed=0, optimise_env=False)
    # recovery error: parameters the image constrains (materials on hit
    # surfaces, env texels the camera or a bounce sees: non-zero gradient at
    # the start)
    seen_m = (ga[:n_free].abs().sum(-1) > 0)
    # the 64 materials the image constrains most (largest albedo gradient at the start)
    top_m = torch.zeros_like(seen_m)
    top_m[torch.argsort(ga[:n_free].abs().sum(-1), descending=True)[:64]] = True
    seen_e = (ge.abs().sum(-1) > 0)
    rel_env = lambda E: float(((E - env).abs().sum(-1)[seen_e] / env.sum(-1)[seen_e]).mean())
    return {"workload": "icosphere8+openbox 512x512, 16 spp, depth 4; 256 albedos (RGB), 256 roughness, "
                        "256x128 RGB env (98,304 env values); the drop-in's estimator, detached sampling",
            "forward": {"value": fwd_rays / fwd_s / 1e6, "unit": "Mrays/s", "ms": 1000 * fwd_s / reps},
            "adjoint": {"value": adj_rays / adj_s / 1e6, "unit": "Mrays/s", "ms": 1000 * adj_s / reps,
                        "grads_per_s": reps / adj_s},
            "adjoint_vs_forward_rays": (adj_rays / adj_s) / (fwd_rays / fwd_s),
            "finite_differences": {"params": len(picks), "h": 1e-3, "within_1pct": int(within),
                                   "worst_rel_err": worst,
                                   "selection": "random among parameters with |grad| >= 1% of the largest of its kind"},
            "inverse_rendering": {
                "steps": steps, "seconds": opt_s,
                "objective": "L2 to a 128-spp target; fresh 16-spp samples every step, the gradient from an independent "
                             "16-spp replay (Adam, lr 0.02 cosine-decayed to 4e-4); loss_eval = L2 of a 128-spp render",
                "loss_first": hist[0], "loss_last": hist[-1],
                "loss_eval_start": eval_loss(a0, r0, e0), "loss_eval_end": eval_loss(a, r, e),
                "loss_eval_at_hidden_params": eval_loss(albedo, rough, env),
                "materials_seen": int(seen_m.sum()), "env_texels_seen": int(seen_e.sum()),
                "albedo_mae_start": float((a0[:n_free] - albedo[:n_free]).abs()[seen_m].mean()),
                "albedo_mae_end": float((a[:n_free] - albedo[:n_free]).abs()[seen_m].mean()),
                "roughness_mae_start": float((r0[:n_free] - rough[:n_free]).abs()[seen_m].mean()),
                "roughness_mae_end": float((r[:n_free] - rough[:n_free]).abs()[seen_m].mean()),
                "env_rel_l1_start": rel_env(e0), "env_rel_l1_end": rel_env(e),
                "albedo_mae_top64_start": float((a0[:n_free] - albedo[:n_free]).abs()[top_m].mean()),
                "albedo_mae_top64_end": float((a[:n_free] - albedo[:n_free]).abs()[top_m].mean()),
                "roughness_mae_top64_start": float((r0[:n_free] - rough[:n_free]).abs()[top_m].mean()),
                "roughness_mae_top64_end": float((r[:n_free] - rough[:n_free]).abs()[top_m].mean()),
                "env_known": {"loss_eval_end": eval_loss(a_k, r_k, env),
                              "albedo_mae_end": float((a_k[:n_free] - albedo[:n_free]).abs()[seen_m].mean()),
                              "albedo_mae_top64_end": float((a_k[:n_free] - albedo[:n_free]).abs()[top_m].mean()),
                              "roughness_mae_end": float((r_k[:n_free] - rough[:n_free]).abs()[seen_m].mean()),
                              "roughness_mae_top64_end": float((r_k[:n_free] - rough[:n_free]).abs()[top_m].mean())}}}


def batch_form(args, local: int):
    """Form (2), the batching workload: 64 requests over three resident scenes
    (ground + 833 boxes = 9,998 triangles; icosphere7 + box = 327,690;
    icosphere8 + box = 1,310,730), resolutions log-uniform 128x128..1920x1080,
    spp in {1,4,16,64}, depth 4..8, random orbit cameras.  One persistent
    launch (autotuned) against the same requests run one after another,
    through the batch kernel and through the drop-in pipeline."""
    import numpy as np
    from pike_gb300 import synth
    from pike_gb300._lib import ptr
    from pike_gb300.batch import Batch, random_requests, scene_context
    srcs = [synth.small_scene(n_boxes=833), synth.displaced_sphere_scene(subdivisions=7, width=16, height=16),
            synth.displaced_sphere_scene(subdivisions=args.subdivisions, width=16, height=16)]
    ctxs = [scene_context(s, local) for s in srcs]
    reqs = sorted(random_requests(64, 3, seed=2025), key=lambda r: r.paths)  # shortest first, in both runs
    batch = Batch(ctxs)
    batch.set_requests(reqs)
    total_paths = batch.info()[0]
    tune_ms = batch.autotune(sample_paths=min(total_paths, 32_000_000))
    cfg = batch.config()
    batch.render(1)  # graph capture + warm-up
    batch.reset()
    batch_ms = batch.render(1)
    lat = batch.latencies()
    # one request at a time through the same kernel
    seq_batch = []
    for r in reqs:
        batch.set_requests([r])
        batch.render(1)
        batch.reset()
        seq_batch.append(batch.render(1))
    batch.close()
    # one request at a time through the drop-in pipeline (spp frames of depth bounces)
    from pike_gb300.batch import _camera_struct
    seq_plain = []
    for r in reqs:
        ctx = ctxs[r.scene]
        ctx.call("pk_configure", r.width, r.height, r.width * r.height)
        ctx.call("pk_set_camera", _camera_struct(r.camera))
        ctx.call("pk_set_render_state", 0, 0.0)
        ctx.call("pk_render_frames", 4, r.depth)  # warm-up (graph capture of every slot at this size)
        ctx.call("pk_set_render_state", 0, 0.0)
        ctx.call("pk_sync")
        ctx.timer_start()
        ctx.call("pk_render_frames", r.spp, r.depth)
        seq_plain.append(ctx.timer_stop())
    for c in ctxs:
        c.close()
    done_b = np.cumsum(seq_batch)
    done_p = np.cumsum(seq_plain)
    return {"workload": "64 requests, 3 resident scenes (9,998 / 327,690 / 1,310,730 triangles), "
                        "128x128..1920x1080 log-uniform, spp {1,4,16,64}, depth 4..8, orbit cameras",
            "paths": int(total_paths), "autotuned": {"block": cfg[0], "stack": cfg[1], "chunk": cfg[2],
                                                     "sample_ms": tune_ms},
            "batch_ms": batch_ms, "paths_per_s": total_paths / (batch_ms / 1000.0),
            "request_order": "ascending path count (shortest first) in every column",
            "batch_latency_ms": {"mean": float(lat.mean()), "median": float(np.median(lat)),
                                 "max": float(lat.max())},
            "sequential_same_kernel": {"total_ms": float(done_b[-1]), "mean_latency_ms": float(done_b.mean())},
            "sequential_dropin": {"total_ms": float(done_p[-1]), "mean_latency_ms": float(done_p.mean())},
            "speedup_vs_sequential_same_kernel": float(done_b[-1]) / batch_ms,
            "speedup_vs_sequential_dropin": float(done_p[-1]) / batch_ms,
            "note": "batch images equal the drop-in's in distribution; the drop-in column renders spp frames "
                    "of 1 sample each (its wavefront queues are sized per request)"}


def binned_form(ctx, args, B: int, first_sample: int, sweep_ms: float):
    """The binned SAH build (PK_BVH_BINNED) of the same scene: build time and
    the drop-in frame rate on its tree (a different topology from bvh.js)."""
    from pike_gb300 import _lib
    times = []
    for _ in range(3):
        ctx.call("pk_sync")
        ctx.timer_start()
        ctx.call("pk_bvh_build", _lib.PK_BVH_BINNED)
        times.append(ctx.timer_stop())
    ctx.call("pk_set_trace_mode", _lib.PK_TRACE_PERSISTENT)
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_render_frames", 4, B)
    ctx.call("pk_reset_stats")
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_sync")
    steps = max(1, min(args.steps, 32))
    ctx.timer_start()
    ctx.call("pk_render_frames", steps, B)
    ms = ctx.timer_stop()
    rays = read_stats(ctx)["rays_traced"]
    return {"build_ms": min(times), "sweep_build_ms": sweep_ms, "value": rays / (ms / 1000.0) / 1e6, "unit": UNIT,
            "ms_per_step": ms / steps, "note": "binned SAH, 16 bins, leaves <= 8; frames differ from the reference's"}


def alias_env_form(args, local: int):
    """Form (1)'s alias-table environment sampling (PK_ENV_ALIAS) against the
    reference's equal-mass histogram on the benchmark scene: the shade
    kernel's launch time at 1920x1080 (pk_set_timing, one frame at a time),
    and the per-pixel variance of 32 single-sample frames at 480x270 (relative
    variance var/mean^2, averaged over lit pixels; same seeds in both modes)."""
    import numpy as np
    from pike_gb300 import _lib
    from pike_gb300._lib import ptr
    out = {"workload": "icosphere8+openbox, 2048x1024 env; shade timing at 1920x1080 (8 bounces), "
                       "variance over 32 frames at 480x270"}
    src = make_scene(args)
    ctx, _ = setup_context(src, local)
    ctx.call("pk_set_camera", camera_struct(src))
    ctx.call("pk_set_frames_in_flight", 1)
    B = args.bounces
    rgbe = np.ascontiguousarray(src.env_rgbe, np.uint8)
    for name, mode in (("histogram", _lib.PK_ENV_HISTOGRAM), ("alias", _lib.PK_ENV_ALIAS)):
        # table build: pk_env_build in histogram mode (upload of the texels
        # and env_sampler.js's tables), and the switch to alias mode (the
        # alias table from the texels already on the device)
        ctx.call("pk_set_env_sampling", _lib.PK_ENV_HISTOGRAM)
        ctx.call("pk_env_build", ptr(rgbe), rgbe.shape[1], rgbe.shape[0])
        ctx.call("pk_sync")
        ctx.timer_start()
        if mode == _lib.PK_ENV_HISTOGRAM:
            ctx.call("pk_env_build", ptr(rgbe), rgbe.shape[1], rgbe.shape[0])
        else:
            ctx.call("pk_set_env_sampling", mode)
        build_ms = ctx.timer_stop()
        ctx.call("pk_set_render_state", 0, 0.0)
        ctx.call("pk_render_frames", 2, B)
        ctx.call("pk_reset_stats")
        ctx.call("pk_set_timing", 1)
        ctx.call("pk_set_render_state", 0, 0.0)
        ctx.call("pk_render_frames", 4, B)
        ctx.call("pk_sync")
        kt = read_timing(ctx)
        ctx.call("pk_set_timing", 0)
        sh = kt["shade"]
        out[name] = {"shade_launch_ms": sh["ms"] / max(sh["launches"], 1), "table_build_ms": build_ms}
    ctx.close()
    small = make_scene(argparse.Namespace(subdivisions=args.subdivisions, width=480, height=270, bounces=B))
    ctx, _ = setup_context(small, local)
    ctx.call("pk_set_camera", camera_struct(small))
    frames = 32
    for name, mode in (("histogram", _lib.PK_ENV_HISTOGRAM), ("alias", _lib.PK_ENV_ALIAS)):
        ctx.call("pk_set_env_sampling", mode)
        ctx.call("pk_set_render_state", 0, 0.0)
        s1 = s2 = 0.0
        col = np.zeros((small.height, small.width, 4), np.float32)
        for _ in range(frames):
            ctx.call("pk_render_frames", 1, B)
            ctx.call("pk_read_color", ptr(col))
            c = np.maximum(col[..., :3].astype(np.float64), 0.0)
            s1 = s1 + c
            s2 = s2 + c * c
        m = s1 / frames
        var = np.maximum(s2 / frames - m * m, 0.0) * frames / (frames - 1)
        lit = m > 1e-6
        out[name]["mean_relative_variance"] = float((var[lit] / m[lit] ** 2).mean())
        out[name]["image_mean"] = float(m.mean())
    ctx.close()
    h, a = out["histogram"], out["alias"]
    out["variance_ratio_alias_over_histogram"] = a["mean_relative_variance"] / h["mean_relative_variance"]
    out["shade_time_ratio_alias_over_histogram"] = a["shade_launch_ms"] / h["shade_launch_ms"]
    return out


def precision_form(args, local: int):
    """Form (1)'s precision workload: the 8,388,608-triangle soup with the
    2048x1024 env at 1920x1080, depth 4: drop-in, FP32 binary reference and
    8-wide traversal on the same sweep-SAH tree; closest-hit agreement (camera
    + first bounce), work per ray and throughput."""
    from pike_gb300 import _lib, synth
    src = synth.triangle_soup_scene()
    ctx, bvh_ms = setup_context(src, local)
    ctx.call("pk_set_camera", camera_struct(src))
    B = 4
    out = {"workload": "triangle soup 8,388,608 tris (centroids U[-50,50]^3, edges log-uniform [0.01,1]), "
                       "1920x1080, depth 4", "bvh_build_ms": bvh_ms}
    modes = {"dropin": _lib.PK_TRACE_PERSISTENT, "fp32_binary": _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_EXACT,
             "wide": _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_WIDE}
    for name, mode in modes.items():
      try:
        ctx.call("pk_sync")
        ctx.timer_start()
        ctx.call("pk_set_trace_mode", mode)
        prep_ms = ctx.timer_stop()
        ctx.call("pk_reset_stats")
        ctx.call("pk_set_counting", 1)
        ctx.call("pk_set_render_state", 0, 0.0)
        ctx.call("pk_render_frames", 1, B)
        ctx.call("pk_sync")
        cnt = read_stats(ctx)
        ctx.call("pk_set_counting", 0)
        warm_graphs(ctx, 0, B)
        ctx.call("pk_reset_stats")
        ctx.call("pk_set_render_state", 0, 0.0)
        ctx.call("pk_sync")
        ctx.timer_start()
        ctx.call("pk_render_frames", 4, B)
        ms = ctx.timer_stop()
        rays = read_stats(ctx)["rays_traced"]
        R = max(cnt["closest_rays"], 1)
        # bytes per fetch unit: the drop-in counts three 20-byte reference nodes per
        # inner step (one 64-byte record here), the wide traversal one 80-byte node
        node_bytes = {"dropin": 20.0, "fp32_binary": 64.0 / 3.0, "wide": 80.0}[name]
        out[name] = {"value": rays / (ms / 1000.0) / 1e6, "unit": UNIT, "ms_per_frame": ms / 4,
                     "structure_ms": prep_ms, "fetch_per_closest_ray": cnt["closest_fetch"] / R,
                     "tests_per_closest_ray": cnt["closest_tests"] / R,
                     "node_bytes_per_closest_ray": node_bytes * cnt["closest_fetch"] / R}
      except Exception as e:  # e.g. a traversal stack overflow reported by the device
        out[name] = {"error": str(e)}
    wide, exact, plain = modes["wide"], modes["fp32_binary"], modes["dropin"]
    t, d = hit_agreement(ctx, exact, wide)
    out["agreement_fp32_binary_vs_wide"] = {"rays": t, "differ": d, "fraction_equal": 1.0 - d / max(t, 1)}
    t, d = hit_agreement(ctx, plain, wide, full=False)
    out["agreement_dropin_vs_wide"] = {"rays": t, "differ": d, "fraction_equal": 1.0 - d / max(t, 1),
                                       "compared": "hit triangle id (t and barycentrics come from different "
                                                   "triangle tests)"}
    ctx.close()
    return out


def gpu_arm(args):
    import ctypes as C

    rank, world, local = dist_env()
    D = Dist(world, local)
    src = make_scene(args)
    ctx, bvh_ms = setup_context(src, local)
    from pike_gb300 import _lib
    mode = _lib.PK_TRACE_CHUNKED if args.trace_mode == "chunked" else _lib.PK_TRACE_PERSISTENT
    if args.trace_mode == "wide":
        mode |= _lib.PK_TRACE_WIDE
    if args.node_records == 32:
        mode |= _lib.PK_TRACE_COMPACT_RECORDS
    ctx.call("pk_set_trace_mode", mode)
    ctx.call("pk_set_frame_overlap", {"auto": _lib.PK_OVERLAP_AUTO, "on": 1, "off": 0}[args.overlap])
    ctx.call("pk_set_frames_in_flight", args.frames_in_flight)
    cam = camera_struct(src)
    ctx.call("pk_set_camera", cam)
    B = args.bounces
    first_sample = rank  # replicas render interleaved samples r, r+N, ...

    # warm-up
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_render_frames", max(args.warmup, 0), B)
    ctx.call("pk_sync")

    # counting frame: the reference algorithm's node fetches / triangle tests (not timed)
    ctx.call("pk_reset_stats")
    ctx.call("pk_set_counting", 1)
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_render_frames", 1, B)
    ctx.call("pk_sync")
    counts = read_stats(ctx)
    ctx.call("pk_set_counting", 0)

    # per-kernel CUDA-event timing (instrumented frames, not the headline)
    ctx.call("pk_reset_stats")
    ctx.call("pk_set_timing", 1)
    tf = 4
    ctx.call("pk_set_render_state", first_sample, 0.0)
    ctx.call("pk_render_frames", tf, B)
    ctx.call("pk_sync")
    kt = read_timing(ctx)
    ctx.call("pk_set_timing", 0)
    warm_graphs(ctx, first_sample, B)

    # timed region (device time, CUDA events on the library's stream)
    clocks = Clocks(local)
    ctx.call("pk_reset_stats")
    ctx.call("pk_set_render_state", first_sample, 0.0)
    D.barrier()
    ctx.call("pk_sync")
    clocks.start()
    ctx.timer_start()
    ctx.call("pk_render_frames", args.steps, B)
    ms = ctx.timer_stop()
    clk = clocks.stop()
    st = read_stats(ctx)
    rays_local = st["rays_traced"]
    D.barrier()
    value, ms_max = replica_throughput(D, rays_local, ms)
    npix = src.width * src.height
    spp_mpix = world * args.steps * npix / (ms_max / 1000.0) / 1e6

    # end to end through the C ABI with host buffers: host wall clock from
    # before the first call to after pk_sync has waited for the last frame and
    # the last image copy (device events bracket the same loop for reference)
    e2e_steps = args.steps
    img = ctx.pinned((src.height, src.width, 4), "uint8")
    h2d = C.sizeof(cam) + 8
    # warm-up of the same per-frame calls (untimed): every frame slot, the
    # display read path
    for s in range(8):
        ctx.call("pk_set_render_state", first_sample + s, 0.0)
        ctx.call("pk_set_camera", cam)
        ctx.call("pk_render_frame", B)
        ctx.call("pk_read_display_async", img.array.ctypes.data_as(C.c_void_p))
    ctx.call("pk_sync")
    ctx.call("pk_reset_stats")
    D.barrier()
    ctx.call("pk_sync")
    t_host0 = time.perf_counter()
    ctx.timer_start()
    for s in range(e2e_steps):
        ctx.call("pk_set_render_state", first_sample + s, 0.0)
        ctx.call("pk_set_camera", cam)
        ctx.call("pk_render_frame", B)
        ctx.call("pk_read_display_async", img.array.ctypes.data_as(C.c_void_p))
    e2e_dev_ms = ctx.timer_stop()
    ctx.call("pk_sync")
    e2e_ms = 1000.0 * (time.perf_counter() - t_host0)
    e2e_rays = read_stats(ctx)["rays_traced"]
    e2e_ms_max = D.max(e2e_ms)
    e2e_value = D.sum(float(e2e_rays)) / (e2e_ms_max / 1000.0) / 1e6
    img.free()
    forms = None
    if rank == 0 and args.trace_mode != "wide" and not args.no_forms:
        forms = {"wide_bvh": wide_form(ctx, args, B, first_sample, mode)}
        forms["adjoint"] = adjoint_form(args, local)
        forms["batching"] = batch_form(args, local)
        forms["binned_bvh"] = binned_form(ctx, args, B, first_sample, bvh_ms)
        forms["alias_env"] = alias_env_form(args, local)
        if not args.no_precision:
            forms["precision_soup"] = precision_form(args, local)

    l2 = l2_peak(ctx) if rank == 0 else None
    if rank == 0:
        peak, peak_kind = load_peak_hbm()
        tr = kt["trace"]
        trace_ms = tr["ms"] / max(tr["launches"], 1)
        R, H = counts["closest_rays"], counts["closest_hits"]
        node_bytes = 80 if args.trace_mode == "wide" else 20
        alg_bytes_frame = (node_bytes * counts["closest_fetch"] + 52 * counts["closest_tests"] + 48 * R + 64 * H
                           + 48 * (R - H))
        alg_bytes_launch = alg_bytes_frame / B
        achieved = alg_bytes_launch / (trace_ms / 1000.0) / 1e9
        traffic = profiled_traffic()
        total_ms = sum(v["ms"] for v in kt.values())
        measured = {"spp_mpix_per_s": spp_mpix, "spp_per_s": spp_mpix / (npix / 1e6),
                    "rays_per_step": rays_local / args.steps, "bvh_build_ms": bvh_ms,
                    "kernel_share": {k: round(v["ms"] / total_ms, 4) for k, v in kt.items() if total_ms}}
        # k_set_state, k_camera, per bounce {closest trace, compaction, shade, shadow trace},
        # k_accumulate, k_postprocess, k_end_frame
        launches_per_frame = 4 * B + 5
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(args, src, world),
            "measured": measured,
            "roofline": {"bound": "hbm", "kernel": "closest-hit traversal (trace.wgsl + fused shade_miss)", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                         "peak_l2": l2["gbs"] if l2 else None,
                         "frac_l2": achieved / l2["gbs"] if l2 and l2["gbs"] else None,
                         "peak_l2_source": l2["source"] if l2 else None,
                         "traffic": traffic,
                         "traffic_source": "carried over: profiles/trace_closest_dram.txt, an ncu capture of this "
                                           "workload's closest-hit launches (dram__bytes_read.sum + "
                                           "dram__bytes_write.sum per launch); not measured in this run",
                         "algorithmic_bytes_per_launch": alg_bytes_launch,
                         "launch_ms": trace_ms,
                         "bytes_model": f"{node_bytes}*node_fetch + 52*tri_test + 48*ray + 64*hit + 48*miss"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": src.width * src.height * 4, "steps": e2e_steps,
                    "timing": "host perf_counter around the calls plus the final pk_sync",
                    "device_ms": e2e_dev_ms},
            "gpu_launches": launches_per_frame * args.steps,
            "clocks": clk,
            "counts_per_frame": counts,
        }
        if forms:
            line["forms"] = forms
        if world == 1 and not args.no_cpu_baseline:
            res = cpu_run(src, B, args.cpu_seconds, os.cpu_count() or 1, warmup=1)
            line["cpu_baseline"] = {"value": res["mrays"], "unit": UNIT, "cores": os.cpu_count() or 1,
                                    "kind": "port", "sample": res["sample"], "bvh_build_s": res["bvh_s"]}
        print(json.dumps(line))
    ctx.close()
    D.close()
    return 0


def main():
    args = parse()
    if args.profile_case:
        profile_case(args.profile_case)
        return 0
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
