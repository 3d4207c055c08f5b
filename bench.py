"""Benchmark of the trace path on one GB300 (or N replicas under torchrun).

Workload (one "step"): closest-hit ray cast of 2,097,152 rays — a 1024x1024 pinhole camera at distance 3
plus 1,048,576 rays with origins uniform in the sphere's AABB expanded 1.5x and directions uniform on
the sphere — against the 1.3M-triangle scene (level-8 displaced icosphere, 1,310,720 triangles, plus a
2-triangle ground plane and a 2-triangle area light; 1,310,724 triangles).  Inputs and outputs stay
resident in HBM for `value`; `e2e` runs the same step through the host-buffer C ABI call
(reina_raycast) with the rays in pinned host memory and the hits written back to pinned host memory every
step (the kernel reads and writes them in place over the coherent CPU-GPU link).
L2 (129 MB) is flushed by writing a 512 MB buffer between timed steps (outside the timed events).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Beside the headline line's required keys, the JSON carries: `render` (the 1.3M-triangle scene at
1920x1080, 64 spp, 12 bounces, NEE+MIS, and the Cornell room, each in the three forms: the wave engine,
the pass-by-pass wavefront and the plain megakernel), `batched` (256 seeded scenes rendered in one
autotuned batched call vs one at a time in the plain forms and on the wave engine; `--batch-scenes`),
`served` (a Poisson request stream through the request server under each wave-slot policy vs one at a
time; `--serve-seconds`), `instanced` (256 instances of one sphere built flat and as two levels: device
memory, build time, ray-cast time; `--instances`), `emissive_cdf` (the emissive CDF build of a
1.3M-triangle emissive mesh on the host and on the GPU), and `cpu_baseline`.
`--profile`, `--profile-render` and `--profile-batch` launch small fixed workloads for ncu and exit.

`--impl reference` times the CPU restatement of the path (oracle/, FP32, all host threads) on a bounded
sample of the same rays per step; the reference's own Vulkan ray-tracing path cannot run on this
hardware (no graphics stack, no RT cores).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "reina-vk_gb300"))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

NODE_BYTES = 80
TRI_BYTES = 48
RAY_BYTES = 32
HIT_BYTES = 16
FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 512 << 20
N_CAMERA_SIDE = 1024
N_RANDOM = 1 << 20
METRIC = "rays/s on 1.3M-tri scene (closest-hit ray cast)"


def _peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def _profiled_traffic() -> float | None:
    """DRAM bytes per launch of the ray-cast kernel from the committed ncu summary (None if absent)."""
    p = ROOT / "profiles" / "raycast_closest_l8.md"
    if not p.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", p.read_text())
    return float(m.group(1)) if m else None


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu_index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max_over_ranks(values, device: str) -> list:
    """Per-rank timings reduced to their maximum over the replicas (the slowest replica sets the job's
    time); the process group must be initialized."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def replica_throughput(world_size: int, units_per_rank: int, seconds: float) -> float:
    """Whole-job throughput of N replicas: all ranks' units over the (max-reduced) time."""
    return world_size * units_per_rank / seconds


def _build_workload(R, ctx):
    import scenes

    t0 = time.perf_counter()
    scene, tris, geo = scenes.large_scene(R, ctx, 8)
    build_s = time.perf_counter() - t0
    rays = scenes.raycast_rays(R, 8, N_CAMERA_SIDE, N_CAMERA_SIDE, N_RANDOM, geo[0][0])
    return scene, tris, rays, build_s


def run_ours(args) -> dict | None:
    import torch

    import build as pkg_build
    import reina_gb300 as R

    ws, rank, local = _dist()
    pkg_build.build()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    ctx = R.Context(local)
    scene, tris, rays, build_s = _build_workload(R, ctx)
    st = scene.stats()
    n = rays.shape[0]
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(n, 8).copy()).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    # Counting build (not timed): BVH8 nodes visited and triangles tested by these rays.
    nodes_v, tris_t = R.raycast_counters(ctx, scene, d_rays.data_ptr(), n, R.RAY_CLOSEST, sptr)
    bytes_per_ray = RAY_BYTES + HIT_BYTES + NODE_BYTES * nodes_v / n + TRI_BYTES * tris_t / n
    any_nodes, any_tris = R.raycast_counters(ctx, scene, d_rays.data_ptr(), n, R.RAY_ANY, sptr)

    def step(flags=R.RAY_CLOSEST):
        R.raycast_device(ctx, scene, d_rays.data_ptr(), n, d_hits.data_ptr(), flags, sptr)

    if args.profile_render:
        # Profiling mode (for ncu): the large scene at 480x270, 4 spp, 12 bounces, NEE+MIS, two frames.
        W, H = 480, 270
        iv, ip = R.camera_matrices((0.0, 0.4, 3.6), (0.0, -0.12, -1.0), (0.0, 1.0, 0.0), np.radians(40.0), W / H)
        pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=4, max_bounces=12, focus_dist=3.6)
        opts = R.render_options(W, H, R.MODE_NEE_MIS, 1, R.ENV_CONSTANT, (0.3, 0.3, 0.35))
        acc = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        for _ in range(2):
            R.render_device(ctx, scene, pc, opts, acc.data_ptr(), 0, sptr)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "render_large_480x270x4spp", "frames": 2}))
        return None

    if args.profile_batch:
        # Profiling mode (for ncu): the first 16 scenes of the batched workload at 2 spp, batched once.
        import scenes

        pool, _ = build_pool(R, ctx, 16)
        jobs, keep = [], []
        for sc, p in pool:
            pc, opts = scenes.batch_job(R, sc, dict(p, spp=min(p["spp"], 2)))
            acc = torch.zeros((p["side"], p["side"], 4), dtype=torch.float32, device="cuda")
            keep.append(acc)
            jobs.append(R.DeviceRenderJob(sc, pc, opts, acc.data_ptr()))
        st_b = R.render_batch_device(ctx, jobs, sptr)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "batch_16_scenes_2spp", "segments": st_b["rays"], "shadow_rays": st_b["shadow_rays"]}))
        return None

    if args.profile:
        # Profiling mode (for ncu): one warm-up, then `steps` closest-hit launches and one any-hit launch.
        step()
        for _ in range(args.steps):
            step()
        step(R.RAY_ANY)
        torch.cuda.synchronize()
        print(json.dumps({"profile": "raycast_l8", "launches": args.steps + 2, "nodes_per_ray": nodes_v / n,
                          "tris_per_ray": tris_t / n, "bytes_per_ray": bytes_per_ray}))
        return None

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        step()
        ends[k].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    # any-hit (shadow-ray form) on the same rays, reported beside the headline
    any_ms = []
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        step(R.RAY_ANY)
        ends[k].record(stream)
    torch.cuda.synchronize()
    any_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    clk = clocks.stop()

    # e2e through the host-buffer C ABI call, pinned host memory, copies in the timed region.
    h_rays = torch.from_numpy(rays.view(np.float32).reshape(n, 8).copy()).pin_memory()
    h_hits = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    for _ in range(max(1, args.warmup)):
        R.raycast_into(ctx, scene, h_rays.data_ptr(), n, h_hits.data_ptr(), R.RAY_CLOSEST)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e2e_total = 0.0
    for _ in range(args.steps):
        flush.zero_()   # L2 flushed before every step, as for `value` (outside the timed call)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        R.raycast_into(ctx, scene, h_rays.data_ptr(), n, h_hits.data_ptr(), R.RAY_CLOSEST)
        torch.cuda.synchronize()
        e2e_total += time.perf_counter() - t0
    e2e_s = e2e_total / args.steps

    mean_ms = float(np.mean(step_ms))
    if ws > 1:
        mean_ms, e2e_s = reduce_max_over_ranks([mean_ms, e2e_s], "cuda")
    if rank != 0:
        return None
    peak, peak_kind = _peak_hbm()
    achieved = bytes_per_ray * n / (mean_ms * 1e-3) / 1e9
    traffic = _profiled_traffic()
    hits_np = d_hits.cpu().numpy().view(np.uint32)[:, 0]
    out = {
        "metric": METRIC,
        "value": replica_throughput(ws, n, mean_ms * 1e-3),
        "unit": "rays/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": mean_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded generators; the reference publishes no dataset)",
        "config": {
            "workload": "raycast_l8: closest hit, 1024x1024 camera + 1,048,576 random rays (2,097,152) "
                        "on the level-8 displaced icosphere + ground + light (1,310,724 tris)",
            "rays_per_step": n,
            "triangles": int(st["triangle_count"]),
            "bvh8_nodes": int(st["node_count"]),
            "bvh_build_s": round(st["build_seconds"], 3),
            "scene_build_s": round(build_s, 3),
            "l2": "flushed between timed steps (512 MB write, outside the timed events)",
            "parallelism": f"replicas x{ws}",
            "hit_fraction": float((hits_np != 0xFFFFFFFF).mean()),
        },
        "e2e": {"value": replica_throughput(ws, n, e2e_s), "unit": "rays/s", "h2d_bytes_per_step": n * RAY_BYTES,
                "d2h_bytes_per_step": n * HIT_BYTES},
        "gpu_launches": args.steps * 2,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     "traffic": traffic,
                     "algorithmic_bytes_per_ray": bytes_per_ray,
                     "nodes_per_ray": nodes_v / n, "tris_per_ray": tris_t / n,
                     "kernel": "raycast_kernel<closest>"},
        "anyhit": {"rays_per_s": n / (float(np.mean(any_ms)) * 1e-3), "ms_per_step": float(np.mean(any_ms)),
                   "nodes_per_ray": any_nodes / n, "tris_per_ray": any_tris / n},
        "clocks": clk,
        "wall_timed_s": wall,
    }
    out["bvh_device_build"] = bvh_device_metrics(R, ctx, scene)
    if not args.no_render:
        out["render"] = render_metrics(R, ctx, torch, args.render_frames, scene)
    if args.instances > 0:
        out["instanced"] = instanced_metrics(R, ctx, torch, args.instances, rays)
    if not args.no_render:
        out["emissive_cdf"] = emissive_metrics(R, ctx)
    if args.batch_scenes > 0:
        pool, setup_s = build_pool(R, ctx, args.batch_scenes)
        out["batched"] = batch_metrics(R, ctx, torch, pool, setup_s, args.batch_mega_scenes)
        if args.serve_seconds > 0:
            out["served"] = serve_metrics(R, ctx, torch, pool, args.serve_seconds, args.serve_rate,
                                          all_policies=args.serve_all_policies, lanes=args.serve_lanes)
        if args.serve_budget_seconds > 0:
            out["served_budget_bound"] = served_budget_bound(R, ctx, torch, args)
    if args.rmse_spp > 0:
        out["rmse_vs_fp64_4096spp"] = rmse_metrics(R, ctx, args.rmse_spp)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(tris, rays, args.cpu_sample)
    return out


def _timed_frames(torch, fn, frames: int) -> float:
    """Mean device time (s) of `frames` calls of fn() on the current stream, after one warm-up call."""
    stream = torch.cuda.current_stream()
    fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(frames):
        fn()
    e.record(stream)
    torch.cuda.synchronize()
    return s.elapsed_time(e) * 1e-3 / frames


def render_metrics(R, ctx, torch, frames: int, scene_large) -> dict:
    """The large scene (1920x1080, 64 spp, 12 bounces, NEE+MIS, light + constant environment) rendered in
    the three forms of reina_render_device (the wave engine, the default; the pass-by-pass wavefront; the
    plain megakernel); and the Cornell room (256x256, 16 spp, 8 bounces) the same way."""
    import scenes

    out = {}
    sptr = torch.cuda.current_stream().cuda_stream
    W, H = 1920, 1080
    iv, ip = R.camera_matrices((0.0, 0.4, 3.6), (0.0, -0.12, -1.0), (0.0, 1.0, 0.0), np.radians(40.0), W / H)
    pc = R.push_consts(iv, ip, total_emissive_weight=scene_large.emissive_weight, spp=64, max_bounces=12,
                       focus_dist=3.6)
    acc = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    for name, mega, pbp in (("wavefront", False, False), ("pass_by_pass", False, True), ("megakernel", True, False)):
        opts = R.render_options(W, H, R.MODE_NEE_MIS, 1, R.ENV_CONSTANT, (0.3, 0.3, 0.35), megakernel=mega,
                                pass_by_pass=pbp)
        _, _, st = R.render(ctx, scene_large, pc, opts)   # ray counts of one frame
        dt = _timed_frames(torch, lambda: R.render_device(ctx, scene_large, pc, opts, acc.data_ptr(), 0, sptr), frames)
        out[f"large_{name}"] = {"s_per_frame": dt, "segments_per_s": st["rays"] / dt,
                                "rays_per_s": (st["rays"] + st["shadow_rays"]) / dt,
                                "segments_per_frame": st["rays"], "shadow_rays_per_frame": st["shadow_rays"]}
        if st["nodes_visited"]:
            out[f"large_{name}"]["roofline"] = segment_roofline(st, dt)
    d = scenes.cornell(R)
    sc = d.to_product(R, ctx)
    iv, ip = scenes.cornell_camera(R, 256, 256)
    pc = R.push_consts(iv, ip, total_emissive_weight=sc.emissive_weight, spp=16, max_bounces=8)
    acc = torch.zeros((256, 256, 4), dtype=torch.float32, device="cuda")
    for name, mega, pbp in (("wavefront", False, False), ("pass_by_pass", False, True), ("megakernel", True, False)):
        opts = R.render_options(256, 256, R.MODE_NEE_MIS, 1, megakernel=mega, pass_by_pass=pbp)
        _, _, st = R.render(ctx, sc, pc, opts)
        dt = _timed_frames(torch, lambda: R.render_device(ctx, sc, pc, opts, acc.data_ptr(), 0, sptr), frames)
        out[f"cornell_{name}"] = {"s_per_frame": dt, "paths_per_s": 256 * 256 * 16 / dt,
                                  "segments_per_s": st["rays"] / dt,
                                  "rays_per_s": (st["rays"] + st["shadow_rays"]) / dt}
    return out


# Algorithmic bytes of the wavefront kernels (per unit; the SoA records of render.cu / batch.cu):
#   extension, per path segment: the ray read (24 B), the queue entry read and the shade-queue entry
#     written (8 B), the hit written (12 B), plus 80 B per BVH8 node visited and 48 B per triangle tested;
#   shadow ray: its 44-byte record, plus 80 B per node and 48 B per triangle;
#   shaded hit: the path state read and written (~76 B), three vertices' index, position, TBN and TBN
#     index (3 x 60 B) and the InstanceProperties record (120 B) = 376 B; a miss-shaded segment 28 B.
SEG_BYTES, SHADOW_REC_BYTES, SHADE_BYTES, MISS_BYTES = 44, 44, 376, 28


def segment_roofline(st: dict, seconds: float) -> dict:
    """Algorithmic bytes of one frame's wavefront kernels (counted by the cooperative kernels) over the
    frame time, against the measured HBM copy peak."""
    peak, kind = _peak_hbm()
    ext = st["rays"] * SEG_BYTES + NODE_BYTES * st["nodes_visited"] + TRI_BYTES * st["triangles_tested"]
    sha = st["shadow_rays"] * SHADOW_REC_BYTES + NODE_BYTES * st["shadow_nodes_visited"] + TRI_BYTES * st["shadow_triangles_tested"]
    shade = st["shaded_hits"] * SHADE_BYTES + (st["rays"] - st["shaded_hits"]) * MISS_BYTES
    total = ext + sha + shade
    achieved = total / seconds / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "peak_source": kind, "unit": "GB/s",
            "frac": achieved / peak, "bytes_per_frame": total, "extension_bytes": ext, "shadow_bytes": sha,
            "shade_bytes": shade, "nodes_per_segment": st["nodes_visited"] / max(1, st["rays"]),
            "tris_per_segment": st["triangles_tested"] / max(1, st["rays"]),
            "nodes_per_shadow_ray": st["shadow_nodes_visited"] / max(1, st["shadow_rays"]),
            "tris_per_shadow_ray": st["shadow_triangles_tested"] / max(1, st["shadow_rays"]),
            "algorithmic_bytes_per_segment": total / max(1, st["rays"])}


def emissive_metrics(R, ctx) -> dict:
    """The emissive CDF build of a scene whose 1.3M-triangle displaced sphere is emissive, on the host and on
    the GPU (reina_scene_set_emissive_build): wall time of each (in reina_scene_build, BVH excluded) and
    whether the packed sampling data agree bit for bit."""
    import scenes

    v, i, _ = R.icosphere(8, 0.1, 1)
    fv, fi = scenes.quad((-2, -1.2, -2), (4, 0, 0), (0, 0, 4))
    out, data = {"workload": f"one emissive mesh of {i.size // 3:,} triangles + a floor"}, []
    for name, where in (("host", R.EMISSIVE_HOST), ("device", R.EMISSIVE_DEVICE)):
        s = R.Scene(ctx)
        s.add_object(v, i, material=R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5), emission=(1.0, 0.8, 0.6)))
        s.add_object(fv, fi, material=R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5)))
        s.set_emissive_build(where)
        s.build()
        out[f"{name}_s"] = s.stats()["emissive_seconds"]
        data.append(s.export_emissive())
        s.close()
    out["identical"] = all(np.array_equal(a.view(np.uint8), b.view(np.uint8)) for a, b in zip(*data))
    return out


def instanced_metrics(R, ctx, torch, n_inst: int, rays) -> dict:
    """n_inst seeded, rotated and scaled instances of one 20,480-triangle sphere in [-1, 1]^3, built flat and
    as two levels: device memory, BVH build time and closest / any-hit ray cast time of the bench's rays
    (camera + random rays, the same counts as the headline step)."""
    import scenes

    v, i, _ = R.icosphere(5, 0.1, 3)
    u = scenes.uniform(7 * n_inst, 11).reshape(n_inst, 7)
    stream = torch.cuda.current_stream()
    n = rays.shape[0]
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(n, 8).copy()).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(512 << 18, dtype=torch.float32, device="cuda")
    out = {"workload": f"{n_inst} instances of a 20,480-triangle sphere ({n_inst * 20480:,} triangles), {n:,} rays"}
    hits = {}
    for name, accel in (("flat", R.ACCEL_FLAT), ("two_level", R.ACCEL_TWO_LEVEL)):
        sc = R.Scene(ctx)
        sc.set_accel(accel)
        oid = sc.define_object(v, i)
        for k in range(n_inst):
            r = u[k]
            T = (scenes.translate(-1 + 2 * r[0], -1 + 2 * r[1], -1 + 2 * r[2]) @ scenes.rotate_axis(r[3:6] - 0.5, 360 * r[6])
                 @ scenes.scale(0.05, 0.05, 0.05))
            sc.add_instance(oid, T, R.Material())
        t0 = time.perf_counter()
        sc.build()
        build_s = time.perf_counter() - t0
        res = {"device_bytes": sc.stats()["device_bytes"], "build_s": build_s}
        for flags, key in ((R.RAY_CLOSEST, "closest_ms"), (R.RAY_ANY, "any_ms")):
            for _ in range(3):
                R.raycast_device(ctx, sc, d_rays.data_ptr(), n, d_hits.data_ptr(), flags, stream.cuda_stream)
            tot = 0.0
            for _ in range(5):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                R.raycast_device(ctx, sc, d_rays.data_ptr(), n, d_hits.data_ptr(), flags, stream.cuda_stream)
                b.record(stream)
                torch.cuda.synchronize()
                tot += a.elapsed_time(b)
            res[key] = tot / 5
            if flags == R.RAY_CLOSEST:
                hits[name] = d_hits.cpu().numpy().view(np.uint32)[:, 0].copy()
        res["closest_rays_per_s"] = n / (res["closest_ms"] * 1e-3)
        out[name] = res
        sc.close()
    out["same_ids_fraction"] = float((hits["flat"] == hits["two_level"]).mean())
    return out


def build_pool(R, ctx, n_scenes: int):
    """The seeded scenes of the batched workload: [(scene, job parameters)] and the host build time."""
    import scenes

    t0 = time.perf_counter()
    built = [scenes.batch_scene(R, ctx, k) for k in range(n_scenes)]
    return built, time.perf_counter() - t0


def batch_metrics(R, ctx, torch, built, setup_s: float, mega_scenes: int) -> dict:
    """The batched workload: n_scenes independent scenes (geodesic spheres with 1k-500k triangles, per-face
    Disney/glass materials, ground, quad light, constant environment; side U[128,1024], spp U{1..64},
    depth U{4..12}, NEE+MIS), all rendered once (a) in one reina_render_batch_device call, (b) one scene
    at a time with reina_render_device (each frame the wave engine's only job) and (c) one scene at a time
    with the pass-by-pass wavefront; all three give the same images (checked here).  The first
    mega_scenes scenes are also rendered (d) one at a time by the plain megakernel, with (a) re-timed on
    the same subset.  Device time by CUDA events around each form."""
    import scenes

    n_scenes = len(built)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    jobs, accs = [], []
    for scene, p in built:
        pc, opts = scenes.batch_job(R, scene, p)
        acc = torch.zeros((p["side"], p["side"], 4), dtype=torch.float32, device="cuda")
        accs.append(acc)
        jobs.append(R.DeviceRenderJob(scene, pc, opts, acc.data_ptr()))
    samples = [p["side"] ** 2 * p["spp"] for _, p in built]
    # autotune the batch (wave size x traversal block on a scaled-down subset of the jobs) and run the
    # timed forms with the winner; the context's tuning is put back afterwards
    saved_tuning = ctx.tuning()
    t0 = time.perf_counter()
    tune = R.autotune_batch(ctx, jobs)
    tune_s = time.perf_counter() - t0
    best = tune["best"]
    ctx.set_tuning(wave_paths=best["wave_paths"], trace_block=best["trace_block"], trace_stack=best["trace_stack"])
    # warm-up: one full wave (1024x1024 at 16 spp) of every depth, one batch each (builds the batch
    # engine at its final size and captures each depth's wave graph), and the largest single-scene
    # frame at 1 spp (grows the single-scene path state to its final size)
    warm_acc = torch.zeros((1024, 1024, 4), dtype=torch.float32, device="cuda")
    for depth in range(4, 13):
        pc, opts = scenes.batch_job(R, built[0][0], {"side": 1024, "spp": 16, "depth": depth, "seed": 1})
        R.render_batch_device(ctx, [R.DeviceRenderJob(built[0][0], pc, opts, warm_acc.data_ptr())], sptr)
    big = max(range(n_scenes), key=lambda k: built[k][1]["side"])
    pc, opts = scenes.batch_job(R, built[big][0], dict(built[big][1], spp=1, depth=4))
    R.render_device(ctx, built[big][0], pc, opts, warm_acc.data_ptr(), 0, sptr)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timed(fn):
        torch.cuda.synchronize()
        ev[0].record(stream)
        r = fn()
        ev[1].record(stream)
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) * 1e-3, r

    def plain(js, mega: bool = False, pbp: bool = False):
        for j in js:
            o = R.render_options(j.opts.width, j.opts.height, j.opts.mode, j.opts.seed, j.opts.env_mode,
                                 tuple(j.opts.env_color), megakernel=mega, pass_by_pass=pbp)
            R.render_device(ctx, j.scene, j.pc, o, j.d_accum, 0, sptr)

    t_batch, st = timed(lambda: R.render_batch_device(ctx, jobs, sptr))
    batched_imgs = [a.clone() for a in accs]
    t_plain, _ = timed(lambda: plain(jobs))
    identical = all(torch.equal(a, b) for a, b in zip(accs, batched_imgs))
    t_pbp, _ = timed(lambda: plain(jobs, pbp=True))
    identical = identical and all(torch.equal(a, b) for a, b in zip(accs, batched_imgs))
    del batched_imgs
    seg, shadow = st["rays"], st["shadow_rays"]
    n_smp = sum(samples)
    out = {
        "workload": f"{n_scenes} scenes: geodesic sphere (log-uniform 1k-500k tris) + ground + quad light, "
                    "per-face Disney/20% glass, side U[128,1024], spp U{1..64}, depth U{4..12}, NEE+MIS",
        "scenes": n_scenes,
        "triangles_total": int(sum(p["triangles"] for _, p in built)),
        "pixels_total": int(sum(p["side"] ** 2 for _, p in built)),
        "samples_total": int(n_smp),
        "scene_setup_s": round(setup_s, 2),
        "wave_paths": ctx.tuning()["wave_paths"],
        "autotune": {"s": round(tune_s, 3), "candidates": tune["candidates"], "best_ms": tune["best_ms"],
                     "default_ms": tune["default_ms"],
                     "chosen": {k: best[k] for k in ("wave_paths", "trace_block", "trace_stack")}},
        "batched": {"s": t_batch, "renders_per_s": n_scenes / t_batch, "segments_per_s": seg / t_batch,
                    "rays_per_s": (seg + shadow) / t_batch, "samples_per_s": n_smp / t_batch},
        "plain_pass_by_pass_one_at_a_time": {"s": t_pbp, "renders_per_s": n_scenes / t_pbp,
                                             "segments_per_s": seg / t_pbp, "samples_per_s": n_smp / t_pbp},
        "wave_engine_one_at_a_time": {"s": t_plain, "renders_per_s": n_scenes / t_plain,
                                      "segments_per_s": seg / t_plain, "samples_per_s": n_smp / t_plain},
        "images_identical_all_forms": bool(identical),
        "speedup_vs_plain_pass_by_pass": t_pbp / t_batch,
        "speedup_vs_wave_engine_one_at_a_time": t_plain / t_batch,
    }
    m = min(mega_scenes, n_scenes)
    if m > 0:
        sub = jobs[:m]
        t_sub, _ = timed(lambda: R.render_batch_device(ctx, sub, sptr))
        t_mega, _ = timed(lambda: plain(sub, mega=True))
        out["megakernel_subset"] = {
            "scenes": m, "samples_total": int(sum(samples[:m])),
            "batched": {"s": t_sub, "renders_per_s": m / t_sub},
            "plain_megakernel": {"s": t_mega, "renders_per_s": m / t_mega},
            "speedup_vs_plain_megakernel": t_mega / t_sub}
    ctx.set_tuning(**saved_tuning)
    return out


def serve_metrics(R, ctx, torch, pool, seconds: float, rate: float, all_policies: bool = False,
                  budget_bytes: int = 120_000_000_000, plain: bool = True, lanes: int = 0) -> dict:
    """The served workload: a seeded Poisson stream of requests (rate per second over `seconds`), each a
    scene of the pool with side/spp/depth drawn like the batched workload, submitted in real time (a)
    one request at a time to reina_render_device in arrival order (the plain form: the frame on the wave
    engine; with `all_policies` also pass by pass) and (b) to the request server (admission budget
    `budget_bytes`, continuous batching; shortest remaining work first, and with `all_policies` also
    first-come and fair share).  Latency is arrival -> image on the host; throughput is requests and rays
    over first arrival -> last completion.  The scenes are handed to the (first) server."""
    import scenes

    rng = np.random.default_rng(2026)
    arrivals, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        arrivals.append(t)
    reqs = []
    for k, at in enumerate(arrivals):
        si = int(rng.integers(0, len(pool)))
        p = dict(scenes.batch_job_params(100000 + k))
        p["seed"] = k + 1
        scene = pool[si][0]
        pc, opts = scenes.batch_job(R, scene, p)
        reqs.append((at, si, pc, opts, p["side"]))
    n = len(reqs)
    samples = sum(r[3].width * r[3].height * r[2].samplesPerPixel for r in reqs)

    def pct(lat):
        return float(np.percentile(lat, 50)), float(np.percentile(lat, 99))

    # (a) plain: one request at a time, in arrival order, images copied to the host; as the frame on
    # the wave engine (reina_render_device's default) and as the pass-by-pass wavefront
    sptr = torch.cuda.current_stream().cuda_stream
    host = {}
    for at, si, pc, opts, side in reqs:
        host.setdefault(side, np.zeros((side, side, 4), np.float32))
    dev = torch.zeros((1024, 1024, 4), dtype=torch.float32, device="cuda")

    def one_at_a_time(pass_by_pass: bool) -> dict:
        torch.cuda.synchronize()
        lat = []
        t0 = time.perf_counter()
        for at, si, pc, opts, side in reqs:
            now = time.perf_counter() - t0
            if now < at:
                time.sleep(at - now)
            o = R.render_options(opts.width, opts.height, opts.mode, opts.seed, opts.env_mode, tuple(opts.env_color),
                                 pass_by_pass=pass_by_pass)
            R.render_device(ctx, pool[si][0], pc, o, dev.data_ptr(), 0, sptr)
            torch.cuda.synchronize()
            host[side][...] = dev.view(-1)[: side * side * 4].view(side, side, 4).cpu().numpy()
            lat.append(time.perf_counter() - t0 - at)
        span = time.perf_counter() - t0 - reqs[0][0]
        p50, p99 = pct(lat)
        return {"p50_s": p50, "p99_s": p99, "mean_s": float(np.mean(lat)), "renders_per_s": n / span,
                "samples_per_s": samples / span, "span_s": span}

    plain_one = one_at_a_time(False) if plain else None
    plain_pbp = one_at_a_time(True) if (plain and all_policies) else None

    # (b) served: the same stream through a request server, once per wave-slot policy (the scenes are
    # handed to the first server and stay with it; the other policies run on servers of their own over
    # fresh copies)
    def serve(policy: str, scenes_pool) -> tuple[dict, bool]:
        srv = R.Server(ctx, budget_bytes=budget_bytes, fifo=policy == "fifo", fair=policy == "fair", wave_lanes=lanes)
        ids = [srv.add_scene(s) for s, _ in scenes_pool]
        outs = [np.zeros((r[3].height, r[3].width, 4), np.float32) for r in reqs]
        rids = [None] * n

        def submitter():
            t_start = time.perf_counter()
            for k, (at, si, pc, opts, side) in enumerate(reqs):
                now = time.perf_counter() - t_start
                if now < at:
                    time.sleep(at - now)
                rids[k] = srv.submit(ids[si], pc, opts, outs[k])

        th = threading.Thread(target=submitter)
        th.start()
        th.join()
        states = [srv.wait(r, -1.0)["state"] for r in rids]
        st = srv.stats()
        srv.close()
        span = st["first_submit_to_last_done_s"]
        return ({"policy": {"fair": "fair share", "fifo": "fifo",
                            "shortest": "shortest remaining work, aging 0.03"}[policy],
                 "p50_s": st["latency_p50_s"], "p99_s": st["latency_p99_s"], "mean_s": st["latency_mean_s"],
                 "renders_per_s": st["completed"] / span, "samples_per_s": samples / span,
                 "segments_per_s": st["rays"] / span, "rays_per_s": (st["rays"] + st["shadow_rays"]) / span,
                 "span_s": span, "completed": st["completed"], "failed": st["failed"], "waves": st["waves"],
                 "scene_uploads": st["scene_uploads"], "scene_evictions": st["scene_evictions"],
                 "peak_resident_gb": st["peak_resident_bytes"] / 1e9, "budget_gb": st["budget_bytes"] / 1e9,
                 "reserved_gb": st["reserved_bytes"] / 1e9, "wave_lanes": lanes or R.SERVER_WAVE_LANES},
                all(s == R.REQ_DONE for s in states))

    served, ok = serve("shortest", pool)   # the server's default policy (shortest first, aging 0.03)
    out = {"workload": f"Poisson {rate:g}/s for {seconds:g} s ({n} requests) over the {len(pool)}-scene pool, "
                       f"side U[128,1024], spp U{{1..64}}, depth U{{4..12}}, NEE+MIS; "
                       f"{budget_bytes / 1e9:g} GB admission budget",
           "requests": n, "samples_total": int(samples), "served": served}
    if plain_one is not None:
        out["wave_engine_one_at_a_time"] = plain_one
        out["renders_per_s_ratio_vs_wave_engine_one_at_a_time"] = served["renders_per_s"] / plain_one["renders_per_s"]
    if all_policies:
        served_fifo, ok2 = serve("fifo", [scenes.batch_scene(R, ctx, k) for k in range(len(pool))])
        served_fair, ok3 = serve("fair", [scenes.batch_scene(R, ctx, k) for k in range(len(pool))])
        ok = ok and ok2 and ok3
        out.update({"served_fifo": served_fifo, "served_fair_share": served_fair})
        if plain_pbp is not None:
            out["plain_pass_by_pass_one_at_a_time"] = plain_pbp
            out["renders_per_s_ratio_vs_plain_pass_by_pass"] = served["renders_per_s"] / plain_pbp["renders_per_s"]
    out["all_done"] = ok
    return out


def served_budget_bound(R, ctx, torch, args) -> dict:
    """The served workload under an admission budget smaller than what its scenes occupy on the device: a
    pool of `--serve-budget-scenes` fresh scenes of the batched distribution, budget = the waves' reserved
    path state + half of the pool's scene bytes, so that least-recently-used idle scenes must be evicted
    (and uploaded again on demand) while the stream runs."""
    import scenes

    pool = [scenes.batch_scene(R, ctx, k) for k in range(args.serve_budget_scenes)]
    scene_bytes = sum(int(sc.stats()["device_bytes"]) for sc, _ in pool)
    probe = R.Server(ctx, budget_bytes=120_000_000_000, wave_lanes=args.serve_lanes)
    reserved = int(probe.stats()["reserved_bytes"])
    probe.close()
    budget = reserved + scene_bytes // 2
    out = serve_metrics(R, ctx, torch, pool, args.serve_budget_seconds, args.serve_rate, budget_bytes=budget,
                        plain=False, lanes=args.serve_lanes)
    out["pool_scene_gb"] = scene_bytes / 1e9
    return out


def bvh_device_metrics(R, ctx, scene) -> dict:
    """The workload's scene built again with the device BVH builder: wall time of both builders (the host
    build is multithreaded C++ on every host core), the device build's kernel time, and whether the two
    structures are byte-identical (nodes and triangle records)."""
    import scenes

    dev, _, _ = scenes.large_scene(R, ctx, 8, bvh=R.BVH_DEVICE)
    sh, sd = scene.stats(), dev.stats()
    hn, ht = scene.export_bvh()
    dn, dt = dev.export_bvh()
    same = bool(np.array_equal(hn, dn) and np.array_equal(ht, dt))
    del dev
    return {"host_s": sh["build_seconds"], "device_s": sd["build_seconds"],
            "device_kernel_s": sd["bvh_kernel_seconds"], "speedup": sh["build_seconds"] / sd["build_seconds"],
            "identical_bytes": same, "nodes": int(sd["node_count"]), "host_threads": os.cpu_count()}


def rmse_metrics(R, ctx, spp: int) -> dict:
    """Converged-image error of the GPU against the FP64 oracle at `spp` samples per pixel (NEE+MIS) on the
    same per-pixel sample streams, per workload (tests/converged.py): the Cornell room (C0), three 32x32
    windows of the 1.3M-triangle scene at 1920x1080 (C2), one scene of the batched workload rendered
    through the batched entry point (C3).  Value per workload: the largest window RMSE / window mean."""
    import converged
    from oracle import oracle as O

    out = {}
    for key, name in (("C0_cornell_256", "cornell_256"), ("C2_large_1920x1080_windows", "large_1920x1080"),
                      ("C3_batch_scene", "batch_scene_3")):
        res = converged.converged_rmse(R, O, ctx, name, spp=spp)
        out[key] = max(res["rmse"])
        out[key + "_detail"] = res
    out["spp"] = spp
    return out


def cpu_baseline(tris, rays, sample: int) -> dict:
    from oracle import oracle as O

    sub = np.ascontiguousarray(rays[:: max(1, rays.shape[0] // sample)][:sample])
    b = O.Bvh(tris)
    threads = O.hw_threads()
    b.raycast(sub[:1024], threads=threads)
    t0 = time.perf_counter()
    b.raycast(sub, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": sub.shape[0] / dt, "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": f"{sub.shape[0]} of the {rays.shape[0]} rays (every {rays.shape[0] // sub.shape[0]}th), "
                      f"FP32 oracle BVH traversal, std::thread x{threads}, BVH build excluded",
            "seconds": dt}


def _oracle_workload():
    """The ray-cast workload (same triangles and rays as the GPU arm, bit for bit) from the oracle's own
    generators, so that the CPU arm loads no product code."""
    import scenes
    from oracle import oracle as O

    v, i = O.icosphere(8, 0.1, 1)
    _, plane, light = scenes.large_scene_geometry_planes()
    tris = np.concatenate([scenes.world_triangles(a, b) for a, b in ((v, i), plane, light)])
    lo, hi = v[:, :3].min(axis=0), v[:, :3].max(axis=0)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.5
    rays = O.raycast_rays(N_CAMERA_SIDE, N_CAMERA_SIDE, (0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 45.0, N_RANDOM, c - h, c + h,
                          seed=1)
    return tris, rays


def run_reference(args) -> dict | None:
    ws, rank, local = _dist()
    if rank != 0:
        return None
    from oracle import oracle as O

    tris, rays = _oracle_workload()
    sample = args.cpu_sample
    sub = np.ascontiguousarray(rays[:: max(1, rays.shape[0] // sample)][:sample])
    b = O.Bvh(tris)
    threads = O.hw_threads()
    for _ in range(args.warmup):
        b.raycast(sub[:4096], threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        b.raycast(sub, threads=threads)
        times.append(time.perf_counter() - t0)
    dt = float(np.mean(times))
    v = sub.shape[0] / dt
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": "rays/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded generators)",
        "config": {"workload": "raycast_l8 (same rays and scene as the GPU arm; each step a bounded sample)",
                   "rays_per_step": sub.shape[0], "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": "rays/s", "cores": threads, "kind": "port",
                         "sample": f"{sub.shape[0]} rays per step, FP32 oracle BVH traversal (oracle/), "
                                   f"std::thread x{threads}"},
        "e2e": {"value": v, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-sample", type=int, default=1 << 21)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true", help="launch the kernels a few times for ncu and exit")
    ap.add_argument("--profile-render", action="store_true", help="render a small frame twice for ncu and exit")
    ap.add_argument("--profile-batch", action="store_true", help="one small batched render for ncu and exit")
    ap.add_argument("--no-render", action="store_true", help="skip the render metrics")
    ap.add_argument("--render-frames", type=int, default=2)
    ap.add_argument("--batch-scenes", type=int, default=256,
                    help="scenes of the batched-render metrics (0 skips them)")
    ap.add_argument("--batch-mega-scenes", type=int, default=32,
                    help="leading scenes also rendered one at a time by the plain megakernel")
    ap.add_argument("--serve-seconds", type=float, default=120.0,
                    help="arrival window of the served workload (0 skips it; 120 is the full stream)")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate (requests/s)")
    ap.add_argument("--serve-all-policies", action="store_true",
                    help="also serve with first-come and fair-share wave slots, and pass by pass one at a time")
    ap.add_argument("--serve-budget-seconds", type=float, default=30.0,
                    help="seconds of the stream served under a binding memory budget (0: skip)")
    ap.add_argument("--serve-budget-scenes", type=int, default=64)
    ap.add_argument("--serve-lanes", type=int, default=0, help="server waves in flight (0: the server default)")
    ap.add_argument("--rmse-spp", type=int, default=4096, help="converged-image RMSE vs the FP64 oracle (0: skip)")
    ap.add_argument("--instances", type=int, default=256,
                    help="instances of the flat vs two-level instancing metrics (0 skips them)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
