"""Converged-image error against the FP64 oracle, shared by the GPU tests and bench.py.

The product renders a frame at `spp` samples per pixel; the oracle renders a few windows of the same frame in
double precision with the same per-pixel sample streams (the seeding depends only on pixel, sample and seed),
so the two images differ by float rounding and by the rare paths that a rounding sends elsewhere, not by
independent Monte Carlo noise.  The error of a window is the RMSE of its RGB values over their mean
(the reference's accumulated image, raytrace.rgen.glsl:264-284).
"""
from __future__ import annotations

import numpy as np

import scenes


def window_rmse(gpu: np.ndarray, ref: np.ndarray, win) -> float:
    x0, y0, x1, y1 = win
    g = gpu[y0:y1, x0:x1, :3].astype(np.float64)
    o = ref[y0:y1, x0:x1, :3].astype(np.float64)
    return float(np.sqrt(np.mean((g - o) ** 2)) / max(o.mean(), 1e-12))


def oracle_windows(O, desc, pc, W, H, windows, mode, env_mode=0, env=(0.0, 0.0, 0.0), seed=1, threads=0):
    """The FP64 oracle's image of the frame, rendered in the given windows only."""
    osc = desc.to_oracle(O)
    img = np.zeros((H, W, 4), np.float32)
    for win in windows:
        img, _ = osc.render(pc, W, H, mode=mode, seed=seed, env_mode=env_mode, env_color=env, window=win, precision=64,
                            threads=threads, accum=img)
    return img


# The workloads whose converged error is reported: (name, scene builder, frame, camera, spp, depth, mode,
# environment, windows).  C0: the Cornell room at 256x256; C2: the 1.3M-triangle scene at 1920x1080 (three
# 32x32 windows: the sphere's lit side, its shadowed side with the ground, a glass-heavy region); C3: one
# scene of the batched workload (a 4,000-triangle geodesic sphere with per-face Disney / glass materials)
# rendered through the batched entry point next to other jobs.
C2_WINDOWS = [(944, 520, 976, 552), (760, 640, 792, 672), (1080, 420, 1112, 452)]


def workloads(R):
    return {
        "cornell_256": dict(desc=lambda: scenes.cornell(R), W=256, H=256, camera=lambda: scenes.cornell_camera(R, 256, 256),
                            depth=8, env_mode=R.ENV_SKY, env=(0.0, 0.0, 0.0), focus=3.4,
                            windows=[(112, 112, 144, 144), (16, 200, 48, 232)]),
        "large_1920x1080": dict(desc=lambda: scenes.large_scene_desc(R), W=1920, H=1080,
                                camera=lambda: scenes.large_camera(R), depth=12, env_mode=R.ENV_CONSTANT,
                                env=scenes.LARGE_ENV, focus=3.6, windows=C2_WINDOWS),
        "batch_scene_3": dict(desc=lambda: scenes.batch_scene_desc(R, 3), W=128, H=128,
                              camera=lambda: R.camera_matrices((0.0, 0.4, 3.6), (0.0, -0.12, -1.0), (0.0, 1.0, 0.0),
                                                               np.radians(40.0), 1.0),
                              depth=8, env_mode=R.ENV_CONSTANT, env=scenes.BATCH_ENV, focus=3.6,
                              windows=[(32, 32, 64, 64), (64, 72, 96, 104)], batched=True),
    }


def converged_rmse(R, O, ctx, name: str, spp: int = 4096, threads: int = 0) -> dict:
    """Renders workload `name` at `spp` (NEE+MIS) on the GPU and its windows with the FP64 oracle; returns the
    per-window relative RMSE and the seconds each side took."""
    import time

    w = workloads(R)[name]
    desc = w["desc"]()
    W, H = w["W"], w["H"]
    iv, ip = w["camera"]()
    ps = desc.to_product(R, ctx)
    pc = R.push_consts(iv, ip, total_emissive_weight=ps.emissive_weight, spp=spp, max_bounces=w["depth"],
                       focus_dist=w["focus"])
    opts = R.render_options(W, H, R.MODE_NEE_MIS, 1, w["env_mode"], w["env"])
    t0 = time.perf_counter()
    if w.get("batched"):   # next to other jobs of the batched workload, through the batched entry point
        others = []
        for k in (0, 1):
            sc = scenes.batch_scene_desc(R, 10 + k).to_product(R, ctx)
            pck, optk = scenes.batch_job(R, sc, dict(scenes.batch_job_params(10 + k), side=96, spp=8))
            others.append(R.RenderJob(sc, pck, optk))
        job = R.RenderJob(ps, pc, opts)
        R.render_batch(ctx, [others[0], job, others[1]])
        gpu = job.accum
    else:
        gpu, _, _ = R.render(ctx, ps, pc, opts)
    t_gpu = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = oracle_windows(O, desc, pc, W, H, w["windows"], R.MODE_NEE_MIS, w["env_mode"], w["env"], threads=threads)
    t_cpu = time.perf_counter() - t0
    return {"rmse": [window_rmse(gpu, ref, win) for win in w["windows"]], "spp": spp, "gpu_s": t_gpu,
            "oracle_fp64_s": t_cpu, "windows": w["windows"], "frame": [W, H]}
