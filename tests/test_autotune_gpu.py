"""The autotuner on the GPU: every traversal variant it chooses between (grid form in three block sizes
x three stack depths x coherence / input ray order, the cooperative form at six refill thresholds) gives
bit-identical hits (any hit: the same hit/miss and a triangle the ray hits); autotuned ray casts, renders and batched
renders pick a valid configuration, cache it, and with the cache in use give exactly the results of the
default configuration."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu

GRID = 255   # REINA_REFILL_GRID: one thread per ray
VARIANTS = [dict(refill=GRID, trace_block=b, trace_stack=s, trace_order=o) for b in (64, 128, 256) for s in (8, 12, 16)
            for o in (0, 1)] + \
           [dict(refill=r, trace_block=128, trace_stack=12) for r in (1, 4, 8, 16, 24, 32)]


@pytest.fixture(scope="module")
def rc_setup(R):
    import torch

    ctx = R.Context(0)
    scene, v, i = scenes.sphere_scene(R, ctx, 5)
    rays = scenes.raycast_rays(R, 5, 256, 256, 65536, v)
    n = rays.shape[0]
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(n, 8).copy()).cuda()
    yield ctx, scene, d_rays, n
    scene.close()
    ctx.close()


@pytest.mark.parametrize("flags", [0, 1])
def test_all_variants_give_identical_hits(R, rc_setup, flags):
    import torch

    ctx, scene, d_rays, n = rc_setup
    ref = None
    for v in VARIANTS:
        ctx.set_tuning(**v)
        d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        R.raycast_device(ctx, scene, d_rays.data_ptr(), n, d_hits.data_ptr(), flags, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        h = d_hits.cpu().numpy().view(np.uint32)
        if flags == 1:   # any hit: which occluder a form reports first may differ; hit or miss may not
            h = h[:, 0] == R.MISS
        if ref is None:
            ref = h
        else:
            assert np.array_equal(h, ref), v
    ctx.set_tuning(refill=0, trace_block=128, trace_stack=12, trace_order=0)   # the defaults


def test_autotune_raycast_caches_and_applies(R, rc_setup):
    import torch

    ctx, scene, d_rays, n = rc_setup
    sp = torch.cuda.current_stream().cuda_stream
    d_ref = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    R.raycast_device(ctx, scene, d_rays.data_ptr(), n, d_ref.data_ptr(), 0, sp)
    d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    res = R.autotune_raycast(ctx, scene, d_rays.data_ptr(), n, d_hits.data_ptr(), 0, sp)
    torch.cuda.synchronize()
    assert res["candidates"] == 13 and 0 < res["best_ms"] <= res["default_ms"]
    best = res["best"]
    assert best["trace_block"] in (64, 128, 256) and best["trace_stack"] in (8, 12, 16)
    assert R.autotune_lookup(ctx, R.TUNE_RAYCAST_CLOSEST, scene.stats()["triangle_count"], n) == best
    assert np.array_equal(d_hits.cpu().numpy().view(np.uint32), d_ref.cpu().numpy().view(np.uint32))
    R.autotune_set_mode(ctx, R.AUTOTUNE_CACHED)
    try:
        d2 = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        R.raycast_device(ctx, scene, d_rays.data_ptr(), n, d2.data_ptr(), 0, sp)
        torch.cuda.synchronize()
        assert np.array_equal(d2.cpu().numpy().view(np.uint32), d_ref.cpu().numpy().view(np.uint32))
    finally:
        R.autotune_set_mode(ctx, R.AUTOTUNE_OFF)


def test_autotune_render_and_batch(R):
    ctx = R.Context(0)
    try:
        d = scenes.material_zoo(R)
        sc = d.to_product(R, ctx)
        W, H = 96, 64
        iv, ip = scenes.cornell_camera(R, W, H)
        pc = R.push_consts(iv, ip, total_emissive_weight=sc.emissive_weight, spp=3, max_bounces=6, focus_dist=3.4)
        opts = R.render_options(W, H, R.MODE_NEE_MIS, 3)
        ref, _, _ = R.render(ctx, sc, pc, opts)
        res = R.autotune_render(ctx, sc, pc, opts)
        assert res["candidates"] == 12 and res["best_ms"] > 0 and res["kind"] == R.TUNE_RENDER
        jobs = [R.RenderJob(sc, pc, opts)]
        for k in range(5):
            iv2, ip2 = scenes.cornell_camera(R, 40 + 8 * k, 32)
            pc2 = R.push_consts(iv2, ip2, total_emissive_weight=sc.emissive_weight, spp=1 + k, max_bounces=4 + k,
                                focus_dist=3.4)
            jobs.append(R.RenderJob(sc, pc2, R.render_options(40 + 8 * k, 32, R.MODE_NEE_MIS, k + 1)))
        bres = R.autotune_batch(ctx, jobs)
        # a batch of ~50k paths: every candidate wave shrinks to 2^16 slots, leaving the two traversal forms
        assert bres["candidates"] == 2 and bres["best"]["wave_paths"] == 1 << 16
        R.autotune_set_mode(ctx, R.AUTOTUNE_CACHED)
        out, _, _ = R.render(ctx, sc, pc, opts)
        assert np.array_equal(out, ref)
        alone = []
        R.autotune_set_mode(ctx, R.AUTOTUNE_OFF)
        for j in jobs:   # each job alone in a batch, default configuration
            one = R.RenderJob(j.scene, j.pc, j.opts)
            R.render_batch(ctx, [one])
            alone.append(one.accum)
        R.autotune_set_mode(ctx, R.AUTOTUNE_CACHED)
        R.render_batch(ctx, jobs)
        for j, a in zip(jobs, alone):
            assert np.array_equal(j.accum, a)
        sc.close()
    finally:
        ctx.close()


def test_wave_refill_forms_give_identical_images(R):
    """The wavefront extension and shadow kernels in the grid form (the default) and the cooperative form
    (wave_refill 4, 8, 16): the same frame, bit for bit, through the wave engine and pass by pass."""
    ctx = R.Context(0)
    try:
        d = scenes.material_zoo(R)
        sc = d.to_product(R, ctx)
        W, H = 80, 56
        iv, ip = scenes.cornell_camera(R, W, H)
        pc = R.push_consts(iv, ip, total_emissive_weight=sc.emissive_weight, spp=4, max_bounces=6, focus_dist=3.4)
        assert ctx.tuning()["wave_refill"] == R.REFILL_GRID and ctx.tuning()["refill"] == 8
        ref = None
        for wr in (0, 4, 8, 16):
            ctx.set_tuning(wave_refill=wr)
            for pbp in (False, True):
                out, _, st = R.render(ctx, sc, pc, R.render_options(W, H, R.MODE_NEE_MIS, 5, pass_by_pass=pbp))
                if ref is None:
                    ref = out
                assert np.array_equal(out, ref), (wr, pbp)
        ctx.set_tuning(wave_refill=0)
        sc.close()
    finally:
        ctx.close()
