"""Batched renders (reina_render_batch): each job's image and per-sample colours are exactly those of the
same job rendered alone in a batch, whatever else shares its waves, however the waves are cut, whatever
the traversal variant, and whether or not the waves are replayed from CUDA graphs — the per-path sample
streams are the same and each pixel's samples are summed in sample order (NaN samples equal NaN
samples).  Against the single-scene entry point (reina_render), whose kernels the compiler schedules
separately (so FMA contraction may differ by an ulp in places), the bar is the per-sample tolerance of
the oracle tests: |a - b| <= 1e-4 |b| + 1e-6 for at least 99.5 % of the samples."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


def job_specs():
    # (scene key, W, H, spp, bounces, mode, env_mode, env, sample_batch, seed)
    return [
        ("cornell", 64, 48, 4, 8, 1, 0, (0, 0, 0), 0, 1),
        ("cornell", 33, 17, 3, 5, 0, 0, (0, 0, 0), 0, 1),
        ("zoo", 40, 40, 2, 10, 1, 1, (0.2, 0.3, 0.4), 0, 5),
        ("zoo", 24, 31, 5, 3, 0, 0, (0, 0, 0), 2, 1),
        ("cornell", 16, 16, 1, 0, 1, 0, (0, 0, 0), 0, 1),
        ("zoo", 50, 20, 7, 12, 1, 0, (0, 0, 0), 1, 9),
        ("sphere", 37, 29, 3, 4, 1, 1, (1.0, 0.9, 0.8), 0, 2),
    ]


@pytest.fixture(scope="module")
def batch_setup(R):
    ctx = R.Context(0)
    sph = scenes.SceneDesc()
    v, i, _ = R.icosphere(4, 0.1, 7)
    sph.add_instance(sph.add_object(v, i), None, R.Material(material_idx=3, albedo=(0.6, 0.5, 0.4), roughness=0.4,
                                                            metallic=0.3, specular_tint=(1, 1, 1), sheen_tint=(1, 1, 1)))
    built = {"cornell": scenes.cornell(R).to_product(R, ctx), "zoo": scenes.material_zoo(R).to_product(R, ctx),
             "sphere": sph.to_product(R, ctx)}
    rng = np.random.default_rng(4)
    jobs, alone = [], []
    for key, W, H, spp, bounces, mode, env_mode, env, sb, seed in job_specs():
        scene = built[key]
        iv, ip = scenes.cornell_camera(R, W, H)
        pc = R.push_consts(iv, ip, sample_batch=sb, total_emissive_weight=scene.emissive_weight, spp=spp,
                           max_bounces=bounces, focus_dist=3.4, defocus=0.02 if key == "zoo" else 0.0)
        opts = R.render_options(W, H, mode, seed, env_mode, env)
        prior = rng.uniform(0, 1, (H, W, 4)).astype(np.float32) if sb else None
        jobs.append((scene, pc, opts, prior))
        one = make_jobs(R, [jobs[-1]])
        st = R.render_batch(ctx, one)
        alone.append((one[0].accum, one[0].samples, st))
    yield ctx, jobs, alone
    ctx.close()


def make_jobs(R, jobs):
    return [R.RenderJob(s, pc, o, accum=None if p is None else p.copy(), want_samples=True) for s, pc, o, p in jobs]


def agree(a, b, rtol=1e-4):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ok = (np.abs(a - b) <= rtol * np.abs(b) + 1e-6) | (np.isnan(a) & np.isnan(b))
    return ok.all(axis=-1)


def test_batch_matches_single_frame_renders(R, batch_setup):
    ctx, jobs, alone = batch_setup
    for k, ((s, pc, o, p), (acc, smp, _)) in enumerate(zip(jobs, alone)):
        ref, ref_smp, _ = R.render(ctx, s, pc, o, accum=None if p is None else p.copy(), want_samples=True)
        assert agree(smp, ref_smp).mean() >= 0.995, k
        img, ref_img = acc[..., :3].astype(np.float64), ref[..., :3].astype(np.float64)
        assert np.abs(img - ref_img).mean() <= 1e-3 * max(np.abs(ref_img).mean(), 1e-6), k


def check_same(batch, alone):
    for k, (j, (acc, smp, _)) in enumerate(zip(batch, alone)):
        assert np.array_equal(j.accum, acc, equal_nan=True), f"job {k}: image differs"
        assert np.array_equal(j.samples, smp, equal_nan=True), f"job {k}: samples differ"


@pytest.mark.parametrize("tuning", [dict(), dict(wave_paths=1000), dict(wave_paths=777, batch_flags=1),
                                    dict(wave_paths=5000, batch_flags=1), dict(wave_paths=3000, batch_flags=2),
                                    dict(wave_paths=1500, batch_flags=3), dict(wave_paths=2000, wave_lanes=1),
                                    dict(wave_paths=1200, wave_lanes=3), dict(wave_paths=900, wave_lanes=4),
                                    dict(trace_block=256, trace_stack=8),
                                    dict(trace_block=64, trace_stack=16)])
def test_batch_equals_alone(R, batch_setup, tuning):
    """All jobs in one call, with the default wave (every job's sample in one wave), with small waves
    (each wave cut across jobs and pixels), packed in list order and with an equal share per job, with
    one to four waves in flight, with graphs and with direct launches, and with other traversal
    variants."""
    ctx, jobs, alone = batch_setup
    ctx.set_tuning(**tuning)
    try:
        batch = make_jobs(R, jobs)
        st = R.render_batch(ctx, batch)
        check_same(batch, alone)
        assert st["rays"] == sum(a[2]["rays"] for a in alone)
        assert st["shadow_rays"] == sum(a[2]["shadow_rays"] for a in alone)
    finally:
        ctx.set_tuning(wave_paths=0, batch_flags=0, trace_block=128, trace_stack=12, wave_lanes=0)


def test_batch_order_and_subsets(R, batch_setup):
    """A job's result does not depend on its neighbours: reversed order, and each job alone in a batch."""
    ctx, jobs, alone = batch_setup
    ctx.set_tuning(wave_paths=2048)
    try:
        rev = make_jobs(R, jobs[::-1])
        R.render_batch(ctx, rev)
        check_same(rev[::-1], alone)
        for k in (0, 3, 5):
            one = make_jobs(R, [jobs[k]])
            R.render_batch(ctx, one)
            check_same(one, [alone[k]])
    finally:
        ctx.set_tuning(wave_paths=0)


def test_batch_device_buffers(R, batch_setup):
    import torch

    ctx, jobs, alone = batch_setup
    dev = []
    keep = []
    for s, pc, o, p in jobs:
        acc = torch.zeros((o.height, o.width, 4), dtype=torch.float32, device="cuda")
        if p is not None:
            acc.copy_(torch.from_numpy(p))
        smp = torch.zeros((o.width * o.height, pc.samplesPerPixel, 3), dtype=torch.float32, device="cuda")
        keep.append((acc, smp))
        dev.append(R.DeviceRenderJob(s, pc, o, acc.data_ptr(), smp.data_ptr()))
    torch.cuda.synchronize()
    R.render_batch_device(ctx, dev, torch.cuda.current_stream().cuda_stream)
    for (acc, smp), (a_acc, a_smp, _) in zip(keep, alone):
        assert np.array_equal(acc.cpu().numpy(), a_acc, equal_nan=True)
        assert np.array_equal(smp.cpu().numpy(), a_smp, equal_nan=True)


def test_many_jobs_over_wave_job_limit(R, batch_setup):
    """600 jobs (more than one wave's job table holds): later jobs wait for a later wave."""
    ctx, jobs, alone = batch_setup
    scene, pc0, _, _ = jobs[0]
    iv, ip = scenes.cornell_camera(R, 8, 6)
    specs = []
    for k in range(600):
        pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=1 + k % 3, max_bounces=2 + k % 5,
                           focus_dist=3.4)
        specs.append((scene, pc, R.render_options(8, 6, k % 2, 1 + k, 0, (0, 0, 0)), None))
    batch = make_jobs(R, specs)
    R.render_batch(ctx, batch)
    for k in (0, 1, 299, 511, 512, 599):
        one = make_jobs(R, [specs[k]])
        R.render_batch(ctx, one)
        assert np.array_equal(batch[k].accum, one[0].accum, equal_nan=True), k
        assert np.array_equal(batch[k].samples, one[0].samples, equal_nan=True), k


def test_batch_rejects_megakernel_flag(R, batch_setup):
    ctx, jobs, _ = batch_setup
    s, pc, o, _ = jobs[0]
    o2 = R.render_options(o.width, o.height, o.mode, o.seed, o.env_mode, tuple(o.env_color), megakernel=True)
    with pytest.raises(R.ReinaError) as e:
        R.render_batch(ctx, [R.RenderJob(s, pc, o2)])
    assert e.value.code == R.REINA_ERR_INVALID
