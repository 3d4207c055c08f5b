"""GPU parity of the wavefront path tracer against the CPU oracle (same per-pixel PCG sample streams),
through the C ABI.

Bar (per the spec of the path): per-sample radiance within 1e-4 relative — checked as the fraction of
samples with |gpu - ref| <= 1e-4 |ref| + 1e-6 on every channel, NaN matching NaN — and the converged
image within 1% RMSE of a 4096-spp FP64 oracle.  Discrete decisions (Fresnel, lobe pick, rejection
loops) and triangle edges can flip between implementations for a few samples, which then follow
different paths; the fractions below bound how many.
"""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def agree(a, b, rtol=RTOL):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ok = (np.abs(a - b) <= rtol * np.abs(b) + 1e-6) | (np.isnan(a) & np.isnan(b))
    return ok.all(axis=-1)


def render_both(R, O, ctx, desc, W, H, spp, bounces, mode, env_mode=0, env=(0, 0, 0), precision=32,
                sample_batch=0, camera=None, window=None, accum=None, defocus=0.0):
    scene = desc.to_product(R, ctx)
    osc = desc.to_oracle(O)
    assert scene.emissive_weight == pytest.approx(osc.emissive_weight, rel=1e-7)
    iv, ip = camera if camera is not None else scenes.cornell_camera(R, W, H)
    pc = R.push_consts(iv, ip, sample_batch=sample_batch, total_emissive_weight=scene.emissive_weight, spp=spp,
                       max_bounces=bounces, focus_dist=3.4, defocus=defocus)
    acc_in = np.zeros((H, W, 4), np.float32) if accum is None else accum
    g_acc, g_smp, st = R.render(ctx, scene, pc, R.render_options(W, H, mode, 1, env_mode, env), accum=acc_in.copy(),
                                want_samples=True)
    o_acc, o_smp = osc.render(pc, W, H, mode=mode, env_mode=env_mode, env_color=env, precision=precision,
                              window=window, accum=acc_in.copy(), want_samples=True)
    return g_acc, g_smp, o_acc, o_smp, st


@pytest.mark.parametrize("mode", [0, 1])
def test_cornell_per_sample_parity(R, O, gpu_ctx, mode):
    """The Cornell room at 256x256, 16 spp, 8 bounces (reina mode and NEE+MIS)."""
    d = scenes.cornell(R)
    g_acc, g_smp, o_acc, o_smp, st = render_both(R, O, gpu_ctx, d, 256, 256, 16, 8, mode)
    assert st["rays"] > 256 * 256 * 16
    if mode == 1:
        assert st["shadow_rays"] > 0
    frac = agree(g_smp, o_smp).mean()
    assert frac >= 0.995, frac
    img_g, img_o = g_acc[..., :3], o_acc[..., :3]
    assert np.isfinite(img_g).all()
    rel = np.abs(img_g - img_o).mean() / img_o.mean()
    assert rel < 2e-3, rel


@pytest.mark.parametrize("mode", [0, 1])
def test_cornell_fp64_per_sample(R, O, gpu_ctx, mode):
    d = scenes.cornell(R)
    g_acc, g_smp, o_acc, o_smp, _ = render_both(R, O, gpu_ctx, d, 64, 64, 8, 8, mode, precision=64)
    frac = agree(g_smp, o_smp).mean()
    assert frac >= 0.98, frac


@pytest.mark.parametrize("mode", [0, 1])
def test_material_zoo_per_sample_parity(R, O, gpu_ctx, mode):
    """Every material (metal, dielectric with Beer absorption, Disney lobes incl. glass, culled faces,
    instance transforms, interpolated normals) against the FP32 oracle."""
    d = scenes.material_zoo(R)
    g_acc, g_smp, o_acc, o_smp, _ = render_both(R, O, gpu_ctx, d, 128, 128, 8, 10, mode)
    frac = agree(g_smp, o_smp).mean()
    assert frac >= 0.99, frac
    nan_g, nan_o = np.isnan(g_smp).any(-1), np.isnan(o_smp).any(-1)
    assert abs(nan_g.mean() - nan_o.mean()) < 1e-3


def test_depth_of_field_and_sky(R, O, gpu_ctx):
    """Hexagonal-aperture depth of field (its draws do not advance the stream) and the sky miss shader."""
    d = scenes.material_zoo(R)
    iv, ip = R.camera_matrices((0.0, 0.3, 5.0), (0.0, -0.05, -1.0), (0.0, 1.0, 0.0), np.radians(35.0), 1.5)
    g_acc, g_smp, o_acc, o_smp, _ = render_both(R, O, gpu_ctx, d, 96, 64, 4, 6, 0, camera=(iv, ip), defocus=0.03)
    assert agree(g_smp, o_smp).mean() >= 0.99


def test_accumulation_across_frames(R, O, gpu_ctx):
    """Frame 2 (sampleBatch = 2) blends into the previous image as (prev*2 + mean)/3."""
    d = scenes.cornell(R)
    W = H = 48
    prev = np.random.default_rng(0).uniform(0, 1, (H, W, 4)).astype(np.float32)
    g_acc, g_smp, o_acc, o_smp, _ = render_both(R, O, gpu_ctx, d, W, H, 4, 6, 0, sample_batch=2, accum=prev)
    assert agree(g_smp, o_smp).mean() >= 0.99
    ok = np.abs(g_acc - o_acc) <= 1e-4 * np.abs(o_acc) + 1e-5
    assert ok.mean() >= 0.98


def test_converged_rmse_vs_fp64_4096spp(R, O, gpu_ctx):
    """Converged image: GPU at 4096 spp against the FP64 oracle at 4096 spp (Cornell, NEE+MIS, 32x32)."""
    d = scenes.cornell(R)
    W = H = 32
    g_acc, _, o_acc, _, _ = render_both(R, O, gpu_ctx, d, W, H, 4096, 8, 1, precision=64)
    g, o = g_acc[..., :3].astype(np.float64), o_acc[..., :3].astype(np.float64)
    rmse = np.sqrt(np.mean((g - o) ** 2)) / o.mean()
    assert rmse <= 0.01, rmse


def test_large_scene_crop_parity(R, O, gpu_ctx):
    """The 1.3M-triangle scene (per-face Disney + 20% glass, constant environment) at 1920x1080: samples
    of a 48x32 crop against the FP32 oracle."""
    import scenes as S

    geo = S.large_scene_geometry(R, 8, 1)
    (sv, si), (pv, pi), (lv, li) = geo
    mats, face = S.large_scene_materials(R, si.size // 3, 1)
    d = S.SceneDesc()
    d.add_instance(d.add_object(sv, si, S.large_scene_tbn(R, 8, 1), si), None, materials=mats, face_material=face)
    d.add_instance(d.add_object(pv, pi), None, R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5)))
    d.add_instance(d.add_object(lv, li), None,
                   R.Material(material_idx=0, albedo=(0.9, 0.9, 0.9), emission=(17.0, 12.0, 4.0), cull_backface=True))
    W, H = 1920, 1080
    iv, ip = R.camera_matrices((0.0, 0.4, 3.6), (0.0, -0.12, -1.0), (0.0, 1.0, 0.0), np.radians(40.0), W / H)
    win = (940, 500, 988, 532)
    g_acc, g_smp, o_acc, o_smp, st = render_both(R, O, gpu_ctx, d, W, H, 2, 12, 1, env_mode=1, env=(0.3, 0.3, 0.35),
                                                 camera=(iv, ip), window=win)
    ys, xs = np.mgrid[win[1]:win[3], win[0]:win[2]]
    pix = (ys * W + xs).reshape(-1)
    frac = agree(g_smp[pix], o_smp[pix]).mean()
    assert frac >= 0.98, frac


@pytest.mark.parametrize("mode", [0, 1])
def test_megakernel_matches_wavefront(R, O, gpu_ctx, mode):
    """The plain single-kernel form and the wavefront form compute the same samples."""
    d = scenes.material_zoo(R)
    scene = d.to_product(R, gpu_ctx)
    W = H = 96
    iv, ip = scenes.cornell_camera(R, W, H)
    pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=4, max_bounces=8, focus_dist=3.4)
    a_w, s_w, st_w = R.render(gpu_ctx, scene, pc, R.render_options(W, H, mode, 1), want_samples=True)
    a_m, s_m, st_m = R.render(gpu_ctx, scene, pc, R.render_options(W, H, mode, 1, megakernel=True), want_samples=True)
    assert agree(s_m, s_w).mean() >= 0.995
    assert abs(int(st_w["rays"]) - int(st_m["rays"])) <= 0.01 * st_w["rays"]
    osc = d.to_oracle(O)
    _, o_smp = osc.render(pc, W, H, mode=mode, want_samples=True)
    assert agree(s_m, o_smp).mean() >= 0.99


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("sample_batch", [0, 2])
def test_pass_by_pass_equals_wave_engine(R, gpu_ctx, mode, sample_batch):
    """The default form (the frame as the wave engine's one job) and the pass-by-pass wavefront give the
    same samples, image and ray counts, bit for bit, also when blending into a previous image."""
    d = scenes.material_zoo(R)
    scene = d.to_product(R, gpu_ctx)
    W, H = 80, 56
    iv, ip = scenes.cornell_camera(R, W, H)
    pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=5, max_bounces=9, focus_dist=3.4)
    pc.sampleBatch = sample_batch
    prev = np.random.default_rng(3).random((H, W, 4), dtype=np.float32)
    out = []
    for pbp in (False, True):
        acc, smp, st = R.render(gpu_ctx, scene, pc, R.render_options(W, H, mode, 7, pass_by_pass=pbp),
                                want_samples=True, accum=prev.copy())
        out.append((acc, smp, st))
    assert np.array_equal(out[0][0], out[1][0], equal_nan=True)
    assert np.array_equal(out[0][1], out[1][1], equal_nan=True)
    assert out[0][2]["rays"] == out[1][2]["rays"] and out[0][2]["shadow_rays"] == out[1][2]["shadow_rays"]


@pytest.mark.parametrize("mode", [0, 1])
def test_render_stats_count_traversal_work(R, gpu_ctx, mode):
    """A frame whose call returns statistics runs the counting kernels of its traversal form: the traversal
    work (nodes, triangles of segments and shadow rays, shaded hits) is reported, the counts repeat from
    call to call, and the image equals the one of the device entry point, which does not count."""
    torch = pytest.importorskip("torch")
    d = scenes.material_zoo(R)
    scene = d.to_product(R, gpu_ctx)
    W, H = 96, 64
    iv, ip = scenes.cornell_camera(R, W, H)
    pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=3, max_bounces=6, focus_dist=3.4)
    opts = R.render_options(W, H, mode, 5)
    acc1, _, st1 = R.render(gpu_ctx, scene, pc, opts)
    acc2, _, st2 = R.render(gpu_ctx, scene, pc, opts)
    keys = ("rays", "shadow_rays", "nodes_visited", "triangles_tested", "shadow_nodes_visited",
            "shadow_triangles_tested", "shaded_hits")
    assert all(st1[k] == st2[k] for k in keys), (st1, st2)
    assert st1["nodes_visited"] >= st1["rays"] > 0
    assert st1["triangles_tested"] > 0
    assert 0 < st1["shaded_hits"] <= st1["rays"]
    if mode == 1:
        assert st1["shadow_nodes_visited"] >= st1["shadow_rays"] > 0
    else:
        assert st1["shadow_rays"] == 0 and st1["shadow_nodes_visited"] == 0
    d_acc = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    R.render_device(gpu_ctx, scene, pc, opts, d_acc.data_ptr(), 0, stream)
    torch.cuda.synchronize()
    assert np.array_equal(acc1, acc2, equal_nan=True)
    assert np.array_equal(d_acc.cpu().numpy(), acc1, equal_nan=True)
