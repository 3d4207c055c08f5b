"""The device code against the reference's own shader source (the fixtures of tests/golden/glsl_ref.npz,
written by tests/golden/gen_glsl_golden.py from reina-vk's GLSL compiled for the host).

Single device shading functions (reina_device_kat) on the fixture's case records: the Wächter-Binder offsets
and the shader RNG bit for bit, sampled directions within 1e-5 (99 % of cases; all within 1e-3) with the
RNG state after the draws and the sampled Disney lobe exact, evalDisney within 1e-4.  Whole renders in the reference's mode
(reina_render: ray generation, the four closest-hit shaders and the sky miss shader, several samples per
pixel, depth of field, a second sample batch blended by the running mean) per pixel within 1e-4 relative,
and the bloom + tone-mapping passes (reina_postprocess)."""
import numpy as np
import pytest

import scenes
from golden import gen_glsl_golden as gen

pytestmark = pytest.mark.gpu

FIX = np.load(gen.OUT)


def close(a, b, rel, abs_=0.0):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return (np.abs(a - b) <= rel * np.abs(b) + abs_) | (np.isnan(a) & np.isnan(b))


@pytest.mark.parametrize("name,kind", [("kat_offset", 0), ("kat_offset_dielectric", 4)])
def test_device_offsets_bit_exact(R, gpu_ctx, name, kind):
    rs = gen.KATS[name][1]
    got = R.device_kat(gpu_ctx, kind, FIX[f"records_{rs}"])[:, :3]
    assert np.array_equal(got.view(np.uint32), FIX[name][:, :3].astype(np.float32).view(np.uint32))


def test_device_rng_bit_exact(R, gpu_ctx):
    """The first three draws of the shader RNG bit for bit, and the state after them (the state update of
    shaderCommon.h.glsl:41, s = s * 747796405 + 1 modulo 2^32, applied three times to the seed)."""
    got = R.device_kat(gpu_ctx, R.KAT_RANDOM, FIX["records_random"])
    assert np.array_equal(got[:, :3], FIX["kat_random"][:, :3].astype(np.float32))
    s = FIX["records_random"][:, 0].view(np.uint32).astype(np.uint64)
    for _ in range(3):
        s = (s * np.uint64(747796405) + np.uint64(1)) & np.uint64(0xFFFFFFFF)
    assert np.array_equal(got[:, 3].view(np.uint32).astype(np.uint64), s)


@pytest.mark.parametrize("name,kind", [("kat_ggx", 1), ("kat_sample_disney", 5), ("kat_diffuse_reflection", 6),
                                       ("kat_random_unit_vec", 7)])
def test_device_sampling_functions(R, gpu_ctx, name, kind):
    rs = gen.KATS[name][1]
    rec = FIX[f"records_{rs}"]
    got = R.device_kat(gpu_ctx, kind, rec)
    want = FIX[name]
    state_col = {1: 3, 5: 5, 6: 3, 7: 3}[kind]
    assert np.array_equal(got[:, 3].view(np.uint32).astype(np.float64), want[:, state_col])
    # CUDA's sinf / cosf / logf / sqrtf against the host C library's: an ulp or two, grown by the lobes'
    # normalizations on a few grazing cases
    ok = close(got[:, :3], want[:, :3], 1e-5, 1e-6).all(axis=1)
    assert ok.mean() >= 0.99 and close(got[:, :3], want[:, :3], 1e-3, 1e-4).all(), ok.mean()
    if kind == 5:
        lobe = R.device_kat(gpu_ctx, R.KAT_SAMPLE_DISNEY_LOBE, rec)
        assert np.array_equal(lobe[:, :2].astype(np.float64), want[:, 3:5])


def test_device_eval_disney(R, gpu_ctx):
    got = R.device_kat(gpu_ctx, R.KAT_EVAL_DISNEY, FIX["records_eval_disney"])
    ok = close(got, FIX["kat_eval_disney"][:, :4], 1e-4, 1e-5)
    assert ok.all(axis=1).mean() >= 0.99


@pytest.mark.parametrize("name,bar", [("render_cornell", 0.995), ("render_cornell_accum", 0.995),
                                      ("render_cornell_dof", 0.995), ("render_zoo_shallow", 0.995),
                                      ("render_zoo", 0.99), ("render_textured", 0.99)])
def test_device_renders_match_reference_shaders(R, gpu_ctx, name, bar):
    scene, W, H, spp, depth, defocus, batches = gen.RENDERS[name]
    desc = getattr(scenes, scene)(R)
    ps = desc.to_product(R, gpu_ctx, accel=R.ACCEL_FLAT)
    img = None
    for b in range(batches):
        pc = gen.push_consts(R, ps, W, H, spp, depth, defocus, b)
        img, _, _ = R.render(gpu_ctx, ps, pc, R.render_options(W, H, R.MODE_REINA, 1), accum=img)
    ok = close(img[..., :3], FIX[name][..., :3], 1e-4, 1e-6).all(-1)
    assert ok.mean() >= bar, ok.mean()


def test_device_postprocess_matches_reference_shaders(R, gpu_ctx):
    radius, threshold, intensity, exposure = gen.POST
    rgba8, bloomed = R.postprocess(gpu_ctx, FIX["post_input"], radius, threshold, intensity, exposure, want_combined=True)
    assert close(bloomed[..., :3], FIX["post_bloomed"][..., :3], 1e-5, 1e-6).all()
    d = np.abs(rgba8.astype(np.int32) - FIX["post_rgba8"].astype(np.int32))
    assert d.max() <= 1 and (d == 0).mean() >= 0.999
