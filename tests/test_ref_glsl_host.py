"""The oracle against the reference's own shader source.

tests/golden/glsl_ref.npz holds outputs of reina-vk's GLSL (shaders/raytrace/*.glsl and
shaders/postprocessing/**/*.glsl, compiled for the host by oracle/glsl/build_ref.py, script
tests/golden/gen_glsl_golden.py): single shader functions on seeded case records, whole reference-mode
renders (ray generation + the four closest-hit shaders + the sky miss shader), and the bloom and
tone-mapping passes.  Where the reference checkout is reachable (REINA_REFERENCE_DIR), every fixture array
is regenerated and must be reproduced bit for bit; everywhere, the oracle must agree with the fixtures:
integer work (RNG states, Wächter-Binder offsets, sampled lobes) exactly, FP32 shading within 1e-5, and
renders sample for sample (1e-4 relative; bit for bit in the Cornell room).
"""
import numpy as np
import pytest

import scenes
from golden import gen_glsl_golden as gen

FIX = np.load(gen.OUT)


def close(a, b, rel, abs_=0.0):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return (np.abs(a - b) <= rel * np.abs(b) + abs_) | (np.isnan(a) & np.isnan(b))


@pytest.fixture(scope="module")
def G():
    from oracle.glsl import ref_glsl

    if ref_glsl.reference_dir() is None:
        pytest.skip("REINA_REFERENCE_DIR unset: the reference's shaders cannot be compiled here")
    ref_glsl.lib()
    return ref_glsl


def test_fixtures_are_what_the_reference_glsl_computes(G, R):
    """Every committed array is reproduced by the reference's shader source compiled now."""
    fresh = gen.generate()
    assert sorted(fresh) == sorted(FIX.files)
    for name in FIX.files:
        assert np.array_equal(fresh[name], FIX[name], equal_nan=True), name


@pytest.mark.parametrize("name", ["kat_offset", "kat_offset_dielectric"])
def test_oracle_offsets_bit_exact(O, name):
    kind, rs = gen.KATS[name]
    got = O.kat8(kind, FIX[f"records_{rs}"])[:, :3].astype(np.float32)
    assert np.array_equal(got.view(np.uint32), FIX[name][:, :3].astype(np.float32).view(np.uint32))


def test_oracle_rng_bit_exact(O):
    got = O.kat8(O.KAT_RANDOM, FIX["records_random"])
    want = FIX["kat_random"]
    assert np.array_equal(got[:, :7], want[:, :7])


@pytest.mark.parametrize("name", ["kat_ggx", "kat_sample_disney", "kat_diffuse_reflection", "kat_random_unit_vec"])
def test_oracle_sampling_functions(O, name):
    """Sampled directions within 1e-5 and every discrete outcome (RNG state after the draws, the Disney
    lobe and refraction flags) exact."""
    kind, rs = gen.KATS[name]
    got, want = O.kat8(kind, FIX[f"records_{rs}"]), FIX[name]
    state_col = {1: 3, 5: 5, 6: 3, 7: 3}[kind]
    assert np.array_equal(got[:, state_col], want[:, state_col])
    if kind == 5:
        assert np.array_equal(got[:, 3:5], want[:, 3:5])
    assert close(got[:, :3], want[:, :3], 1e-5, 1e-6).all()


def test_oracle_eval_disney_and_pdfs(O):
    rec = FIX["records_eval_disney"]
    got, want = O.kat8(O.KAT_EVAL_DISNEY, rec)[:, :4], FIX["kat_eval_disney"][:, :4]
    assert close(got, want, 1e-5, 1e-7).all()
    got = O.kat8(O.KAT_PDFS, FIX["records_sample_disney"])
    want = FIX["kat_pdfs"].copy()
    want[:, 2] = 0.0   # pdfGlassTransmission: never called by the reference's shaders, not restated
    assert close(got[:, :6], want[:, :6], 1e-5, 1e-7).all()


def test_oracle_reflectance(O):
    got = O.kat8(O.KAT_REFLECTANCE, FIX["records_reflectance"])[:, 0]
    assert close(got, FIX["kat_reflectance"][:, 0], 1e-5, 1e-7).all()


def _oracle_render(R, O, name):
    scene, W, H, spp, depth, defocus, batches = gen.RENDERS[name]
    desc = getattr(scenes, scene)(R)
    osc = desc.to_oracle(O)
    ctx = R.Context(-1)
    ps = desc.to_product(R, ctx, accel=R.ACCEL_FLAT)
    img = None
    for b in range(batches):
        pc = gen.push_consts(R, ps, W, H, spp, depth, defocus, b)
        img, _ = osc.render(pc, W, H, mode=R.MODE_REINA, accum=img)
    ctx.close()
    return img


@pytest.mark.parametrize("name", ["render_cornell", "render_cornell_accum", "render_cornell_dof"])
def test_oracle_cornell_renders_bit_exact(R, O, name):
    """The Cornell room (Lambertian walls, boxes, light; depth of field; a second sample batch blended by the
    running mean) renders bit for bit like the reference's shaders."""
    got = _oracle_render(R, O, name)
    assert np.array_equal(got, FIX[name], equal_nan=True)


@pytest.mark.parametrize("name,bar", [("render_zoo_shallow", 1.0), ("render_zoo", 0.995), ("render_textured", 0.995)])
def test_oracle_renders_match_reference(R, O, name, bar):
    """Metal, dielectric (Beer absorption) and every Disney lobe; textures with alpha, bump and normal maps.
    Per pixel within 1e-4 relative: all of them at 3 path vertices; at 8 a rare discrete decision taken on
    the other side of an ulp may send a path elsewhere (the bar)."""
    got = _oracle_render(R, O, name)
    ok = close(got[..., :3], FIX[name][..., :3], 1e-4, 1e-6).all(-1)
    assert ok.mean() >= bar, ok.mean()


def test_oracle_postprocess_matches_reference(O):
    radius, threshold, intensity, exposure = gen.POST
    rgba8, bloomed = O.postprocess(FIX["post_input"], radius, threshold, intensity, exposure)
    assert close(bloomed[..., :3], FIX["post_bloomed"][..., :3], 1e-5, 1e-7).all()
    d = np.abs(rgba8.astype(np.int32) - FIX["post_rgba8"].astype(np.int32))
    assert d.max() <= 1 and (d == 0).mean() >= 0.999
