"""CPU checks of the oracle's renderer: analytic furnace test, determinism, seeding and scene data."""
import numpy as np
import pytest

import scenes


def _furnace_scene(R, level=3):
    d = scenes.SceneDesc()
    v, i, _ = R.icosphere(level, 0.0, 1)
    d.add_instance(d.add_object(v, i), None, R.Material(material_idx=0, albedo=(1.0, 1.0, 1.0)))
    return d


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("mode", [0, 1])
def test_white_furnace(R, O, precision, mode):
    """An albedo-1 Lambertian convex object under a constant environment L: every sample returns L."""
    d = _furnace_scene(R)
    osc = d.to_oracle(O)
    iv, ip = R.camera_matrices((0.0, 0.0, 3.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0), np.radians(45.0), 1.0)
    pc = R.push_consts(iv, ip, spp=4, max_bounces=4, direct_clamp=100.0)
    L = (0.5, 0.25, 2.0)
    acc, smp = osc.render(pc, 32, 32, mode=mode, env_mode=1, env_color=L, precision=precision, want_samples=True)
    tol = 2e-6 if precision == 32 else 1e-12
    assert np.allclose(smp, np.asarray(L, np.float32), rtol=tol, atol=0)
    assert np.allclose(acc[..., :3], np.asarray(L, np.float32), rtol=tol, atol=0)


def test_render_is_deterministic_and_threads_agree(R, O):
    d = scenes.cornell(R)
    osc = d.to_oracle(O)
    iv, ip = scenes.cornell_camera(R, 24, 24)
    pc = R.push_consts(iv, ip, total_emissive_weight=osc.emissive_weight, spp=2, max_bounces=4)
    a1, s1 = osc.render(pc, 24, 24, mode=1, threads=1, want_samples=True)
    a2, s2 = osc.render(pc, 24, 24, mode=1, threads=4, want_samples=True)
    assert np.array_equal(s1, s2) and np.array_equal(a1, a2)
    assert np.isfinite(a1).all() and a1[..., :3].mean() > 0.01


def test_emissive_weight_agrees_with_scene_assembly(R, O, host_ctx):
    d = scenes.cornell(R)
    osc = d.to_oracle(O)
    ps = d.to_product(R, host_ctx, require_emissive=True)
    assert ps.emissive_weight == pytest.approx(osc.emissive_weight, rel=1e-7)
    area = 0.5 * 0.4
    lum = 0.2126 * 17 + 0.7152 * 12 + 0.0722 * 4
    assert osc.emissive_weight == pytest.approx(area * lum, rel=1e-5)


def test_seed_hash_is_the_documented_function(O):
    def h(pixel, sample, seed):
        M = 0xFFFFFFFF
        x = ((seed * 0x9E3779B1) & M) ^ ((pixel * 0x85EBCA77 + 0x165667B1) & M) ^ ((sample * 0xC2B2AE3D + 0x27D4EB2F) & M)
        x ^= x >> 16
        x = (x * 0x7FEB352D) & M
        x ^= x >> 15
        x = (x * 0x846CA68B) & M
        x ^= x >> 16
        return x
    for args in [(0, 0, 1), (12345, 7, 1), (65535, 4095, 99), (2 ** 32 - 1, 2 ** 32 - 1, 2 ** 32 - 1)]:
        assert O.seed_hash(*args) == h(*args)


def test_running_mean_across_frames(R, O):
    """Frame k (sampleBatch = k) blends as (prev*k + mean)/(k + 1) (raytrace.rgen.glsl:279-284)."""
    d = scenes.cornell(R)
    osc = d.to_oracle(O)
    iv, ip = scenes.cornell_camera(R, 16, 16)
    pc0 = R.push_consts(iv, ip, total_emissive_weight=osc.emissive_weight, spp=2, max_bounces=3, sample_batch=0)
    a0, _ = osc.render(pc0, 16, 16, mode=0)
    pc1 = R.push_consts(iv, ip, total_emissive_weight=osc.emissive_weight, spp=2, max_bounces=3, sample_batch=1)
    a1, _ = osc.render(pc1, 16, 16, mode=0, accum=a0.copy())
    fresh, _ = osc.render(pc1, 16, 16, mode=0, accum=np.zeros_like(a0))
    # with a zero previous image the blend halves the frame mean
    assert np.allclose(fresh[..., :3] * 2.0, (a1[..., :3] * 2.0 - a0[..., :3]), rtol=1e-5, atol=1e-6)
