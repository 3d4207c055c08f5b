"""GPU parity of the post-process (bloom + ACES tone map -> RGBA8) against the oracle, through the C ABI.
Bar: the bloomed HDR image within 1e-5 relative, RGBA8 within 1 LSB (exp/expf ulp differences can move
a value across a rounding boundary)."""
import json
from pathlib import Path

import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _check(R, O, ctx, img, radius, threshold, intensity, exposure):
    out, comb = R.postprocess(ctx, img, radius, threshold, intensity, exposure, want_combined=True)
    oout, ocomb = O.postprocess(img, radius, threshold, intensity, exposure)
    fin = np.isfinite(ocomb)
    assert np.array_equal(np.isnan(comb), np.isnan(ocomb))
    assert np.allclose(comb[fin], ocomb[fin], rtol=1e-5, atol=1e-7)
    diff = np.abs(out.astype(np.int16) - oout.astype(np.int16))
    assert diff.max() <= 1
    assert (diff == 0).mean() >= 0.999
    return out, comb


def test_bloom_golden(R, O, gpu_ctx):
    kat = json.loads((GOLDEN / "bloom_kat.json").read_text())
    img = np.asarray(kat["image"], np.float32)
    _, comb = _check(R, O, gpu_ctx, img, kat["radius"], kat["threshold"], kat["intensity"], 0.0)
    assert np.allclose(comb, np.asarray(kat["combined"], np.float32), rtol=1e-5, atol=1e-7)


def test_tonemap_golden(R, gpu_ctx):
    kat = json.loads((GOLDEN / "tonemap_kat.json").read_text())
    hdr = np.asarray(kat["hdr"], np.float32)
    img = np.concatenate([hdr, np.ones((hdr.shape[0], 1), np.float32)], 1).reshape(1, -1, 4)
    for ex, ref in kat["out"].items():
        out, _ = R.postprocess(gpu_ctx, img, 5.0, 1.0, 0.0, float(ex))
        d = np.abs(out[0, :, :3].astype(np.int16) - np.asarray(ref, np.int16))
        assert d.max() <= 1 and (d == 0).mean() >= 0.99


def test_full_hd_with_config_defaults(R, O, gpu_ctx):
    """1920x1080 HDR image with config.toml's bloom (radius 5, threshold 1, intensity 0.05, exposure 1):
    289-tap X kernel, 163-tap Y kernel, a NaN pixel spreading over its support."""
    g = np.random.default_rng(11)
    img = np.zeros((1080, 1920, 4), np.float32)
    img[..., :3] = g.exponential(0.4, (1080, 1920, 3))
    img[500:520, 900:960, :3] = 30.0
    img[100, 100, :3] = np.nan
    img[..., 3] = 1
    _check(R, O, gpu_ctx, img, 5.0, 1.0, 0.05, 1.0)


def test_rendered_image(R, O, gpu_ctx):
    d = scenes.cornell(R)
    scene = d.to_product(R, gpu_ctx)
    iv, ip = scenes.cornell_camera(R, 128, 128)
    pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=8, max_bounces=8)
    acc, _, _ = R.render(gpu_ctx, scene, pc, R.render_options(128, 128, R.MODE_NEE_MIS, 1))
    out, _ = _check(R, O, gpu_ctx, acc, 5.0, 1.0, 0.05, 1.0)
    assert out[..., :3].mean() > 5
