"""CPU checks of the oracle itself: known-answer vectors, watertightness, BVH vs brute force."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_rng_matches_golden(O):
    kat = json.loads((GOLDEN / "rng_kat.json").read_text())
    for seed, rec in kat.items():
        w, f, d = O.rng(int(seed), len(rec["words"]))
        assert w.tolist() == rec["words"], seed
        assert np.array_equal(f, np.asarray(rec["values_f32"], np.float32)), seed
        assert np.allclose(d, np.asarray(rec["words"], np.float64) / 4294967295.0, rtol=0, atol=0)


def test_rng_can_return_exactly_one(O):
    # float(word) rounds to nearest, so words >= 2^32 - 128 give exactly 1.0 (the GLSL comment says
    # "between 0 and 1 inclusive").
    w = np.uint32(0xFFFFFFF0)
    assert np.float32(w) / np.float32(4294967295.0) == np.float32(1.0)


def _icosphere_np(level):
    t = (1 + 5 ** 0.5) / 2
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7),
         (9, 8, 1)]
    verts = list(v)
    for _ in range(level):
        cache = {}

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                m = (verts[a] + verts[b]) / 2
                verts.append(m / np.linalg.norm(m))
                cache[k] = len(verts) - 1
            return cache[k]

        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return np.asarray(verts, np.float32), np.asarray(f, np.uint32)


def _rays(orig, dirs):
    from oracle.oracle import RAY_DTYPE

    r = np.zeros(len(dirs), RAY_DTYPE)
    r["org"] = orig
    r["dir"] = dirs
    r["tmin"] = 0.0
    r["tmax"] = 1e4
    return r


@pytest.mark.parametrize("precision", [32, 64])
def test_watertight_through_vertices_and_edges(O, precision):
    """Rays from inside a closed mesh aimed exactly at its vertices and edge midpoints never miss."""
    v, f = _icosphere_np(3)
    tris = v[f].reshape(-1, 9)
    edges = np.concatenate([(v[f[:, 0]] + v[f[:, 1]]) / 2, (v[f[:, 1]] + v[f[:, 2]]) / 2]).astype(np.float32)
    targets = np.concatenate([v, edges])
    for origin in [(0.0, 0.0, 0.0), (0.1, -0.05, 0.2)]:
        dirs = targets - np.asarray(origin, np.float32)
        r = _rays(origin, dirs)
        h = O.raycast_brute(tris, r, precision=precision)
        assert (h["prim"] != O.MISS).all()


def test_bvh_equals_brute_force(O):
    v, f = _icosphere_np(4)
    rng = np.random.default_rng(3)
    tris = (v[f] * (1 + 0.05 * rng.standard_normal((len(v[f]), 3, 1)))).astype(np.float32).reshape(-1, 9)
    n = 20000
    org = rng.uniform(-1.6, 1.6, (n, 3)).astype(np.float32)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d[:200, 1:] = 0.0   # axis-aligned directions exercise zero reciprocal components
    r = _rays(org, d)
    r["org"] = org
    b = O.Bvh(tris)
    for anyhit in (False, True):
        hb = b.raycast(r, any_hit=anyhit)
        hf = O.raycast_brute(tris, r, any_hit=anyhit)
        assert np.array_equal(hb["prim"] != O.MISS, hf["prim"] != O.MISS)
        if not anyhit:
            assert np.array_equal(hb.view(np.uint32), hf.view(np.uint32))


def test_fp64_agrees_with_fp32(O):
    v, f = _icosphere_np(4)
    tris = v[f].reshape(-1, 9)
    rng = np.random.default_rng(5)
    n = 20000
    org = rng.uniform(-1.5, 1.5, (n, 3)).astype(np.float32)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    r = _rays(org, d)
    r["org"] = org
    h32 = O.raycast_brute(tris, r, precision=32)
    h64 = O.raycast_brute(tris, r, precision=64)
    same = h32["prim"] == h64["prim"]
    assert same.mean() > 0.999
    hit = same & (h32["prim"] != O.MISS)
    for k in "tuv":
        err = np.abs(h32[k][hit] - h64[k][hit]) / np.maximum(np.abs(h64[k][hit]), 1.0)
        assert np.quantile(err, 0.999) < 1e-5


def test_tonemap_matches_golden(O):
    kat = json.loads((GOLDEN / "tonemap_kat.json").read_text())
    hdr = np.asarray(kat["hdr"], np.float32)
    img = np.concatenate([hdr, np.ones((hdr.shape[0], 1), np.float32)], 1).reshape(1, -1, 4)
    for ex, ref in kat["out"].items():
        # intensity 0 isolates the tone map from the bloom
        out, comb = O.postprocess(img, radius=5.0, threshold=1.0, intensity=0.0, exposure=float(ex))
        assert np.array_equal(out[0, :, :3], np.asarray(ref, np.uint8)), ex
        assert (out[0, :, 3] == 255).all()


def test_bloom_matches_golden(O):
    kat = json.loads((GOLDEN / "bloom_kat.json").read_text())
    img = np.asarray(kat["image"], np.float32)
    ref = np.asarray(kat["combined"], np.float32)
    for precision in (32, 64):
        _, comb = O.postprocess(img, kat["radius"], kat["threshold"], kat["intensity"], 0.0, precision=precision)
        assert np.allclose(comb, ref, rtol=2e-6, atol=1e-7)


def test_bloom_spreads_nan_like_the_reference(O):
    """A NaN pixel reaches every output within the kernel support (its weight is multiplied, not tested)."""
    img = np.zeros((8, 40, 4), np.float32)
    img[4, 20, :3] = np.nan
    _, comb = O.postprocess(img, radius=5.0, threshold=1.0, intensity=0.05, exposure=0.0)
    K = int(40 * 5.0 / 100 * 3 + 0.5)
    assert np.isnan(comb[4, 20 - K:20 + K + 1, 0]).all()
    assert not np.isnan(comb[4, 20 + K + 1:, 0]).any()


@pytest.mark.parametrize("level,amp,seed", [(0, 0.0, 1), (3, 0.1, 1), (6, 0.1, 1), (5, 0.25, 9)])
def test_oracle_icosphere_equals_product(R, O, level, amp, seed):
    """The oracle's own generator of the ray-cast workload (used by the timed CPU arm, which loads no
    product code) writes the product generator's bits."""
    v, i, _ = R.icosphere(level, amp, seed)
    ov, oi = O.icosphere(level, amp, seed)
    assert np.array_equal(v.view(np.uint32), ov.view(np.uint32))
    assert np.array_equal(np.asarray(i).reshape(-1), oi)


def test_oracle_rays_equal_product(R, O):
    v, _ = O.icosphere(4, 0.1, 1)
    lo, hi = v[:, :3].min(axis=0), v[:, :3].max(axis=0)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.5
    a = R.raycast_rays(96, 64, (0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 45.0, 20000, c - h, c + h, seed=1)
    b = O.raycast_rays(96, 64, (0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 45.0, 20000, c - h, c + h, seed=1)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
