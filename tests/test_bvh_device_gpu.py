"""The device BVH builder (REINA_BVH_DEVICE) against the host builder: for the same triangles and options
both must write the same BVH8 node and triangle-record bytes (so every ray cast through either finds the
same hits), on the 1.3M-triangle scene, the Cornell room, random soups, duplicated triangles (no axis
can be binned: object medians on tasks of thousands of primitives), planar and tiny inputs, forced object
medians from a shallow depth (the radix-select and rank-median paths), both bin-count limits, and the
bottom levels of a two-level scene."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


def _build(R, ctx, v, i, where, bins=0, median_depth=0, accel=None):
    s = R.Scene(ctx)
    if accel is not None:
        s.set_accel(accel)
    s.set_bvh_build(where, bins, median_depth)
    s.add_object(v, i)
    s.build()
    return s


def _same(R, ctx, v, i, bins=0, median_depth=0):
    h = _build(R, ctx, v, i, R.BVH_HOST, bins, median_depth)
    d = _build(R, ctx, v, i, R.BVH_DEVICE, bins, median_depth)
    hn, ht = h.export_bvh()
    dn, dt = d.export_bvh()
    sh, sd = h.stats(), d.stats()
    assert sd["bvh_device"] == 1 and sh["bvh_device"] == 0
    assert sh["node_count"] == sd["node_count"] and sh["max_depth"] == sd["max_depth"]
    assert np.array_equal(hn, dn), "BVH8 nodes differ"
    assert np.array_equal(ht, dt), "triangle records differ"
    return sh, sd


def _soup(n, seed, spread=10.0, size=0.05):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, (n, 1, 3)).astype(np.float32)
    t = (c + rng.normal(0.0, size, (n, 3, 3))).astype(np.float32).reshape(-1, 3)
    return t, np.arange(3 * n, dtype=np.uint32)


def test_large_scene_same_bytes(R, gpu_ctx):
    vs, ids, off = [], [], 0
    for v, i in scenes.large_scene_geometry(R):
        v = np.asarray(v, np.float32)[:, :3]
        vs.append(v)
        ids.append(np.asarray(i, np.uint32).reshape(-1) + off)
        off += v.shape[0]
    sh, sd = _same(R, gpu_ctx, np.concatenate(vs), np.concatenate(ids))
    assert sd["triangle_count"] > 1_000_000
    assert sd["bvh_kernel_seconds"] > 0.0


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 9, 33, 2047, 2048, 2049, 4097, 50_000])
def test_soups_same_bytes(R, gpu_ctx, n):
    v, i = _soup(n, seed=n)
    _same(R, gpu_ctx, v, i)


def test_duplicates_take_object_medians(R, gpu_ctx):
    """Identical triangles: the centroid bounds have no extent, every split is an object median by id,
    down from a 9000-primitive task (radix select) to the small ones (rank in a warp)."""
    tri = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]], np.float32)
    v = np.tile(tri, (9000, 1))
    i = np.arange(v.shape[0], dtype=np.uint32)
    _same(R, gpu_ctx, v, i)
    # and a soup with a heavy duplicate cluster
    v2, i2 = _soup(20_000, seed=7)
    v2[: 3 * 6000] = np.tile(tri, (6000, 1))
    _same(R, gpu_ctx, v2, i2)


def test_forced_medians_and_bins(R, gpu_ctx):
    v, i = _soup(300_000, seed=11)
    _same(R, gpu_ctx, v, i, median_depth=3)    # object medians on tasks of ~37,000 primitives and below
    _same(R, gpu_ctx, v, i, median_depth=14)
    v, i = _soup(60_000, seed=12)
    _same(R, gpu_ctx, v, i, bins=4)
    _same(R, gpu_ctx, v, i, bins=64)


def test_planar_and_signed_zero(R, gpu_ctx):
    """All triangles in the plane z = 0 (one axis cannot be binned), half of them written with -0.0."""
    v, i = _soup(30_000, seed=3)
    v[:, 2] = 0.0
    v[::2, 2] = -0.0
    _same(R, gpu_ctx, v, i)


def _from_desc(R, ctx, d, where, accel=None):
    s = R.Scene(ctx)
    if accel is not None:
        s.set_accel(accel)
    s.set_bvh_build(where)
    for tex in d.textures:
        s.define_texture_rgba8(tex)
    for v4, idx, t9, ti, uv, ui in d.objects:
        s.define_object(v4, idx, tbns=t9, tbn_indices=ti, tex_coords=uv, tex_indices=ui)
    for obj, T, mats, fm in d.instances:
        if fm is None:
            s.add_instance(obj, T, mats[0])
        else:
            s.add_instance_per_face(obj, T, mats, fm)
    s.build()
    return s


def test_cornell_same_render(R, gpu_ctx):
    """Scenes built either way render the same image (the bytes of the structure are the same)."""
    d = scenes.cornell(R)
    imgs = []
    for where in (R.BVH_HOST, R.BVH_DEVICE):
        s = _from_desc(R, gpu_ctx, d, where)
        iv, ip = scenes.cornell_camera(R, 64, 64)
        pc = R.push_consts(iv, ip, total_emissive_weight=s.emissive_weight, spp=4, max_bounces=4, focus_dist=3.4)
        img, _, _ = R.render(gpu_ctx, s, pc, R.render_options(64, 64, R.MODE_NEE_MIS, 1, R.ENV_SKY, (0.0, 0.0, 0.0)))
        imgs.append(img)
        imgs.append(s.export_bvh())
    assert np.array_equal(imgs[0], imgs[2])
    assert np.array_equal(imgs[1][0], imgs[3][0]) and np.array_equal(imgs[1][1], imgs[3][1])


def test_two_level_bottom_levels_on_device(R, gpu_ctx):
    d = scenes.instanced_field(R)
    out = []
    for where in (R.BVH_HOST, R.BVH_DEVICE):
        s = _from_desc(R, gpu_ctx, d, where, accel=R.ACCEL_TWO_LEVEL)
        assert s.stats()["two_level"] == 1
        out.append(s.export_bvh())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_device_build_input_errors(R, gpu_ctx):
    v, i = _soup(100, seed=1)
    v[17, 1] = np.nan
    for where in (R.BVH_HOST, R.BVH_DEVICE):
        with pytest.raises(R.ReinaError, match="non-finite"):
            _build(R, gpu_ctx, v, i, where)
    s = R.Scene(gpu_ctx)
    with pytest.raises(R.ReinaError, match="64 SAH bins"):
        s.set_bvh_build(R.BVH_DEVICE, 128, 0)
