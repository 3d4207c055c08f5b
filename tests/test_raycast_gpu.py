"""GPU parity of the ray-cast kernels (closest hit / any hit) against the CPU oracle, through the C ABI.

Bar: triangle ids and hit/miss bit-exact against the FP32 oracle, and (being the same IEEE expressions)
t, u, v bit-exact too; against the FP64 oracle, t/u/v within 1e-5 relative (|a-b| <= 1e-5 * max(|b|, 1))
wherever both pick the same triangle, with FP64/FP32 id disagreements counted separately.
"""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _assert_closest_parity(hits, ref32, ref64=None, max_fp64_disagree=2e-4):
    assert np.array_equal(hits["prim"], ref32["prim"]), int((hits["prim"] != ref32["prim"]).sum())
    assert np.array_equal(hits.view(np.uint32), ref32.view(np.uint32)), "t/u/v must be bit-identical to FP32 oracle"
    if ref64 is not None:
        same = ref64["prim"] == hits["prim"]
        assert (~same).mean() <= max_fp64_disagree
        h = same & (hits["prim"] != 0xFFFFFFFF)
        for k in "tuv":
            err = np.abs(hits[k][h].astype(np.float64) - ref64[k][h]) / np.maximum(np.abs(ref64[k][h]), 1.0)
            assert err.max() <= TOL, (k, float(err.max()))


def _assert_any_parity(O, hits, ref_closest, tris, rays):
    hit = hits["prim"] != 0xFFFFFFFF
    assert np.array_equal(hit, ref_closest["prim"] != 0xFFFFFFFF)
    # The returned triangle must really be hit by the ray in [tmin, tmax], with the oracle's t/u/v.
    idx = np.flatnonzero(hit)
    rng = np.random.default_rng(0)
    for j in rng.choice(idx, size=min(2000, idx.size), replace=False):
        ok, rec = O.test_triangle(tris[hits["prim"][j]], rays[j:j + 1])
        assert ok
        assert rec["t"] == hits["t"][j] and rec["u"] == hits["u"][j] and rec["v"] == hits["v"][j]


@pytest.fixture(scope="module")
def c1(R, gpu_ctx):
    """The ray-cast workload: L6 displaced icosphere (81,920 tris), 1024x1024 camera + 1M random rays."""
    scene, v, i = scenes.sphere_scene(R, gpu_ctx, 6)
    rays = scenes.raycast_rays(R, 6, 1024, 1024, 1 << 20, v)
    tris = scenes.world_triangles(v, i)
    return scene, rays, tris


def test_c1_closest_bit_exact(R, O, gpu_ctx, c1):
    scene, rays, tris = c1
    assert rays.shape[0] == 2 * (1 << 20)
    hits = R.raycast(gpu_ctx, scene, rays, R.RAY_CLOSEST)
    b = O.Bvh(tris)
    ref32 = b.raycast(rays, precision=32)
    ref64 = b.raycast(rays, precision=64)
    assert 0.2 < (hits["prim"] != R.MISS).mean() < 0.9
    _assert_closest_parity(hits, ref32, ref64)


def test_c1_any_hit(R, O, gpu_ctx, c1):
    scene, rays, tris = c1
    hits = R.raycast(gpu_ctx, scene, rays, R.RAY_ANY)
    ref = O.Bvh(tris).raycast(rays, precision=32)
    _assert_any_parity(O, hits, ref, tris, rays)


def test_c1_brute_force_subset(R, O, gpu_ctx, c1):
    """The BVH8 loses no hit: a brute-force scan over all 81,920 triangles agrees on a ray subset."""
    scene, rays, tris = c1
    sub = np.ascontiguousarray(rays[:: 1024])
    hits = R.raycast(gpu_ctx, scene, sub)
    ref = O.raycast_brute(tris, sub)
    assert np.array_equal(hits.view(np.uint32), ref.view(np.uint32))


def test_watertight_on_gpu(R, O, gpu_ctx):
    """Rays from inside the (undisplaced) icosphere through its vertices and edge midpoints never miss."""
    v, i, _ = R.icosphere(4, 0.0, 1)
    scene = R.Scene(gpu_ctx)
    scene.add_object(v, i)
    scene.build()
    f = i.reshape(-1, 3)
    p = v[:, :3]
    targets = np.concatenate([p, (p[f[:, 0]] + p[f[:, 1]]) / 2, (p[f[:, 1]] + p[f[:, 2]]) / 2]).astype(np.float32)
    for origin in [(0.0, 0.0, 0.0), (0.05, 0.1, -0.2)]:
        rays = np.zeros(len(targets), R.RAY_DTYPE)
        rays["org"] = origin
        rays["dir"] = targets - np.asarray(origin, np.float32)
        rays["tmax"] = 1e4
        hits = R.raycast(gpu_ctx, scene, rays)
        assert (hits["prim"] != R.MISS).all()
        ref = O.raycast_brute(scenes.world_triangles(v, i), rays)
        assert np.array_equal(hits.view(np.uint32), ref.view(np.uint32))


def test_edge_cases(R, O, gpu_ctx):
    v, i, _ = R.icosphere(3, 0.1, 2)
    scene = R.Scene(gpu_ctx)
    scene.add_object(v, i)
    # a degenerate (zero-area) triangle and a far-away single triangle
    scene.add_object(np.array([[0, 0, 0, 1], [0, 0, 0, 1], [1, 1, 1, 1]], np.float32), np.array([0, 1, 2], np.uint32))
    scene.add_object(np.array([[50, 0, 0, 1], [51, 0, 0, 1], [50, 1, 0, 1]], np.float32), np.array([0, 1, 2], np.uint32))
    scene.build()
    tris = np.concatenate([scenes.world_triangles(v, i),
                           np.array([[0, 0, 0, 0, 0, 0, 1, 1, 1], [50, 0, 0, 51, 0, 0, 50, 1, 0]], np.float32)])
    rng = np.random.default_rng(7)
    n = 4096
    rays = np.zeros(n, R.RAY_DTYPE)
    rays["org"] = rng.uniform(-2, 2, (n, 3))
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d[:256, 1:] = 0.0                      # +-x axis rays
    d[256:512, [0, 2]] = 0.0               # +-y axis rays
    rays["dir"] = d
    rays["tmax"] = 1e4
    rays["tmin"][512:768] = 0.5            # ranged rays
    rays["tmax"][768:1024] = 0.3
    rays["tmax"][1024:1100] = -1.0         # empty interval: tmax < tmin -> miss
    rays["org"][1100] = (50.25, 0.25, -5.0)   # hits the far triangle head-on
    rays["dir"][1100] = (0.0, 0.0, 1.0)
    rays["dir"][1101] = (0.0, 0.0, 0.0)    # zero direction -> miss
    for flags in (R.RAY_CLOSEST, R.RAY_ANY):
        hits = R.raycast(gpu_ctx, scene, rays, flags)
        ref = O.raycast_brute(tris, rays, any_hit=bool(flags))
        assert np.array_equal(hits["prim"] != R.MISS, ref["prim"] != R.MISS)
        if flags == R.RAY_CLOSEST:
            assert np.array_equal(hits.view(np.uint32), ref.view(np.uint32))
    assert (hits["prim"][1024:1100] == R.MISS).all()
    closest = R.raycast(gpu_ctx, scene, rays)
    assert closest["prim"][1100] == tris.shape[0] - 1
    assert closest["prim"][1101] == R.MISS
    # count 0 is a no-op
    assert R.raycast(gpu_ctx, scene, rays[:0]).shape == (0,)


def test_empty_scene_all_miss(R, gpu_ctx):
    scene = R.Scene(gpu_ctx)
    scene.build()
    rays = np.zeros(100, R.RAY_DTYPE)
    rays["dir"] = (0, 0, 1)
    rays["tmax"] = 7.0
    hits = R.raycast(gpu_ctx, scene, rays)
    assert (hits["prim"] == R.MISS).all() and (hits["t"] == 7.0).all()


def test_large_scene_subset_and_counters(R, O, gpu_ctx):
    """The 1.3M-triangle scene: ids, t, u, v bit-exact against the FP32 oracle on 256k rays and within 1e-5 of
    the FP64 oracle; the counting build reports plausible visits."""
    torch = pytest.importorskip("torch")
    scene, tris, geo = scenes.large_scene(R, gpu_ctx, 8)
    st = scene.stats()
    assert st["triangle_count"] == 1310720 + 4
    rays = scenes.raycast_rays(R, 8, 512, 256, 1 << 17, geo[0][0])
    hits = R.raycast(gpu_ctx, scene, rays)
    bvh = O.Bvh(tris)
    ref = bvh.raycast(rays)
    assert np.array_equal(hits.view(np.uint32), ref.view(np.uint32))
    _assert_closest_parity(hits, ref, bvh.raycast(rays, precision=64))
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    R.raycast_device(gpu_ctx, scene, d_rays.data_ptr(), rays.shape[0], d_hits.data_ptr(), R.RAY_CLOSEST, stream)
    torch.cuda.synchronize()
    dev = d_hits.cpu().numpy().view(np.uint32).reshape(-1)
    assert np.array_equal(dev, hits.view(np.uint32).reshape(-1))
    nodes, ntris = R.raycast_counters(gpu_ctx, scene, d_rays.data_ptr(), rays.shape[0], R.RAY_CLOSEST, stream)
    per_ray_nodes = nodes / rays.shape[0]
    assert 1.0 <= per_ray_nodes < 200
    assert 0.0 < ntris / rays.shape[0] < 500
    # the counts behind the byte accounting against the CPU traversal of the same exported BVH8, which
    # tests triangles as soon as it reaches them (the GPU postpones some, so it may visit a few more nodes)
    bvh_nodes, trecs = scene.export_bvh()
    h8, cpu_nodes, cpu_tris = O.bvh8_raycast(bvh_nodes, trecs, rays)
    assert np.array_equal(h8["prim"], hits["prim"])
    print(f"node visits gpu/cpu {nodes / cpu_nodes:.4f}, triangle tests gpu/cpu {ntris / cpu_tris:.4f}")
    assert 0.98 <= nodes / cpu_nodes <= 1.10
    assert 0.98 <= ntris / cpu_tris <= 1.10


def test_raycast_page_locked_host_buffers(R, gpu_ctx):
    """Page-locked host buffers are traced in place (no staging copies); the hits equal the device path."""
    import torch

    scene, v, i = scenes.sphere_scene(R, gpu_ctx, 4)
    rays = scenes.raycast_rays(R, 4, 64, 64, 4096, v)
    n = rays.shape[0]
    h_rays = torch.from_numpy(rays.view(np.float32).reshape(n, 8).copy()).pin_memory()
    h_hits = torch.zeros((n, 4), dtype=torch.float32).pin_memory()
    for flags in (R.RAY_CLOSEST, R.RAY_ANY):
        R.raycast_into(gpu_ctx, scene, h_rays.data_ptr(), n, h_hits.data_ptr(), flags)
        ref = R.raycast(gpu_ctx, scene, rays, flags)   # pageable: copied in chunks
        assert np.array_equal(h_hits.numpy().view(np.uint32).reshape(-1), ref.view(np.uint32).reshape(-1))
    scene.close()
