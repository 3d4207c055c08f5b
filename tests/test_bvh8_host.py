"""The product's BVH8 on the CPU: the oracle traverses the exported nodes and triangle records (its own
restatement of the compressed 8-wide layout) and must find exactly the hits of its own independent
binary BVH, for closest and any hit, on displaced spheres and on an instanced scene; the visit counts it
reports back the ray cast's byte accounting (checked against the GPU counting build in
tests/test_raycast_gpu.py)."""
import numpy as np
import pytest

import scenes


def _cast_both(R, O, scene, tris, rays, any_hit):
    nodes, trecs = scene.export_bvh()
    h8, nv, nt = O.bvh8_raycast(nodes, trecs, rays, any_hit)
    ref = O.Bvh(tris).raycast(rays, any_hit=any_hit)
    return h8, ref, nv, nt


@pytest.mark.parametrize("level", [1, 4, 6])
def test_exported_bvh8_finds_the_oracle_hits(R, O, host_ctx, level):
    v, i, _ = R.icosphere(level, 0.1, 3)
    s = R.Scene(host_ctx)
    s.add_object(v, i)
    s.build()
    tris = scenes.world_triangles(v, i)
    rays = scenes.raycast_rays(R, level, 96, 96, 20000, v)
    for any_hit in (False, True):
        h8, ref, nv, nt = _cast_both(R, O, s, tris, rays, any_hit)
        if any_hit:   # any hit: the same rays are blocked (which triangle is found first may differ)
            assert np.array_equal(h8["prim"] == O.MISS, ref["prim"] == O.MISS)
        else:
            assert np.array_equal(h8["prim"], ref["prim"])
            hit = ref["prim"] != O.MISS
            assert np.allclose(h8["t"][hit], ref["t"][hit], rtol=1e-3, atol=1e-5)   # unrefined FP32 t
        assert nv >= rays.shape[0] and nt > 0


def test_exported_bvh8_instanced_scene(R, O, host_ctx):
    """Several instances of one model plus planes (the flattened instance layout); the oracle's BVH is
    built over the world-space triangles of the exported records, in id order."""
    d = scenes.material_zoo(R)
    s = d.to_product(R, host_ctx, accel=R.ACCEL_FLAT)
    assert s.stats()["two_level"] == 0
    _, trecs = s.export_bvh()
    rec = trecs.copy().view(np.float32).reshape(-1, 12)
    ids = trecs.copy().view(np.uint32).reshape(-1, 12)[:, 3]
    tris = np.ascontiguousarray(rec[np.argsort(ids)][:, [0, 1, 2, 4, 5, 6, 8, 9, 10]])
    rays = R.raycast_rays(64, 64, (0.0, 0.0, 3.4), (0.0, 0.0, 0.0), 40.0, 8192, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0),
                          seed=5)
    h8, ref, nv, nt = _cast_both(R, O, s, tris, rays, False)
    assert np.array_equal(h8["prim"], ref["prim"])
    assert (ref["prim"] != O.MISS).mean() > 0.5
