"""Two-level scenes on the host: the automatic choice, the exported structure (top level over instance
boxes, one bottom level per model in object space, per-instance world-to-object records) traversed by the
oracle's CPU restatement, against the oracle's own instanced ray cast (per instance: the world ray through
the same float matrix, the oracle's BVH over the model); hit ids are global in both."""
import numpy as np
import pytest

import scenes


def build(R, ctx, d, accel=None):
    return d.to_product(R, ctx, accel=accel)


def oracle_instanced(O, d, scene):
    rec, _ = scene.export_two_level()
    inst = O.InstancedScene()
    for m in scenes.instance_models(d):
        inst.add_model(m)
    for k, (obj, T, _, _) in enumerate(d.instances):
        inst.add_instance(obj, rec[k, :12].view(np.float32), int(rec[k, 13]))
    return inst, rec


def field_rays(R, n=20000, seed=3):
    return R.raycast_rays(64, 64, (0.0, 0.0, 3.4), (0.0, 0.0, 0.0), 40.0, n, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0),
                          seed=seed)


def test_auto_choice_and_records(R, host_ctx):
    d = scenes.instanced_field(R)
    s = build(R, host_ctx, d)
    st = s.stats()
    assert st["two_level"] == 1 and st["blas_count"] == len(d.objects)
    rec, refs = s.export_two_level()
    assert rec.shape == (len(d.instances), 16)
    assert np.array_equal(np.sort(refs), np.arange(len(d.instances)))
    first = 0
    for k, (obj, T, _, _) in enumerate(d.instances):
        assert rec[k, 13] == first
        first += d.objects[obj][1].size // 3
        inv = rec[k, :12].view(np.float32).reshape(3, 4).astype(np.float64)
        ref = np.linalg.inv(np.asarray(T, np.float64))[:3]
        assert np.allclose(inv, ref, rtol=1e-6, atol=1e-6)
    flat = build(R, host_ctx, scenes.cornell(R))   # no repeated model worth two levels
    assert flat.stats()["two_level"] == 0
    assert flat.export_two_level()[0].shape[0] == 0


def test_exported_two_level_finds_the_oracle_hits(R, O, host_ctx):
    d = scenes.instanced_field(R)
    s = build(R, host_ctx, d)
    nodes, tris = s.export_bvh()
    inst, rec = oracle_instanced(O, d, s)
    _, refs = s.export_two_level()
    rays = field_rays(R)
    for any_hit in (False, True):
        h2, nv, nt = O.bvh8_two_level_raycast(nodes, tris, refs, rec, rays, any_hit)
        ref = inst.raycast(rays, any_hit)
        if any_hit:
            assert np.array_equal(h2["prim"] == O.MISS, ref["prim"] == O.MISS)
        else:
            assert np.array_equal(h2["prim"], ref["prim"])
        assert (ref["prim"] != O.MISS).mean() > 0.5 and nv > 0 and nt > 0


def test_two_level_agrees_with_flat(R, O, host_ctx):
    """The same scene flattened: the world-space test rounds differently, so ids may differ only where two
    surfaces are hit at the same distance to rounding (the room's boxes stand on the floor: their bottom
    faces are coplanar with it) or a ray grazes a shared edge."""
    d = scenes.instanced_field(R)
    s2 = build(R, host_ctx, d)
    s1 = build(R, host_ctx, d, accel=R.ACCEL_FLAT)
    assert s1.stats()["two_level"] == 0 and s2.stats()["triangle_count"] == s1.stats()["triangle_count"]
    rays = field_rays(R)
    n1, t1 = s1.export_bvh()
    h1, _, _ = O.bvh8_raycast(n1, t1, rays)
    inst, _ = oracle_instanced(O, d, s2)
    h2 = inst.raycast(rays)
    diff = h1["prim"] != h2["prim"]
    assert diff.mean() < 0.01
    t1, t2 = h1["t"][diff].astype(np.float64), h2["t"][diff].astype(np.float64)
    assert np.all(np.abs(t1 - t2) <= 1e-5 * np.maximum(np.abs(t2), 1.0))


def test_two_level_requires_invertible_transforms(R, host_ctx):
    v, i, _ = R.icosphere(1, 0.0, 1)
    sing = np.diag([1.0, 1.0, 0.0, 1.0])
    d = scenes.SceneDesc()
    o = d.add_object(v, i)
    for k in range(4):
        d.add_instance(o, scenes.translate(k, 0, 0) @ (sing if k == 2 else np.eye(4)), R.Material())
    assert build(R, host_ctx, d).stats()["two_level"] == 0      # automatic: falls back to flat
    with pytest.raises(R.ReinaError) as e:
        build(R, host_ctx, d, accel=R.ACCEL_TWO_LEVEL)
    assert e.value.code == R.REINA_ERR_INVALID
    s = R.Scene(host_ctx)
    s.add_object(v, i)
    s.build()
    with pytest.raises(R.ReinaError):
        s.set_accel(R.ACCEL_FLAT)    # after the build
    with pytest.raises(R.ReinaError):
        R.Scene(host_ctx).set_accel(7)
