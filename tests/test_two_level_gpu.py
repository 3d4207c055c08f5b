"""Two-level scenes on the GPU: ray casts bit-exact against the oracle's instanced restatement (ids and
refined t/u/v), renders through both traversals agreeing with the flattened scene and the oracle, the
megakernel, and batches that mix flat and two-level scenes (each job equal to itself alone)."""
import numpy as np
import pytest

import scenes
from test_two_level_host import field_rays, oracle_instanced

pytestmark = pytest.mark.gpu


def agree(a, b, rtol=1e-4):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ok = (np.abs(a - b) <= rtol * np.abs(b) + 1e-6) | (np.isnan(a) & np.isnan(b))
    return ok.all(axis=-1)


@pytest.fixture(scope="module")
def field(R, gpu_ctx):
    d = scenes.instanced_field(R)
    two = d.to_product(R, gpu_ctx)
    flat = d.to_product(R, gpu_ctx, accel=R.ACCEL_FLAT)
    assert two.stats()["two_level"] == 1 and flat.stats()["two_level"] == 0
    return d, two, flat


def test_two_level_raycast_bit_exact(R, O, gpu_ctx, field):
    d, two, _ = field
    inst, _ = oracle_instanced(O, d, two)
    rays = np.concatenate([field_rays(R, 100000, 5), R.raycast_rays(256, 256, (0.0, 0.0, 3.4), (0.0, 0.0, 0.0), 40.0, 0,
                                                                    (-1, -1, -1), (1, 1, 1), seed=1)])
    hits = R.raycast(gpu_ctx, two, rays)
    ref = inst.raycast(rays)
    assert np.array_equal(hits["prim"], ref["prim"])
    assert np.array_equal(hits.view(np.uint32), ref.view(np.uint32))   # refined t, u, v too
    assert (ref["prim"] != O.MISS).mean() > 0.5
    any_hits = R.raycast(gpu_ctx, two, rays, R.RAY_ANY)
    assert np.array_equal(any_hits["prim"] == O.MISS, ref["prim"] == O.MISS)


def test_two_level_counters(R, gpu_ctx, field):
    import torch

    _, two, flat = field
    rays = field_rays(R, 65536, 9)
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    n2, t2 = R.raycast_counters(gpu_ctx, two, d_rays.data_ptr(), rays.shape[0], R.RAY_CLOSEST, stream)
    n1, t1 = R.raycast_counters(gpu_ctx, flat, d_rays.data_ptr(), rays.shape[0], R.RAY_CLOSEST, stream)
    assert n2 > rays.shape[0] and t2 > 0 and n1 > 0 and t1 > 0


@pytest.mark.parametrize("mode", [0, 1])
def test_two_level_render_matches_flat_and_oracle(R, O, gpu_ctx, field, mode):
    d, two, flat = field
    W = H = 96
    iv, ip = scenes.cornell_camera(R, W, H)
    pc = R.push_consts(iv, ip, total_emissive_weight=two.emissive_weight, spp=4, max_bounces=6, focus_dist=3.4)
    opts = R.render_options(W, H, mode, 1, 0, (0, 0, 0))
    _, s2, _ = R.render(gpu_ctx, two, pc, opts, want_samples=True)
    _, s1, _ = R.render(gpu_ctx, flat, pc, opts, want_samples=True)
    assert agree(s2, s1).mean() >= 0.99
    _, so = d.to_oracle(O).render(pc, W, H, mode=mode, want_samples=True)
    assert agree(s2, so).mean() >= 0.99
    _, sm, _ = R.render(gpu_ctx, two, pc, R.render_options(W, H, mode, 1, 0, (0, 0, 0), megakernel=True),
                        want_samples=True)
    assert agree(sm, s2).mean() >= 0.99


def test_batch_mixes_flat_and_two_level(R, gpu_ctx, field):
    _, two, flat = field
    cornell = scenes.cornell(R).to_product(R, gpu_ctx)
    specs = []
    for k, (scene, W, H, spp, mode) in enumerate([(two, 40, 32, 3, 1), (cornell, 32, 24, 2, 1), (flat, 24, 24, 2, 0),
                                                  (two, 16, 40, 4, 0)]):
        iv, ip = scenes.cornell_camera(R, W, H)
        pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=spp, max_bounces=5, focus_dist=3.4)
        specs.append((scene, pc, R.render_options(W, H, mode, 2 + k, 0, (0, 0, 0))))
    batch = [R.RenderJob(s, pc, o, want_samples=True) for s, pc, o in specs]
    R.render_batch(gpu_ctx, batch)
    for j, (s, pc, o) in zip(batch, specs):
        one = [R.RenderJob(s, pc, o, want_samples=True)]
        R.render_batch(gpu_ctx, one)
        assert np.array_equal(j.samples, one[0].samples, equal_nan=True)
        assert np.array_equal(j.accum, one[0].accum, equal_nan=True)
