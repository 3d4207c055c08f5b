"""The request server (reina_server_*): continuous batching of render requests submitted while others
run, admission by device-memory budget, LRU eviction of scenes and kept images, progressive
accumulation under an image key, cancellation and budget rejection.

Every finished request must hold exactly the image the same request gets alone (one job in a batched
render): the served kernels trace the same per-path sample streams and sum each pixel's samples in
sample order, whatever else is running.  Against the single-scene entry point the bar is the per-sample
tolerance (see test_batch_gpu)."""
import threading
import time

import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


def sphere_desc(R, level=4, seed=7):
    d = scenes.SceneDesc()
    v, i, _ = R.icosphere(level, 0.1, seed)
    d.add_instance(d.add_object(v, i), None, R.Material(material_idx=3, albedo=(0.6, 0.5, 0.4), roughness=0.4,
                                                        metallic=0.3, specular_tint=(1, 1, 1), sheen_tint=(1, 1, 1)))
    return d


def descs(R):
    return {"cornell": scenes.cornell(R), "zoo": scenes.material_zoo(R), "sphere": sphere_desc(R)}


def request_specs():
    # (scene key, W, H, spp, bounces, mode, env_mode, env, seed)
    out = []
    keys = ["cornell", "zoo", "sphere"]
    rng = np.random.default_rng(11)
    for k in range(18):
        key = keys[k % 3]
        W, H = int(rng.integers(8, 72)), int(rng.integers(8, 72))
        out.append((key, W, H, int(rng.integers(1, 6)), int(rng.integers(0, 10)), int(k % 2), int(k % 4 == 3),
                    (0.2, 0.25, 0.3), k + 1))
    return out


def make_pc(R, scene_weight, W, H, spp, bounces):
    iv, ip = scenes.cornell_camera(R, W, H)
    return R.push_consts(iv, ip, total_emissive_weight=scene_weight, spp=spp, max_bounces=bounces, focus_dist=3.4)


def render_alone(R, ctx, scene, pc, opts, accum=None):
    """The request's image rendered alone: one job in a batched render."""
    j = R.RenderJob(scene, pc, opts, accum=accum)
    R.render_batch(ctx, [j])
    return j.accum


@pytest.fixture(scope="module")
def alone(R):
    """Each request rendered alone on a context of its own; checked against reina_render within the
    per-sample tolerance."""
    ctx = R.Context(0)
    built = {k: d.to_product(R, ctx) for k, d in descs(R).items()}
    weights = {k: s.emissive_weight for k, s in built.items()}
    out = []
    for key, W, H, spp, b, mode, env_mode, env, seed in request_specs():
        pc = make_pc(R, weights[key], W, H, spp, b)
        opts = R.render_options(W, H, mode, seed, env_mode, env)
        acc = render_alone(R, ctx, built[key], pc, opts)
        single, _, _ = R.render(ctx, built[key], pc, opts)
        assert np.abs(acc[..., :3] - single[..., :3]).mean() <= 1e-3 * max(np.abs(single[..., :3]).mean(), 1e-6)
        out.append(acc)
    for s in built.values():
        s.close()
    ctx.close()
    return weights, out


def start_server(R, ctx, **kw):
    srv = R.Server(ctx, **kw)
    ids = {}
    for k, d in descs(R).items():
        ids[k] = srv.add_scene(d.to_product(R, ctx))
    return srv, ids


def submit_all(R, srv, ids, weights, specs, stagger_s=0.0, threads=1):
    outs = [None] * len(specs)
    rids = [None] * len(specs)

    def worker(t):
        for n in range(t, len(specs), threads):
            key, W, H, spp, b, mode, env_mode, env, seed = specs[n]
            outs[n] = np.full((H, W, 4), np.nan, np.float32)
            rids[n] = srv.submit(ids[key], make_pc(R, weights[key], W, H, spp, b),
                                 R.render_options(W, H, mode, seed, env_mode, env), outs[n])
            if stagger_s:
                time.sleep(stagger_s)

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    return rids, outs


@pytest.mark.parametrize("policy,lanes", [("fair", 0), ("fifo", 0), ("shortest", 0), ("shortest_no_aging", 1),
                                          ("shortest_strong_aging", 16)])
def test_same_alone_and_in_the_mix(R, alone, policy, lanes):
    """Requests submitted from 3 threads while earlier ones run: each result equals its lone render
    (fair-share, first-come first-served and shortest-remaining-work wave packing, with and without
    aging; one to sixteen waves in flight)."""
    weights, ref = alone
    ctx = R.Context(0)
    aging = {"shortest_no_aging": -1.0, "shortest_strong_aging": 5.0}.get(policy, 0.0)
    ctx_srv, ids = start_server(R, ctx, wave_paths=4096, fifo=policy == "fifo", fair=policy == "fair",
                                shortest=policy.startswith("shortest"), aging=aging, wave_lanes=lanes)
    srv = ctx_srv
    rids, outs = submit_all(R, srv, ids, weights, request_specs(), stagger_s=0.002, threads=3)
    for n, rid in enumerate(rids):
        st = srv.wait(rid, 120.0)
        assert st["state"] == R.REQ_DONE, st
        assert np.array_equal(outs[n], ref[n], equal_nan=True), f"request {n} differs from its lone render"
    s = srv.stats()
    assert s["completed"] == len(rids) and s["failed"] == 0
    assert 0 < s["latency_p50_s"] <= s["latency_p99_s"] <= s["latency_max_s"]
    assert s["waves"] > 1 and s["rays"] > 0
    srv.close()
    ctx.close()


def test_budget_forces_lru_eviction(R, alone):
    """A budget that holds the path state, one scene and the running requests: scenes are evicted and
    uploaded again, and the results do not change."""
    weights, ref = alone
    ctx = R.Context(0)
    d = descs(R)
    sizes = {}
    for k, desc in d.items():
        s = desc.to_product(R, ctx)
        sizes[k] = s.stats()["device_bytes"]
        s.close()
    wave = 4096
    reserved = R.SERVER_WAVE_LANES * wave * 164 + (64 << 20)
    specs = request_specs()
    biggest_req = max(W * H * 40 for _, W, H, *_ in specs)
    budget = reserved + max(sizes.values()) + 2 * biggest_req + 4096
    srv, ids = start_server(R, ctx, budget_bytes=budget, wave_paths=wave, max_active=2)
    rids, outs = submit_all(R, srv, ids, weights, specs)
    for n, rid in enumerate(rids):
        st = srv.wait(rid, 120.0)
        assert st["state"] == R.REQ_DONE, st
        assert np.array_equal(outs[n], ref[n], equal_nan=True), n
    s = srv.stats()
    assert s["scene_evictions"] > 0 and s["scene_uploads"] > 0
    assert s["peak_resident_bytes"] + s["reserved_bytes"] <= budget
    srv.close()
    ctx.close()


def test_request_larger_than_budget_is_rejected(R):
    ctx = R.Context(0)
    wave = 4096
    srv, ids = start_server(R, ctx, budget_bytes=R.SERVER_WAVE_LANES * wave * 164 + (64 << 20) + (8 << 20), wave_paths=wave)
    with pytest.raises(R.ReinaError) as e:
        srv.submit(ids["cornell"], make_pc(R, 1.0, 1024, 1024, 1, 1), R.render_options(1024, 1024),
                   np.zeros((1024, 1024, 4), np.float32))
    assert e.value.code == R.REINA_ERR_BUDGET
    srv.close()
    ctx.close()


def test_progressive_accumulation_under_a_key(R):
    """Request 1 (sampleBatch 0) and request 2 (sampleBatch 1) on the same image key: the kept image is
    the running mean reina_render gives when called twice on one accumulation buffer."""
    ctx = R.Context(0)
    d = scenes.cornell(R)
    lone = d.to_product(R, ctx)
    W, H = 40, 30
    pc0 = make_pc(R, lone.emissive_weight, W, H, 3, 6)
    pc1 = make_pc(R, lone.emissive_weight, W, H, 3, 6)
    pc1.sampleBatch = 1
    opts = R.render_options(W, H, 1, 5)
    a0 = render_alone(R, ctx, lone, pc0, opts)
    a1 = render_alone(R, ctx, lone, pc1, opts, accum=a0.copy())
    srv = R.Server(ctx, wave_paths=2048)
    sid = srv.add_scene(d.to_product(R, ctx))
    out0 = np.zeros((H, W, 4), np.float32)
    r0 = srv.submit(sid, pc0, opts, out0, image_key=77)
    r1 = srv.submit(sid, pc1, opts, None, image_key=77)   # waits for r0's image
    assert srv.wait(r0, 60.0)["state"] == R.REQ_DONE
    assert srv.wait(r1, 60.0)["state"] == R.REQ_DONE
    assert np.array_equal(out0, a0)
    assert np.array_equal(srv.fetch_image(77), a1)
    # a progressive request on a key without an image fails
    bad = srv.submit(sid, pc1, opts, None, image_key=78)
    st = srv.wait(bad, 60.0)
    assert st["state"] == R.REQ_FAILED and st["error"] == R.REINA_ERR_STATE
    srv.close()
    lone.close()
    ctx.close()


def test_kept_images_are_evicted_and_restored(R):
    """Kept images beyond the budget move to host memory and come back for the next progressive request."""
    ctx = R.Context(0)
    d = scenes.cornell(R)
    lone = d.to_product(R, ctx)
    scene_bytes = lone.stats()["device_bytes"]
    W, H = 64, 64
    wave = 4096
    # room for the scene and two kept images besides the running request (40 B/px): the third key evicts
    budget = R.SERVER_WAVE_LANES * wave * 164 + (64 << 20) + scene_bytes + 2 * W * H * 40
    srv = R.Server(ctx, budget_bytes=budget, wave_paths=wave, max_active=1)
    sid = srv.add_scene(d.to_product(R, ctx))
    firsts = []
    for key in range(1, 6):
        pc = make_pc(R, lone.emissive_weight, W, H, 1, 4)
        opts = R.render_options(W, H, 1, key)
        srv.wait(srv.submit(sid, pc, opts, None, image_key=key), 60.0)
        firsts.append((pc, opts, render_alone(R, ctx, lone, pc, opts)))
    s = srv.stats()
    assert s["image_evictions"] > 0
    for key in range(1, 6):
        pc, opts, a = firsts[key - 1]
        pc.sampleBatch = 1
        st = srv.wait(srv.submit(sid, pc, opts, None, image_key=key), 60.0)
        assert st["state"] == R.REQ_DONE
        want = render_alone(R, ctx, lone, pc, opts, accum=a.copy())
        assert np.array_equal(srv.fetch_image(key), want), key
    assert srv.stats()["image_restores"] > 0
    srv.close()
    lone.close()
    ctx.close()


def test_cancel_and_close_with_pending_requests(R):
    ctx = R.Context(0)
    srv, ids = start_server(R, ctx, wave_paths=4096)
    pc = make_pc(R, 1.0, 256, 256, 64, 12)
    outs = [np.zeros((256, 256, 4), np.float32) for _ in range(4)]
    rids = [srv.submit(ids["zoo"], pc, R.render_options(256, 256, 0, k), outs[k]) for k in range(4)]
    srv.cancel(rids[3])
    st = srv.wait(rids[3], 120.0)
    assert st["state"] in (R.REQ_CANCELLED, R.REQ_DONE)
    srv.close()   # the others are cancelled or done; nothing hangs
    ctx.close()
