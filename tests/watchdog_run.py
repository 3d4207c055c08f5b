"""Child process of tests/test_watchdog_gpu.py: runs ordinary workloads on the library named by
REINA_GB300_LIB (the watchdog build, whose traversal step limit is a few steps) and records, per entry
point, the status it returned and the device error bits it reported, as JSON in argv[1]."""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent / "reina-vk_gb300"))

import reina_gb300 as R  # noqa: E402
import scenes  # noqa: E402


def status(fn):
    try:
        fn()
        return {"code": 0, "message": ""}
    except R.ReinaError as e:
        return {"code": e.code, "message": str(e)}


def main(out_path: str) -> None:
    import torch

    ctx = R.Context(0)
    out = {}
    # scenes whose trees are deeper than the watchdog build's step limit: a 20,480-triangle sphere for the
    # ray casts, the material zoo (7,700 triangles) for the renders
    sphere, v, _ = scenes.sphere_scene(R, ctx, 5)
    rays = scenes.raycast_rays(R, 5, 32, 32, 1024, v)
    sc = scenes.material_zoo(R).to_product(R, ctx, accel=R.ACCEL_FLAT)
    out["raycast"] = status(lambda: R.raycast(ctx, sphere, rays))
    out["raycast_any"] = status(lambda: R.raycast(ctx, sphere, rays, R.RAY_ANY))
    iv, ip = scenes.cornell_camera(R, 32, 32)
    pc = R.push_consts(iv, ip, total_emissive_weight=sc.emissive_weight, spp=2, max_bounces=4, focus_dist=3.4)
    for name, kw in (("render", {}), ("render_pass_by_pass", {"pass_by_pass": True}), ("render_megakernel", {"megakernel": True})):
        opts = R.render_options(32, 32, R.MODE_NEE_MIS, 1, **kw)
        out[name] = status(lambda: R.render(ctx, sc, pc, opts))
    # asynchronous entry points: nothing fails at the call; reina_ctx_device_error reports the bits
    stream = torch.cuda.current_stream().cuda_stream
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    acc = torch.zeros((32, 32, 4), dtype=torch.float32, device="cuda")
    calls = {
        "raycast_device": lambda: R.raycast_device(ctx, sphere, d_rays.data_ptr(), rays.shape[0], d_hits.data_ptr(), R.RAY_CLOSEST, stream),
        "render_device_pass_by_pass": lambda: R.render_device(ctx, sc, pc, R.render_options(32, 32, R.MODE_NEE_MIS, 1, pass_by_pass=True),
                                                              acc.data_ptr(), 0, stream),
        "render_device_noalloc": lambda: R.render_device_noalloc(ctx, sc, pc, R.render_options(32, 32, R.MODE_NEE_MIS, 1),
                                                                 acc.data_ptr(), 0, stream),
    }
    for name, fn in calls.items():
        call = status(fn)
        bits = {"bits": -1}
        try:
            bits["bits"] = R.device_error(ctx, stream)
        except R.ReinaError as e:
            bits = {"bits": None, "code": e.code, "message": str(e)}
        after = R.device_error(ctx, stream)   # the word was cleared by the read
        out[name] = {"call": call, "error": bits, "after": after}
    # the context stays usable: a device computation without traversal
    kat = R.device_kat(ctx, R.KAT_RANDOM, np.zeros((4, 40), np.float32))
    out["context_usable"] = bool(np.isfinite(kat).all())
    Path(out_path).write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main(sys.argv[1])
