"""Child process of tests/test_checked_gpu.py: renders a fixed set of workloads with the library named by
REINA_GB300_LIB and saves the results to the .npz file given as argv[1]."""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent / "reina-vk_gb300"))

import reina_gb300 as R  # noqa: E402
import scenes  # noqa: E402


def main(out_path: str) -> None:
    ctx = R.Context(0)
    out = {}
    room = scenes.textured_room(R).to_product(R, ctx)
    field = scenes.instanced_field(R).to_product(R, ctx)
    cornell = scenes.cornell(R).to_product(R, ctx)
    for name, sc in (("room", room), ("field", field), ("cornell", cornell)):
        iv, ip = scenes.cornell_camera(R, 48, 40)
        pc = R.push_consts(iv, ip, total_emissive_weight=sc.emissive_weight, spp=3, max_bounces=6, focus_dist=3.4)
        for mode in (0, 1):
            acc, smp, _ = R.render(ctx, sc, pc, R.render_options(48, 40, mode, 1, 0, (0, 0, 0)), want_samples=True)
            out[f"{name}_{mode}"] = smp
        rays = R.raycast_rays(64, 64, (0.0, 0.0, 3.4), (0.0, 0.0, 0.0), 40.0, 8192, (-1, -1, -1), (1, 1, 1), seed=2)
        out[f"{name}_hits"] = R.raycast(ctx, sc, rays).view(np.uint32)
    jobs = []
    for k, sc in enumerate((room, field, cornell, room)):
        iv, ip = scenes.cornell_camera(R, 24 + 8 * k, 20)
        pc = R.push_consts(iv, ip, total_emissive_weight=sc.emissive_weight, spp=2, max_bounces=5, focus_dist=3.4)
        jobs.append(R.RenderJob(sc, pc, R.render_options(24 + 8 * k, 20, k % 2, 1 + k, 0, (0, 0, 0)), want_samples=True))
    R.render_batch(ctx, jobs)
    for k, j in enumerate(jobs):
        out[f"batch_{k}"] = j.samples
    np.savez(out_path, **out)


if __name__ == "__main__":
    main(sys.argv[1])
