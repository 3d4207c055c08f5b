"""Converged images against the FP64 oracle at 4096 samples per pixel (NEE+MIS), per workload: the Cornell
room, windows of the 1.3M-triangle scene at 1920x1080 (per-face Disney + 20 % glass, constant environment,
12 bounces) and one scene of the batched workload rendered through the batched entry point next to other
jobs.  The relative RMSE of every window must be at most 1 % (the accumulated image of
raytrace.rgen.glsl:264-284; the same per-pixel sample streams on both sides, so float rounding and the
rare paths it redirects are what differ)."""
import pytest

import converged

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cornell_256", "large_1920x1080", "batch_scene_3"])
def test_converged_rmse_within_one_percent(R, O, gpu_ctx, name):
    res = converged.converged_rmse(R, O, gpu_ctx, name, spp=4096)
    assert max(res["rmse"]) <= 0.01, res
