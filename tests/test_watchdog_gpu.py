"""The device watchdog: with the traversal step limit of the watchdog build (a few steps), ordinary rays
run past it, and every entry point must report it instead of trapping or hanging — the kernels end the
ray, set the step-limit bit of the error word and return; the synchronous calls (reina_raycast,
reina_render in every form) fail with REINA_ERR_DEVICE, the asynchronous ones (reina_raycast_device,
reina_render_device, reina_render_device_noalloc) succeed at the call and reina_ctx_device_error then
returns the bit and REINA_ERR_DEVICE, clearing the word; the context stays usable.  Nothing waits on a
flag another kernel writes, so the test cannot hang the GPU (the reference surfaces errors as exceptions
caught in src/main.cpp:11-14)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent
STEP_LIMIT_BIT = 2


def test_step_limit_reported_by_every_entry_point(R, tmp_path):
    sys.path.insert(0, str(HERE.parent / "reina-vk_gb300"))
    import build

    lib = build.build_watchdog()
    out = tmp_path / "watchdog.json"
    env = dict(os.environ, REINA_GB300_LIB=str(lib))
    res = subprocess.run([sys.executable, str(HERE / "watchdog_run.py"), str(out)], env=env, capture_output=True,
                         text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    got = json.loads(out.read_text())
    for name in ("raycast", "raycast_any", "render", "render_pass_by_pass", "render_megakernel"):
        assert got[name]["code"] == R.REINA_ERR_DEVICE, (name, got[name])
        assert "step limit" in got[name]["message"], (name, got[name])
    for name in ("raycast_device", "render_device_pass_by_pass", "render_device_noalloc"):
        g = got[name]
        assert g["call"]["code"] == 0, (name, g)
        assert g["error"]["code"] == R.REINA_ERR_DEVICE and "step limit" in g["error"]["message"], (name, g)
        assert g["after"] == 0, (name, g)
    assert got["context_usable"]
