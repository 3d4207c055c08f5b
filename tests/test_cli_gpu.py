"""The headless renderer (reina_render, the reference's run loop without a window): it loads a glTF
scene and config.toml, renders frame after frame, saves PNGs on the SaveManager schedule plus the final
frame; the final PNG equals the same frames rendered and post-processed through the library's API."""
import struct
import subprocess
import zlib

import numpy as np
import pytest

from test_loaders_host import CONFIG, make_gltf, read_png

pytestmark = pytest.mark.gpu


def test_cli_renders_and_saves(R, tmp_path):
    import build as pkg_build

    pkg_build.build()
    cli = pkg_build.CLI
    (tmp_path / "config.toml").write_text(CONFIG.replace("save_on_samples = [300, 100, 200]", "save_on_samples = [4, 7]")
                                          .replace("save_on_times = [30.5, 10]", "save_on_times = [1000]"))
    (tmp_path / "s.glb").write_bytes(make_gltf(True))
    out = tmp_path / "out"
    out.mkdir()
    W, H, frames = 48, 40, 3
    res = subprocess.run([str(cli), "--config", str(tmp_path / "config.toml"), "--scene", str(tmp_path / "s.glb"),
                          "--width", str(W), "--height", str(H), "--frames", str(frames), "--out", str(out),
                          "--camera", "1,0.5,6", "--look-at", "1,0.5,0", "--fov", "40", "--mode", "nee"],
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    # samples before frames 0, 1, 2 are 0, 4, 8 (4 spp per frame): 4 < 8 -> output_4spp.png at frame 2
    assert sorted(p.name for p in out.iterdir()) == ["output_4spp.png", "output_final.png"]
    img = read_png((out / "output_final.png").read_bytes())
    assert img.shape == (H, W, 4)

    c = R.load_config(tmp_path / "config.toml")
    ctx = R.Context(0)
    try:
        s = R.Scene(ctx)
        s.add_gltf(tmp_path / "s.glb")
        s.build(require_emissive=True)
        iv, ip = R.camera_matrices((1, 0.5, 6), (0, 0, -6), (0, 1, 0), np.radians(40.0), W / H, 0.1, 100.0)
        acc = np.zeros((H, W, 4), np.float32)
        for f in range(frames):
            pc = R.push_consts(iv, ip, sample_batch=f, total_emissive_weight=s.emissive_weight,
                               focus_dist=c.focus_dist, defocus=c.defocus_multiplier, direct_clamp=c.direct_clamp,
                               indirect_clamp=c.indirect_clamp, spp=c.samples_per_pixel, max_bounces=c.max_bounces)
            acc, _, _ = R.render(ctx, s, pc, R.render_options(W, H, R.MODE_NEE_MIS, 1), accum=acc)
        rgba, _ = R.postprocess(ctx, acc, c.bloom.radius, c.bloom.threshold, c.bloom.intensity, c.tonemap.exposure)
        assert np.array_equal(rgba, img)
        s.close()
    finally:
        ctx.close()


def test_cli_takes_scene_and_camera_from_config(R, tmp_path):
    """The config's optional [render] / [scene] / [camera] keys stand in for the options: the same image
    as passing them on the command line."""
    import build as pkg_build

    pkg_build.build()
    cli = pkg_build.CLI
    base = (CONFIG.replace("save_on_samples = [300, 100, 200]", "save_on_samples = []")
            .replace("save_on_times = [30.5, 10]", "save_on_times = []"))
    (tmp_path / "s.glb").write_bytes(make_gltf(True))
    (tmp_path / "plain.toml").write_text(base)
    (tmp_path / "keys.toml").write_text(base + f'\n[render]\nwidth = 40\nheight = 32\nseed = 3\nmode = "nee"\n'
                                        f'[scene]\npath = "{tmp_path / "s.glb"}"\n'
                                        f'[camera]\npos = [1, 0.5, 6]\nlook_at = [1, 0.5, 0]\nfov = 40\n')
    outs = []
    for name, extra in (("plain", ["--scene", str(tmp_path / "s.glb"), "--width", "40", "--height", "32", "--seed", "3",
                                   "--mode", "nee", "--camera", "1,0.5,6", "--look-at", "1,0.5,0", "--fov", "40"]),
                        ("keys", [])):
        out = tmp_path / name
        out.mkdir()
        res = subprocess.run([str(cli), "--config", str(tmp_path / f"{name}.toml"), "--frames", "2", "--out", str(out),
                              *extra], capture_output=True, text=True, timeout=300)
        assert res.returncode == 0, res.stderr
        outs.append(read_png((out / "output_final.png").read_bytes()))
    assert outs[0].shape == (32, 40, 4) and np.array_equal(outs[0], outs[1])
