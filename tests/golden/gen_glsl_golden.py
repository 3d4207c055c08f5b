"""Writes tests/golden/glsl_ref.npz: outputs of the reference's own shader source (reina-vk shaders/**/*.glsl,
compiled for the host by oracle/glsl/build_ref.py and run through oracle/glsl/ref_glsl.py) on seeded inputs.
These fixtures pin the oracle and the device code to the reference wherever the reference's sources are
not available (the GPU machine): known answers of single shader functions, whole renders of the ray-generation,
closest-hit and miss shaders in the reference's own mode, and the bloom + tone-mapping passes.

Needs REINA_REFERENCE_DIR (a reina-vk checkout).  Run: python tests/golden/gen_glsl_golden.py
tests/test_ref_glsl_host.py regenerates every array and checks it against the committed file.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
for p in (str(ROOT), str(ROOT / "reina-vk_gb300"), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

OUT = HERE / "glsl_ref.npz"


def kat_records() -> dict[str, np.ndarray]:
    """Case records (40 floats) for every known-answer kind, seeded."""
    import kat_cases

    g = np.random.default_rng(2024)
    seeds = np.concatenate([np.array([0, 1, 0xFFFFFFFF, 12345, 16777223], np.uint64),
                            g.integers(0, 2**32, 123, dtype=np.uint64)]).astype(np.uint32)
    rec = {}
    r = np.zeros((seeds.size, 40), np.float32)
    r[:, 0] = seeds.view(np.float32)
    rec["random"] = r
    rec["offset"] = kat_cases.offset_cases()[0]
    rec["ggx"] = kat_cases.ggx_cases()[0]
    rec["eval_disney"] = kat_cases.disney_cases()
    off = kat_cases.offset_cases()[0].copy()
    d = g.normal(size=(off.shape[0], 3))
    off[:, 6:9] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rec["offset_dielectric"] = off
    sd = kat_cases.disney_cases(512, 9)
    sd[:, 15] = np.where(np.arange(512) % 3 == 0, g.uniform(0.3, 1.0, 512), sd[:, 15])   # glass lobe often
    sd[:, 17] = g.choice([1.0 / 1.5, 1.5, 1.0 / 1.33], 512)
    sd[:, 37] = g.integers(0, 2**32, 512, dtype=np.uint64).astype(np.uint32).view(np.float32)
    sd[:, 8] = sd[:, 37]
    sd[:, 38] = g.uniform(0.0, 5.0, 512)
    sd[:, 39] = g.uniform(0.0, 5.0, 512)
    rec["sample_disney"] = sd
    refl = np.zeros((256, 40), np.float32)
    refl[:, 0] = g.uniform(-1.0, 1.0, 256)
    refl[:, 1] = g.choice([1.0 / 1.5, 1.5, 1.45, 1.0 / 1.45], 256)
    rec["reflectance"] = refl
    tm = np.zeros((384, 40), np.float32)
    tm[:, 0:3] = np.exp(g.uniform(-6.0, 5.0, (384, 3)))
    tm[:, 3] = g.choice([-1.0, 0.0, 1.0, 2.5], 384)
    rec["tonemap"] = tm
    ga = np.zeros((128, 40), np.float32)
    ga[:, 0] = np.round(g.uniform(-60, 60, 128))
    ga[:, 1] = g.choice([1.0, 5.0, 12.5], 128)
    rec["gauss"] = ga
    return rec


# (kind, record set) of each known-answer output in the file
KATS = {
    "kat_offset": (0, "offset"), "kat_ggx": (1, "ggx"), "kat_eval_disney": (2, "eval_disney"), "kat_random": (3, "random"),
    "kat_offset_dielectric": (4, "offset_dielectric"), "kat_sample_disney": (5, "sample_disney"),
    "kat_diffuse_reflection": (6, "sample_disney"), "kat_random_unit_vec": (7, "sample_disney"),
    "kat_gaussian": (8, "sample_disney"), "kat_hexagon": (9, "sample_disney"), "kat_reflectance": (10, "reflectance"),
    "kat_tonemap": (12, "tonemap"), "kat_gauss": (13, "gauss"), "kat_pdfs": (14, "sample_disney"),
}

# reference-mode renders: (scene, width, height, spp, depth, defocus, sample batches)
RENDERS = {
    "render_cornell": ("cornell", 32, 32, 1, 8, 0.0, 1),
    "render_cornell_accum": ("cornell", 32, 32, 4, 8, 0.0, 2),
    "render_cornell_dof": ("cornell", 32, 32, 2, 4, 0.08, 1),
    "render_zoo_shallow": ("material_zoo", 48, 48, 1, 3, 0.0, 1),
    "render_zoo": ("material_zoo", 48, 48, 2, 8, 0.0, 1),
    "render_textured": ("textured_room", 32, 32, 1, 2, 0.0, 1),
}


def push_consts(R, ps, W, H, spp, depth, defocus, batch):
    import scenes

    iv, ip = scenes.cornell_camera(R, W, H)
    return R.push_consts(iv, ip, sample_batch=batch, total_emissive_weight=ps.emissive_weight, spp=spp,
                         max_bounces=depth, focus_dist=3.4, defocus=defocus)


def hdr_image() -> np.ndarray:
    g = np.random.default_rng(11)
    img = np.exp(g.normal(-1.5, 1.2, (24, 40, 4))).astype(np.float32)
    img[5:8, 10:13, :3] = 30.0
    img[..., 3] = 1.0
    return img


POST = (4.0, 1.0, 0.05, 0.5)   # bloom radius, threshold, intensity; exposure


def generate() -> dict[str, np.ndarray]:
    import reina_gb300 as R
    import scenes
    import glsl_scene
    from oracle.glsl import ref_glsl as G

    R.load_library()
    out = {}
    recs = kat_records()
    for name, rec in recs.items():
        out[f"records_{name}"] = rec
    for name, (kind, rs) in KATS.items():
        out[name] = G.kat(kind, recs[rs])
    ctx = R.Context(-1)
    built = {}
    for name, (scene, W, H, spp, depth, defocus, batches) in RENDERS.items():
        if scene not in built:
            desc = getattr(scenes, scene)(R)
            built[scene] = (desc, desc.to_product(R, ctx, accel=R.ACCEL_FLAT))
        desc, ps = built[scene]
        glsl_scene.load(G, R, desc, ps)
        img = None
        for b in range(batches):
            pc = push_consts(R, ps, W, H, spp, depth, defocus, b)
            img = G.render(glsl_scene.push_bytes(pc), W, H, img)
        out[name] = img
    ctx.close()
    bloomed, rgba8 = G.postprocess(hdr_image(), *POST)
    out["post_input"] = hdr_image()
    out["post_bloomed"] = bloomed
    out["post_rgba8"] = rgba8
    return out


if __name__ == "__main__":
    arrays = generate()
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(arrays)} arrays)")
