"""Generates the known-answer fixtures in tests/golden/ from the formulas they pin, restated here in plain
Python/numpy independently of the oracle's C++ (the reference itself ships no tests or vectors).

    python tests/golden/gen_golden.py

rng_kat.json: `random()` of shaders/raytrace/shaderCommon.h.glsl:39-45 — state' = state*747796405 + 1
(mod 2^32), word = ((state' >> ((state' >> 28) + 4)) ^ state') * 277803737, word ^= word >> 22,
value = float(word) / 4294967295.0f — for the seeds {0, 1, 0xFFFFFFFF, 12345, 65536*256+7}, 16 draws each.
offset_kat.json: offsetPositionAlongNormal (closestHitCommon.h.glsl:156-177) on float32 points and normals.
ggx_kat.json: sampleGGXVNDF (brdfDisney.h.glsl:9-40) in float64 with the shader RNG's draws.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
M32 = 0xFFFFFFFF


def rng_words(seed: int, n: int) -> list[int]:
    s = seed & M32
    out = []
    for _ in range(n):
        s = (s * 747796405 + 1) & M32
        w = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & M32
        w = ((w >> 22) ^ w) & M32
        out.append(w)
    return out


def rng_values(words: list[int]) -> list[float]:
    w = np.asarray(words, dtype=np.uint32).astype(np.float32)
    return [float(x) for x in (w / np.float32(4294967295.0)).astype(np.float32)]


F = np.float32
ACES_IN = [(0.59719, 0.35458, 0.04823), (0.07600, 0.90834, 0.01566), (0.02840, 0.13383, 0.83777)]
ACES_OUT = [(1.60475, -0.53108, -0.07367), (-0.10208, 1.10813, -0.00605), (-0.00327, -0.07276, 1.07602)]


def tonemap_f32(rgb: np.ndarray, exposure: float) -> np.ndarray:
    """tonemapping.comp.glsl:66-84 in float32: c * 2^exposure; c * ACESInputMat (GLSL row vector times a
    column-built matrix = dot with each listed vector); RRTAndODTFit; * ACESOutputMat; clamp; RGBA8."""
    c = rgb.astype(F) * F(2.0 ** exposure)

    def mat(c, rows):
        return np.stack([(c[:, 0] * F(r[0]) + c[:, 1] * F(r[1])) + c[:, 2] * F(r[2]) for r in rows], axis=1).astype(F)

    v = mat(c, ACES_IN)
    a = v * (v + F(0.0245786)) - F(0.000090537)
    b = v * (F(0.983729) * v + F(0.4329510)) + F(0.238081)
    v = (a / b).astype(F)
    o = mat(v, ACES_OUT)
    o = np.nan_to_num(np.clip(o, F(0), F(1)), nan=0.0)
    return np.rint(o.astype(np.float64) * 255.0).astype(np.uint8)


def bloom_f32(img: np.ndarray, radius: float, threshold: float, intensity: float) -> np.ndarray:
    """blurCommon.h.glsl blurAxis X (threshold) then Y, then combine.comp.glsl, in float32."""
    H, W = img.shape[:2]

    def blur(src, xaxis, thr):
        side = W if xaxis else H
        K = int(F(side) * F(radius) / F(100.0) * F(3.0) + F(0.5))
        w = [np.exp(F(-(i * i)) / (F(2.0) * F(radius) * F(radius))).astype(F) for i in range(-K, K + 1)]
        wsum = F(0.0)
        for x in w:
            wsum = F(wsum + x)
        out = np.zeros_like(src)
        for y in range(H):
            for x in range(W):
                c = np.zeros(3, F)
                for i in range(-K, K + 1):
                    cx, cy = (x + i, y) if xaxis else (x, y + i)
                    if not (0 <= cx < W and 0 <= cy < H):
                        continue
                    p = src[cy, cx, :3]
                    if thr is not None:
                        lum = F(F(p[0] * F(0.299)) + F(p[1] * F(0.587))) + F(p[2] * F(0.114))
                        if lum < F(thr):
                            continue
                    c = (c + p * w[i + K]).astype(F)
                out[y, x, :3] = c / wsum if wsum >= F(0.0001) else 0
                out[y, x, 3] = 1
        return out

    b = blur(blur(img, True, threshold), False, None)
    res = img.copy()
    res[..., :3] = img[..., :3] + b[..., :3] * F(intensity)
    res[..., 3] = 1
    return res


def offset_f32(p: np.ndarray, n: np.ndarray) -> np.ndarray:
    """offsetPositionAlongNormal (closestHitCommon.h.glsl:156-177) in float32: of_i = int(256 * n)
    (truncation toward zero), p's bit pattern moved by of_i away from zero, and p + n / 65536 where
    |p| < 1/32."""
    p = p.astype(F)
    n = n.astype(F)
    of_i = np.trunc((F(256.0) * n).astype(F)).astype(np.int64)
    bits = p.view(np.int32).astype(np.int64)
    moved = np.where(p < 0, bits - of_i, bits + of_i).astype(np.int32).view(F)
    near = (p + (F(1.0 / 65536.0) * n).astype(F)).astype(F)
    return np.where(np.abs(p) < F(1.0 / 32.0), near, moved).astype(F)


def ggx_vndf_f64(V, ax, ay, seed):
    """sampleGGXVNDF (brdfDisney.h.glsl:9-40) in float64 with the shader RNG's two draws and the shaders'
    k_pi = 3.14159265; returns the half vector and the RNG state after the draws."""
    w = rng_words(seed, 2)
    s = seed & M32
    for _ in range(2):
        s = (s * 747796405 + 1) & M32
    r1, r2 = w[0] / 4294967295.0, w[1] / 4294967295.0
    V = np.array(V, np.float64)
    flip = V[2] < 0
    if flip:
        V[2] = -V[2]
    Vh = np.array([ax * V[0], ay * V[1], V[2]])
    Vh = Vh / np.sqrt(Vh @ Vh)
    lensq = Vh[0] ** 2 + Vh[1] ** 2
    T1 = np.array([-Vh[1], Vh[0], 0.0]) * (1.0 / np.sqrt(lensq)) if lensq > 0 else np.array([1.0, 0.0, 0.0])
    T2 = np.cross(Vh, T1)
    r = np.sqrt(r1)
    phi = 2.0 * 3.14159265 * r2   # k_pi of shaderCommon.h.glsl:47, not the exact pi
    t1 = r * np.cos(phi)
    t2 = r * np.sin(phi)
    sm = 0.5 * (1.0 + Vh[2])
    t2 = (1.0 - sm) * np.sqrt(1.0 - t1 * t1) + sm * t2
    Nh = T1 * t1 + T2 * t2 + Vh * np.sqrt(max(0.0, 1.0 - t1 * t1 - t2 * t2))
    if flip:
        Nh[2] = -Nh[2]
    h = np.array([ax * Nh[0], ay * Nh[1], max(0.0, Nh[2])])
    return (h / np.sqrt(h @ h)).tolist(), s


def main() -> None:
    seeds = [0, 1, 0xFFFFFFFF, 12345, 65536 * 256 + 7]
    rng = {}
    for s in seeds:
        w = rng_words(s, 16)
        rng[str(s)] = {"words": w, "values_f32": rng_values(w)}
    (HERE / "rng_kat.json").write_text(json.dumps(rng, indent=1) + "\n")
    print("wrote", HERE / "rng_kat.json")

    g = np.random.default_rng(2024)
    hdr = np.concatenate([np.zeros((1, 3)), np.full((1, 3), 1e-4), np.full((1, 3), 0.18), np.ones((1, 3)),
                          np.full((1, 3), 100.0), g.exponential(1.0, (59, 3))]).astype(F)
    tm = {"hdr": hdr.tolist(), "out": {}}
    for ex in (0.0, 1.0, -1.5):
        tm["out"][str(ex)] = tonemap_f32(hdr, ex).tolist()
    (HERE / "tonemap_kat.json").write_text(json.dumps(tm) + "\n")
    print("wrote", HERE / "tonemap_kat.json")

    img = np.zeros((12, 16, 4), F)
    img[..., :3] = g.uniform(0.0, 0.6, (12, 16, 3))
    img[3, 5, :3] = (8.0, 4.0, 2.0)
    img[9, 12, :3] = (1.5, 1.5, 1.5)
    img[..., 3] = 1
    combined = bloom_f32(img, 25.0, 1.0, 0.3)
    (HERE / "bloom_kat.json").write_text(json.dumps({"radius": 25.0, "threshold": 1.0, "intensity": 0.3,
                                                     "image": img.tolist(), "combined": combined.tolist()}) + "\n")
    print("wrote", HERE / "bloom_kat.json")

    # offset: points near and away from the origin threshold, both signs, large magnitudes; unit normals
    pts = np.concatenate([g.uniform(-2, 2, (40, 3)), g.uniform(-0.04, 0.04, (20, 3)), g.uniform(-3e4, 3e4, (8, 3)),
                          np.array([[0.0, -0.0, 1.0 / 32.0], [-1.0 / 32.0, 1e-30, 5e-39]])]).astype(F)
    nrm = g.normal(size=(pts.shape[0], 3))
    nrm = (nrm / np.linalg.norm(nrm, axis=1, keepdims=True)).astype(F)
    off = offset_f32(pts, nrm)
    (HERE / "offset_kat.json").write_text(json.dumps({
        "p_bits": pts.view(np.uint32).tolist(), "n_bits": nrm.view(np.uint32).tolist(),
        "out_bits": off.view(np.uint32).tolist()}) + "\n")
    print("wrote", HERE / "offset_kat.json")

    # GGX VNDF: view directions on both hemispheres, isotropic and anisotropic roughness, several seeds
    cases = []
    for k in range(48):
        v = g.normal(size=3)
        v /= np.linalg.norm(v)
        ax, ay = float(g.uniform(0.01, 1.0)), float(g.uniform(0.01, 1.0)) if k % 2 else None
        ay = ax if ay is None else ay
        seed = int(g.integers(0, 2 ** 32))
        vf = [float(F(x)) for x in v]
        axf, ayf = float(F(ax)), float(F(ay))
        h, s_after = ggx_vndf_f64(vf, axf, ayf, seed)
        cases.append({"V": vf, "ax": axf, "ay": ayf, "seed": seed, "h": h, "state_after": s_after})
    (HERE / "ggx_kat.json").write_text(json.dumps(cases, indent=0) + "\n")
    print("wrote", HERE / "ggx_kat.json")


if __name__ == "__main__":
    main()
