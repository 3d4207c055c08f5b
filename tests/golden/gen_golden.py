"""Generates the known-answer fixtures in tests/golden/ from the formulas they pin, restated here in plain
Python/numpy independently of the oracle's C++ (the reference itself ships no tests or vectors).

    python tests/golden/gen_golden.py

rng_kat.json: `random()` of shaders/raytrace/shaderCommon.h.glsl:39-45 — state' = state*747796405 + 1
(mod 2^32), word = ((state' >> ((state' >> 28) + 4)) ^ state') * 277803737, word ^= word >> 22,
value = float(word) / 4294967295.0f — for the seeds {0, 1, 0xFFFFFFFF, 12345, 65536*256+7}, 16 draws each.
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


if __name__ == "__main__":
    main()
