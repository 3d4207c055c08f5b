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


def main() -> None:
    seeds = [0, 1, 0xFFFFFFFF, 12345, 65536 * 256 + 7]
    rng = {}
    for s in seeds:
        w = rng_words(s, 16)
        rng[str(s)] = {"words": w, "values_f32": rng_values(w)}
    (HERE / "rng_kat.json").write_text(json.dumps(rng, indent=1) + "\n")
    print("wrote", HERE / "rng_kat.json")


if __name__ == "__main__":
    main()
