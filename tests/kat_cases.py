"""Case records (40 floats) of the single-function known-answer checks shared by the host and GPU tests:
the committed fixtures (offset, GGX VNDF) and seeded Disney evaluation cases."""
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def offset_cases():
    d = json.loads((GOLDEN / "offset_kat.json").read_text())
    p = np.asarray(d["p_bits"], np.uint32).view(np.float32)
    n = np.asarray(d["n_bits"], np.uint32).view(np.float32)
    rec = np.zeros((p.shape[0], 40), np.float32)
    rec[:, 0:3] = p
    rec[:, 3:6] = n
    return rec, np.asarray(d["out_bits"], np.uint32)


def ggx_cases():
    d = json.loads((GOLDEN / "ggx_kat.json").read_text())
    rec = np.zeros((len(d), 40), np.float32)
    for k, c in enumerate(d):
        rec[k, 0:3] = c["V"]
        rec[k, 6] = c["ax"]
        rec[k, 7] = c["ay"]
        rec[k, 8] = np.array([c["seed"]], np.uint32).view(np.float32)[0]
    return rec, np.array([c["h"] for c in d]), np.array([c["state_after"] for c in d], np.uint64)


def frame(n):
    up = np.array([1.0, 0, 0]) if abs(n[1]) > 0.99 else np.array([0, 1.0, 0])
    t = np.cross(up, n)
    t /= np.linalg.norm(t)
    return t, np.cross(n, t), n


def disney_cases(count=256, seed=4):
    g = np.random.default_rng(seed)
    rec = np.zeros((count, 40), np.float32)
    for k in range(count):
        rec[k, 0:9] = g.uniform(0.05, 1.0, 9)                   # base, specTint, sheenTint
        rec[k, 9:17] = g.uniform(0.0, 1.0, 8)                   # aniso, rough, subsurface, ccGloss, metal, cc, trans, sheen
        rec[k, 10] = g.uniform(0.05, 1.0)
        rec[k, 17] = g.choice([0.0, 1.0 / 1.5, 1.5])            # eta (NEE evaluates with 0)
        rec[k, 18] = float(k % 4 == 3)                          # didRefract
        n = g.normal(size=3)
        n /= np.linalg.norm(n)
        wi = g.normal(size=3)
        wi /= np.linalg.norm(wi)
        if wi @ n < 0.05:
            wi = wi - 2 * (wi @ n) * n + 0.1 * n
            wi /= np.linalg.norm(wi)
        wo = g.normal(size=3)
        wo /= np.linalg.norm(wo)
        if k % 5 and wo @ n < 0:
            wo = -wo
        t, b, nn = frame(n)
        rec[k, 19:22] = n
        rec[k, 22:25] = wi
        rec[k, 25:28] = wo
        rec[k, 28:37] = np.concatenate([t, b, nn])
    return rec
