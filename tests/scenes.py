"""Seeded synthetic scenes shared by the tests and bench.py, built through the library's scene API.

ray-cast workload: a level-L icosphere (20*4^L triangles) radially displaced by 3-octave value noise of
amplitude 0.1; rays = a width x height pinhole camera at distance 3 (fovy 45 degrees, pixel centres)
plus n_random rays with origins uniform in the mesh AABB expanded 1.5x and directions uniform on the
sphere (SplitMix64, seed 1).
large scene: the level-8 displaced icosphere (1,310,720 triangles) on a 2-triangle ground plane with one
quad area light above it; per-face Disney parameters drawn from SplitMix64 with 20% of the faces glass
(dielectric, IOR 1.5, absorption U[0, 2]).
"""
from __future__ import annotations

import numpy as np


def splitmix_stream(seed: int):
    state = seed & 0xFFFFFFFFFFFFFFFF
    M = 0xFFFFFFFFFFFFFFFF
    while True:
        state = (state + 0x9E3779B97F4A7C15) & M
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        yield (z ^ (z >> 31)) >> 11


def uniform(n: int, seed: int) -> np.ndarray:
    """n doubles in [0, 1) from SplitMix64 (vectorised restatement of the same recurrence)."""
    M = np.uint64(0xFFFFFFFFFFFFFFFF)
    k = np.arange(1, n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) + k * np.uint64(0x9E3779B97F4A7C15)) & M
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) / float(1 << 53)


def world_triangles(v: np.ndarray, i: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(v[np.asarray(i).reshape(-1, 3)][:, :, :3].reshape(-1, 9), dtype=np.float32)


def raycast_rays(R, level: int, width: int, height: int, n_random: int, v: np.ndarray, seed: int = 1):
    lo = v[:, :3].min(axis=0)
    hi = v[:, :3].max(axis=0)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.5
    return R.raycast_rays(width, height, (0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 45.0, n_random, c - h, c + h, seed=seed)


def sphere_scene(R, ctx, level: int, amplitude: float = 0.1, seed: int = 1):
    v, i, _ = R.icosphere(level, amplitude, seed)
    scene = R.Scene(ctx)
    scene.add_object(v, i)
    scene.build()
    return scene, v, i


GROUND_Y = -1.2
LIGHT_Y = 2.5


def large_scene_geometry(R, level: int = 8, seed: int = 1):
    """Returns [(vertices (N,4), indices)] for sphere, ground plane and light quad (world space)."""
    v, i, _ = R.icosphere(level, 0.1, seed)
    g = 10.0
    plane_v = np.array([[-g, GROUND_Y, -g, 1], [g, GROUND_Y, -g, 1], [g, GROUND_Y, g, 1], [-g, GROUND_Y, g, 1]], np.float32)
    plane_i = np.array([0, 2, 1, 0, 3, 2], np.uint32)  # normal +y
    s = 0.75
    light_v = np.array([[-s, LIGHT_Y, -s, 1], [s, LIGHT_Y, -s, 1], [s, LIGHT_Y, s, 1], [-s, LIGHT_Y, s, 1]], np.float32)
    light_i = np.array([0, 1, 2, 0, 2, 3], np.uint32)  # normal -y
    return [(v, i), (plane_v, plane_i), (light_v, light_i)]


def large_scene_materials(R, n_faces: int, seed: int = 1):
    """Per-face Disney parameters (baseColor U[0,1]^3, metallic, roughness U[0.05,1], specular, clearcoat,
    sheen) with 20% of the faces glass (dielectric, IOR 1.5, absorption U[0,2]).  To keep the number of
    InstanceProperties records bounded, faces draw from a palette of 4096 materials."""
    n_mat = 4096
    u = uniform(n_mat * 12, seed).reshape(n_mat, 12)
    mats = []
    for k in range(n_mat):
        r = u[k]
        if r[11] < 0.2:
            mats.append(R.Material(material_idx=2, albedo=tuple(0.6 + 0.4 * r[0:3]), ior=1.5, absorption=2.0 * r[3],
                                   roughness=0.0))
        else:
            mats.append(R.Material(material_idx=3, albedo=tuple(r[0:3]), metallic=r[3], roughness=0.05 + 0.95 * r[4],
                                   specular_tint=(1.0, 1.0, 1.0), clearcoat=r[6], sheen=r[7], clearcoat_gloss=r[8],
                                   sheen_tint=(1.0, 1.0, 1.0), ior=1.5, specular_transmission=0.0,
                                   subsurface=0.0, anisotropic=0.0))
    face = (uniform(n_faces, seed + 7) * n_mat).astype(np.uint32)
    return mats, face


def large_scene(R, ctx, level: int = 8, seed: int = 1, light_emission=(17.0, 12.0, 4.0)):
    geo = large_scene_geometry(R, level, seed)
    scene = R.Scene(ctx)
    (sv, si), (pv, pi), (lv, li) = geo
    sid = scene.define_object(sv, si)
    mats, face = large_scene_materials(R, si.size // 3, seed)
    scene.add_instance_per_face(sid, None, mats, face)
    scene.add_object(pv, pi, material=R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5)))
    scene.add_object(lv, li, material=R.Material(material_idx=0, albedo=(0.9, 0.9, 0.9), emission=light_emission,
                                                 cull_backface=True))
    scene.build(require_emissive=True)
    tris = np.concatenate([world_triangles(a, b) for a, b in geo])
    return scene, tris, geo
