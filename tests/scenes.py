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
    """Returns [(vertices (N,4), indices)] for sphere, ground plane and light quad (world space).
    large_scene_tbn() gives the sphere's per-vertex tangent frames."""
    v, i, _ = R.icosphere(level, 0.1, seed)
    _, plane, light = large_scene_geometry_planes()
    return [(v, i), plane, light]


def large_scene_geometry_planes():
    """(None, ground plane, light quad) of the large scene, world space."""
    g = 10.0
    plane_v = np.array([[-g, GROUND_Y, -g, 1], [g, GROUND_Y, -g, 1], [g, GROUND_Y, g, 1], [-g, GROUND_Y, g, 1]], np.float32)
    plane_i = np.array([0, 2, 1, 0, 3, 2], np.uint32)  # normal +y
    s = 0.75
    light_v = np.array([[-s, LIGHT_Y, -s, 1], [s, LIGHT_Y, -s, 1], [s, LIGHT_Y, s, 1], [-s, LIGHT_Y, s, 1]], np.float32)
    light_i = np.array([0, 1, 2, 0, 2, 3], np.uint32)  # normal -y
    return None, (plane_v, plane_i), (light_v, light_i)


def large_scene_materials(R, n_faces: int, seed: int = 1, n_mat: int = 4096):
    """Per-face Disney parameters (baseColor U[0,1]^3, metallic, roughness U[0.05,1], specular, clearcoat,
    sheen) with 20% of the faces glass (dielectric, IOR 1.5, absorption U[0,2]).  To keep the number of
    InstanceProperties records bounded, faces draw from a palette of n_mat materials."""
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


def large_scene_tbn(R, level: int = 8, seed: int = 1):
    """Per-vertex TBNs of the large scene's sphere (N = undisplaced radial direction)."""
    _, _, n = R.icosphere(level, 0.1, seed)
    return tbn_from_normals(n)


def tbn_from_normals(n: np.ndarray) -> np.ndarray:
    """Per-vertex frames (columns T, B, N) with T = normalize(up x N)."""
    up = np.where(np.abs(n[:, 1:2]) > 0.99, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    t = np.cross(up, n)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(n, t)
    return np.concatenate([t, b, n], axis=1).astype(np.float32)


def large_scene(R, ctx, level: int = 8, seed: int = 1, light_emission=(17.0, 12.0, 4.0)):
    geo = large_scene_geometry(R, level, seed)
    scene = R.Scene(ctx)
    (sv, si), (pv, pi), (lv, li) = geo
    sid = scene.define_object(sv, si, tbns=large_scene_tbn(R, level, seed), tbn_indices=si)
    mats, face = large_scene_materials(R, si.size // 3, seed)
    scene.add_instance_per_face(sid, None, mats, face)
    scene.add_object(pv, pi, material=R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5)))
    scene.add_object(lv, li, material=R.Material(material_idx=0, albedo=(0.9, 0.9, 0.9), emission=light_emission,
                                                 cull_backface=True))
    scene.build(require_emissive=True)
    tris = np.concatenate([world_triangles(a, b) for a, b in geo])
    return scene, tris, geo


# ---------------------------------------------------------------------------------------------------
# Batched workload: independent scenes of uneven size, each a displaced geodesic sphere (triangle count
# log-uniform over [1k, 500k]) with per-face Disney / glass materials, a ground plane and one quad light
# under a constant environment, rendered at a square resolution with side U[128, 1024], spp U{1..64} and
# depth U{4..12} with NEE + MIS.

BATCH_ENV = (0.3, 0.3, 0.35)


def batch_job_params(index: int, seed: int = 1) -> dict:
    u = uniform(4, 1_000_003 * seed + index)
    tris = float(np.exp(np.log(1000.0) + u[0] * (np.log(500000.0) - np.log(1000.0))))
    freq = int(np.clip(round(np.sqrt(tris / 20.0)), 7, 158))
    return {"frequency": freq, "triangles": 20 * freq * freq + 4, "side": 128 + min(896, int(u[1] * 897)),
            "spp": 1 + min(63, int(u[2] * 64)), "depth": 4 + min(8, int(u[3] * 9)), "seed": index + 1}


def batch_scene(R, ctx, index: int, seed: int = 1, n_mat: int = 256):
    p = batch_job_params(index, seed)
    v, i, n = R.geodesic(p["frequency"], 0.1, 7919 * seed + index)
    scene = R.Scene(ctx)
    sid = scene.define_object(v, i, tbns=tbn_from_normals(n), tbn_indices=i)
    mats, face = large_scene_materials(R, i.size // 3, 7919 * seed + index, n_mat)
    scene.add_instance_per_face(sid, None, mats, face)
    _, (pv, pi), (lv, li) = large_scene_geometry_planes()
    scene.add_object(pv, pi, material=R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5)))
    scene.add_object(lv, li, material=R.Material(material_idx=0, albedo=(0.9, 0.9, 0.9), emission=(17.0, 12.0, 4.0),
                                                 cull_backface=True))
    scene.build(require_emissive=True)
    return scene, p


def batch_job(R, scene, p: dict):
    """(push constants, options) of one batched job."""
    side = p["side"]
    iv, ip = R.camera_matrices((0.0, 0.4, 3.6), (0.0, -0.12, -1.0), (0.0, 1.0, 0.0), np.radians(40.0), 1.0)
    pc = R.push_consts(iv, ip, total_emissive_weight=scene.emissive_weight, spp=p["spp"], max_bounces=p["depth"],
                       focus_dist=3.6)
    opts = R.render_options(side, side, R.MODE_NEE_MIS, p["seed"], R.ENV_CONSTANT, BATCH_ENV)
    return pc, opts


# ---------------------------------------------------------------------------------------------------
# Scene descriptions built identically through the library's scene API and through the oracle.

def translate(x, y, z):
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = (x, y, z)
    return m


def rotate_y(deg):
    a = np.radians(deg)
    c, s = np.cos(a), np.sin(a)
    m = np.eye(4, dtype=np.float32)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    return m


def scale(x, y, z):
    return np.diag([x, y, z, 1.0]).astype(np.float32)


def col_major(m) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, np.float32).T.reshape(16))


class SceneDesc:
    def __init__(self):
        self.objects = []     # (v4, idx, tbn9, tbn_idx)
        self.instances = []   # (obj, 4x4 math transform, [materials], face_material or None)

    def add_object(self, v4, idx, tbn9=None, tbn_idx=None) -> int:
        v4 = np.asarray(v4, np.float32)
        if v4.shape[1] == 3:
            v4 = np.concatenate([v4, np.ones((v4.shape[0], 1), np.float32)], 1)
        self.objects.append((v4, np.asarray(idx, np.uint32).reshape(-1), tbn9, tbn_idx))
        return len(self.objects) - 1

    def add_instance(self, obj, transform=None, material=None, materials=None, face_material=None):
        T = np.eye(4, dtype=np.float32) if transform is None else np.asarray(transform, np.float32)
        self.instances.append((obj, T, materials if materials is not None else [material], face_material))

    def to_product(self, R, ctx, require_emissive=False):
        s = R.Scene(ctx)
        for v4, idx, t9, ti in self.objects:
            s.define_object(v4, idx, tbns=t9, tbn_indices=ti)
        for obj, T, mats, fm in self.instances:
            if fm is None:
                s.add_instance(obj, T, mats[0])
            else:
                s.add_instance_per_face(obj, T, mats, fm)
        s.build(require_emissive=require_emissive)
        return s

    def to_oracle(self, O):
        s = O.Scene()
        for v4, idx, t9, ti in self.objects:
            s.add_object(v4, idx, t9, ti)
        for obj, T, mats, fm in self.instances:
            s.add_instance(obj, col_major(T), mats, fm)
        s.finalize()
        return s


def quad(corner, e1, e2):
    """Quad corner, corner+e1, corner+e1+e2, corner+e2 with normal along e1 x e2."""
    c, a, b = (np.asarray(x, np.float32) for x in (corner, e1, e2))
    v = np.stack([c, c + a, c + a + b, c + b])
    return v, np.array([0, 1, 2, 0, 2, 3], np.uint32)


def unit_cube():
    v = np.array([[-.5, -.5, -.5], [.5, -.5, -.5], [.5, .5, -.5], [-.5, .5, -.5],
                  [-.5, -.5, .5], [.5, -.5, .5], [.5, .5, .5], [-.5, .5, .5]], np.float32)
    i = np.array([0, 2, 1, 0, 3, 2, 4, 5, 6, 4, 6, 7, 0, 4, 7, 0, 7, 3, 1, 2, 6, 1, 6, 5, 0, 1, 5, 0, 5, 4,
                  3, 7, 6, 3, 6, 2], np.uint32)
    return v, i


GREY = (0.73, 0.73, 0.73)
RED = (0.65, 0.05, 0.05)
GREEN = (0.12, 0.45, 0.15)
CORNELL_LIGHT = (17.0, 12.0, 4.0)


def cornell(R, seed: int = 1) -> SceneDesc:
    """The procedural Cornell-style room: 5 walls (10 tris), 2 boxes rotated about y by seeded angles
    (24 tris, one cube object instanced twice), an emissive back-face-culled ceiling quad (2 tris)."""
    u = uniform(2, seed)
    d = SceneDesc()
    lam = lambda c: R.Material(material_idx=0, albedo=c)
    walls = [
        (quad((-1, -1, 1), (2, 0, 0), (0, 0, -2)), GREY),    # floor, normal +y
        (quad((-1, 1, -1), (2, 0, 0), (0, 0, 2)), GREY),     # ceiling, normal -y
        (quad((-1, -1, -1), (2, 0, 0), (0, 2, 0)), GREY),    # back, normal +z
        (quad((-1, -1, 1), (0, 0, -2), (0, 2, 0)), RED),     # left, normal +x
        (quad((1, -1, -1), (0, 0, 2), (0, 2, 0)), GREEN),    # right, normal -x
    ]
    for (v, i), col in walls:
        d.add_instance(d.add_object(v, i), None, lam(col))
    cube = d.add_object(*unit_cube())
    t1 = 15.0 + 5.0 * u[0]
    t2 = 15.0 + 5.0 * u[1]
    d.add_instance(cube, translate(-0.35, -0.4, -0.3) @ rotate_y(t1) @ scale(0.6, 1.2, 0.6), lam(GREY))
    d.add_instance(cube, translate(0.35, -0.7, 0.35) @ rotate_y(-t2) @ scale(0.6, 0.6, 0.6), lam(GREY))
    lv, li = quad((-0.25, 0.999, -0.2), (0.5, 0, 0), (0, 0, 0.4))   # normal -y
    d.add_instance(d.add_object(lv, li), None,
                   R.Material(material_idx=0, albedo=(0.78, 0.78, 0.78), emission=CORNELL_LIGHT, cull_backface=True))
    return d


def cornell_camera(R, width: int, height: int):
    iv, ip = R.camera_matrices((0.0, 0.0, 3.4), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0), np.radians(40.0), width / height)
    return iv, ip


def sphere_tbn(level: int, amplitude: float, seed: int, R):
    """Icosphere with per-vertex TBNs (N = undisplaced radial direction, T = normalize(up x N))."""
    v, i, n = R.icosphere(level, amplitude, seed)
    up = np.where(np.abs(n[:, 1:2]) > 0.99, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    t = np.cross(up, n)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(n, t)
    tbn = np.concatenate([t, b, n], axis=1).astype(np.float32)   # columns T, B, N
    return v, i, tbn, i.copy()


def material_zoo(R, seed: int = 3) -> SceneDesc:
    """Cornell room plus spheres of every material: metal (fuzzy), dielectric with Beer absorption, and
    Disney variants (diffuse+sheen+subsurface, metallic, clearcoat, transmissive glass lobe), one of them
    back-face culled and one scaled/rotated by its instance transform."""
    d = cornell(R, seed)
    v, i, tbn, ti = sphere_tbn(3, 0.05, seed, R)
    sph = d.add_object(v, i, tbn, ti)
    mats = [
        R.Material(material_idx=1, albedo=(0.9, 0.8, 0.6), roughness=0.2),
        R.Material(material_idx=2, albedo=(0.8, 0.9, 0.95), ior=1.5, absorption=1.5, roughness=0.05, interp_normals=True),
        R.Material(material_idx=3, albedo=(0.7, 0.3, 0.2), roughness=0.6, subsurface=0.4, sheen=0.8,
                   sheen_tint=(0.5, 0.5, 0.5), specular_tint=(1, 1, 1), interp_normals=True),
        R.Material(material_idx=3, albedo=(0.95, 0.75, 0.3), metallic=0.9, roughness=0.3, anisotropic=0.5,
                   specular_tint=(1, 1, 1), sheen_tint=(1, 1, 1)),
        R.Material(material_idx=3, albedo=(0.2, 0.4, 0.8), clearcoat=1.0, clearcoat_gloss=0.7, roughness=0.4,
                   specular_tint=(1, 1, 1), sheen_tint=(1, 1, 1), cull_backface=True),
        R.Material(material_idx=3, albedo=(0.9, 0.95, 0.9), specular_transmission=0.8, ior=1.45, roughness=0.15,
                   specular_tint=(1, 1, 1), sheen_tint=(1, 1, 1)),
    ]
    pos = [(-0.6, -0.75, 0.5), (0.0, -0.75, 0.6), (0.6, -0.75, 0.5), (-0.55, 0.3, 0.2), (0.55, 0.2, 0.1),
           (0.0, 0.35, 0.4)]
    for k, (m, p) in enumerate(zip(mats, pos)):
        T = translate(*p) @ rotate_y(20.0 * k) @ scale(0.22, 0.22 if k != 3 else 0.3, 0.22)
        d.add_instance(sph, T, m)
    return d
