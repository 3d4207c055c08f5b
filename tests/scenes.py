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


def large_scene_desc(R, level: int = 8, seed: int = 1, light_emission=(17.0, 12.0, 4.0)) -> "SceneDesc":
    """The large scene as a description (both the product and the oracle can build it)."""
    geo = large_scene_geometry(R, level, seed)
    (sv, si), (pv, pi), (lv, li) = geo
    mats, face = large_scene_materials(R, si.size // 3, seed)
    d = SceneDesc()
    d.add_instance(d.add_object(sv, si, large_scene_tbn(R, level, seed), si), None, materials=mats, face_material=face)
    d.add_instance(d.add_object(pv, pi), None, R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5)))
    d.add_instance(d.add_object(lv, li), None,
                   R.Material(material_idx=0, albedo=(0.9, 0.9, 0.9), emission=light_emission, cull_backface=True))
    return d


LARGE_ENV = (0.3, 0.3, 0.35)


def large_camera(R, W: int = 1920, H: int = 1080):
    """The large scene's camera (1920x1080 frame of the render workload)."""
    return R.camera_matrices((0.0, 0.4, 3.6), (0.0, -0.12, -1.0), (0.0, 1.0, 0.0), np.radians(40.0), W / H)


def batch_scene_desc(R, index: int, seed: int = 1, n_mat: int = 256) -> "SceneDesc":
    """Scene `index` of the batched workload as a description (see batch_scene)."""
    p = batch_job_params(index, seed)
    v, i, n = R.geodesic(p["frequency"], 0.1, 7919 * seed + index)
    mats, face = large_scene_materials(R, i.size // 3, 7919 * seed + index, n_mat)
    d = SceneDesc()
    d.add_instance(d.add_object(v, i, tbn_from_normals(n), i), None, materials=mats, face_material=face)
    _, (pv, pi), (lv, li) = large_scene_geometry_planes()
    d.add_instance(d.add_object(pv, pi), None, R.Material(material_idx=0, albedo=(0.5, 0.5, 0.5)))
    d.add_instance(d.add_object(lv, li), None,
                   R.Material(material_idx=0, albedo=(0.9, 0.9, 0.9), emission=(17.0, 12.0, 4.0), cull_backface=True))
    return d


def large_scene(R, ctx, level: int = 8, seed: int = 1, light_emission=(17.0, 12.0, 4.0), bvh=None):
    geo = large_scene_geometry(R, level, seed)
    scene = R.Scene(ctx)
    if bvh is not None:   # R.BVH_HOST or R.BVH_DEVICE
        scene.set_bvh_build(bvh)
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
        self.objects = []     # (v4, idx, tbn9, tbn_idx, uv, uv_idx)
        self.instances = []   # (obj, 4x4 math transform, [materials], face_material or None)
        self.textures = []    # (H, W, 4) uint8, row 0 at v = 0

    def add_object(self, v4, idx, tbn9=None, tbn_idx=None, uv=None, uv_idx=None) -> int:
        v4 = np.asarray(v4, np.float32)
        if v4.shape[1] == 3:
            v4 = np.concatenate([v4, np.ones((v4.shape[0], 1), np.float32)], 1)
        self.objects.append((v4, np.asarray(idx, np.uint32).reshape(-1), tbn9, tbn_idx, uv, uv_idx))
        return len(self.objects) - 1

    def add_texture(self, rgba8) -> int:
        self.textures.append(np.ascontiguousarray(rgba8, np.uint8))
        return len(self.textures) - 1

    def add_instance(self, obj, transform=None, material=None, materials=None, face_material=None):
        T = np.eye(4, dtype=np.float32) if transform is None else np.asarray(transform, np.float32)
        self.instances.append((obj, T, materials if materials is not None else [material], face_material))

    def to_product(self, R, ctx, require_emissive=False, accel=None):
        s = R.Scene(ctx)
        if accel is not None:
            s.set_accel(accel)
        for tex in self.textures:
            s.define_texture_rgba8(tex)
        for v4, idx, t9, ti, uv, ui in self.objects:
            s.define_object(v4, idx, tbns=t9, tbn_indices=ti, tex_coords=uv, tex_indices=ui)
        for obj, T, mats, fm in self.instances:
            if fm is None:
                s.add_instance(obj, T, mats[0])
            else:
                s.add_instance_per_face(obj, T, mats, fm)
        s.build(require_emissive=require_emissive)
        return s

    def to_oracle(self, O):
        s = O.Scene()
        for tex in self.textures:
            s.add_texture(tex)
        for v4, idx, t9, ti, uv, ui in self.objects:
            s.add_object(v4, idx, t9, ti, uv, ui)
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


# ---------------------------------------------------------------------------------------------------
# Textured room: the Cornell walls with UVs and tangent frames, seeded procedural textures (albedo with
# transparent and half-transparent cells, tangent-space normal map, smooth height map, tint), and every
# texture stage on every material: Disney floor (albedo + alpha, bump map, normal map, UVs x2 so they
# wrap), Lambertian back wall (tint + normal map), metal left wall (tint + normal map), Lambertian right
# wall (albedo + alpha, so paths pass through its transparent cells), ceiling textured without UVs
# (samples UV (0, 0)), a bump-mapped Lambertian box, a dielectric box (tint + normal map) and a textured
# Disney sphere with spherical UVs.

def textured_quad(corner, e1, e2, uv_scale=1.0):
    """Quad with UVs (0,0), (s,0), (s,s), (0,s) and the tangent frame T = e1, B = e2, N = e1 x e2."""
    v, i = quad(corner, e1, e2)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32) * uv_scale
    t = np.asarray(e1, np.float64) / np.linalg.norm(e1)
    b = np.asarray(e2, np.float64) / np.linalg.norm(e2)
    n = np.cross(t, b)
    tbn = np.tile(np.concatenate([t, b, n / np.linalg.norm(n)]).astype(np.float32), (4, 1))
    return v, i, tbn, uv


def merge_quads(quads):
    vs, idx, tbns, uvs = [], [], [], []
    base = 0
    for v, i, t, u in quads:
        vs.append(v)
        idx.append(i + base)
        tbns.append(t)
        uvs.append(u)
        base += len(v)
    i = np.concatenate(idx).astype(np.uint32)
    return np.concatenate(vs), i, np.concatenate(tbns), i.copy(), np.concatenate(uvs), i.copy()


def textured_box(uv_scale=1.0):
    """Unit cube as six textured quads (outward normals)."""
    h = 0.5
    faces = [((-h, -h, h), (1, 0, 0), (0, 1, 0)), ((h, -h, -h), (-1, 0, 0), (0, 1, 0)),
             ((h, -h, h), (0, 0, -1), (0, 1, 0)), ((-h, -h, -h), (0, 0, 1), (0, 1, 0)),
             ((-h, h, h), (1, 0, 0), (0, 0, -1)), ((-h, -h, -h), (1, 0, 0), (0, 0, 1))]
    return merge_quads([textured_quad(c, a, b, uv_scale) for c, a, b in faces])


def room_textures(seed: int = 1):
    rng = np.random.default_rng(seed)
    # 0: albedo checker 32x32 in 4x4 cells, alpha 0 / 128 / 255 per cell
    cells = rng.integers(0, 6, (8, 8))
    col = np.where((np.add.outer(np.arange(8), np.arange(8)) % 2)[..., None] == 0, [230, 200, 150], [60, 110, 190])
    albedo = np.zeros((32, 32, 4), np.uint8)
    albedo[..., :3] = np.kron(col, np.ones((4, 4, 1))).astype(np.uint8)
    alpha = np.where(cells == 0, 0, np.where(cells == 1, 128, 255))
    albedo[..., 3] = np.kron(alpha, np.ones((4, 4))).astype(np.uint8)
    # 1: normal map 24x24: tilted tangent-space normals
    nx, ny = rng.uniform(-0.6, 0.6, (2, 24, 24))
    n = np.stack([nx, ny, np.ones_like(nx)], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    nmap = np.zeros((24, 24, 4), np.uint8)
    nmap[..., :3] = np.clip(np.round((n * 0.5 + 0.5) * 255), 0, 255).astype(np.uint8)
    nmap[..., 3] = 255
    # 2: height map 32x32 (red channel): smooth bumps plus noise
    y, x = np.mgrid[0:32, 0:32] / 32.0
    hgt = 0.5 + 0.35 * np.sin(2 * np.pi * 2 * x) * np.cos(2 * np.pi * 3 * y) + rng.uniform(-0.1, 0.1, (32, 32))
    height = np.zeros((32, 32, 4), np.uint8)
    height[..., 0] = np.clip(np.round(hgt * 255), 0, 255).astype(np.uint8)
    height[..., 1:3] = 40
    height[..., 3] = 255
    # 3: tint 16x16
    tint = np.concatenate([rng.integers(90, 256, (16, 16, 3)), np.full((16, 16, 1), 255)], -1).astype(np.uint8)
    return [albedo, nmap, height, tint]


def textured_room(R, seed: int = 1) -> SceneDesc:
    d = SceneDesc()
    for t in room_textures(seed):
        d.add_texture(t)
    ALB, NRM, HGT, TNT = 0, 1, 2, 3
    M = R.Material
    one = dict(specular_tint=(1, 1, 1), sheen_tint=(1, 1, 1))
    floor = textured_quad((-1, -1, 1), (2, 0, 0), (0, 0, -2), 2.0)
    back = textured_quad((-1, -1, -1), (2, 0, 0), (0, 2, 0))
    left = textured_quad((-1, -1, 1), (0, 0, -2), (0, 2, 0))
    right = textured_quad((1, -1, -1), (0, 0, 2), (0, 2, 0))
    for (v, i, t, uv), mat in [
        (floor, M(material_idx=3, albedo=(0.9, 0.9, 0.9), roughness=0.5, texture_id=ALB, normal_map_id=NRM,
                  bump_map_id=HGT, **one)),
        (back, M(material_idx=0, albedo=(0.8, 0.8, 0.8), texture_id=TNT, normal_map_id=NRM)),
        (left, M(material_idx=1, albedo=(0.9, 0.6, 0.5), roughness=0.25, texture_id=TNT, normal_map_id=NRM)),
        (right, M(material_idx=0, albedo=(0.3, 0.8, 0.3), texture_id=ALB)),
    ]:
        d.add_instance(d.add_object(v, i, t, i, uv, i), None, mat)
    cv, ci = quad((-1, 1, -1), (2, 0, 0), (0, 0, 2))   # ceiling, no UVs: samples UV (0, 0)
    d.add_instance(d.add_object(cv, ci), None, M(material_idx=0, albedo=(0.8, 0.8, 0.8), texture_id=TNT))
    bv, bi, bt, bti, buv, bui = textured_box(1.5)
    box = d.add_object(bv, bi, bt, bti, buv, bui)
    d.add_instance(box, translate(-0.4, -0.55, -0.35) @ rotate_y(25.0) @ scale(0.5, 0.9, 0.5),
                   M(material_idx=0, albedo=(0.85, 0.85, 0.85), bump_map_id=HGT))
    d.add_instance(box, translate(0.45, -0.75, 0.3) @ rotate_y(-20.0) @ scale(0.45, 0.5, 0.45),
                   M(material_idx=2, albedo=(0.95, 0.95, 0.95), ior=1.5, absorption=0.8, roughness=0.02,
                     texture_id=TNT, normal_map_id=NRM))
    v, i, tbn, ti = sphere_tbn(3, 0.0, seed, R)
    p = v[:, :3] / np.linalg.norm(v[:, :3], axis=1, keepdims=True)
    uv = np.stack([np.arctan2(p[:, 2], p[:, 0]) / (2 * np.pi) + 0.5, np.arccos(np.clip(p[:, 1], -1, 1)) / np.pi], 1)
    sph = d.add_object(v, i, tbn, ti, uv.astype(np.float32), i)
    d.add_instance(sph, translate(0.1, 0.25, -0.2) @ scale(0.28, 0.28, 0.28),
                   M(material_idx=3, albedo=(1, 1, 1), roughness=0.35, metallic=0.4, clearcoat=0.5, texture_id=ALB,
                     normal_map_id=NRM, interp_normals=True, **one))
    lv, li = quad((-0.25, 0.999, -0.2), (0.5, 0, 0), (0, 0, 0.4))
    d.add_instance(d.add_object(lv, li), None,
                   M(material_idx=0, albedo=(0.78, 0.78, 0.78), emission=CORNELL_LIGHT, cull_backface=True))
    return d


def rotate_axis(axis, deg):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    t = np.radians(deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R3 = np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * (K @ K)
    m = np.eye(4)
    m[:3, :3] = R3
    return m


def instanced_field(R, n: int = 24, seed: int = 7) -> SceneDesc:
    """One displaced sphere model (level 3, with TBNs) instanced n times with seeded rotations, anisotropic
    scales and translations inside the Cornell room, each with its own material; the room and its light
    stay single instances.  Instancing repeats the sphere enough that the automatic choice builds two
    levels."""
    d = cornell(R, seed)
    v, i, tbn, ti = sphere_tbn(3, 0.08, seed, R)
    sph = d.add_object(v, i, tbn, ti)
    u = uniform(9 * n, seed + 1).reshape(n, 9)
    for k in range(n):
        r = u[k]
        T = (translate(-0.75 + 1.5 * r[0], -0.8 + 1.4 * r[1], -0.7 + 1.3 * r[2]) @ rotate_axis(r[3:6] - 0.5, 360 * r[6])
             @ scale(0.08 + 0.12 * r[7], 0.08 + 0.12 * r[8], 0.1))
        if k % 3 == 0:
            m = R.Material(material_idx=1, albedo=(0.9, 0.8, 0.6), roughness=0.3 * r[0])
        elif k % 3 == 1:
            m = R.Material(material_idx=2, albedo=(0.9, 0.95, 0.9), ior=1.45, absorption=r[1], roughness=0.02)
        else:
            m = R.Material(material_idx=3, albedo=tuple(r[0:3]), roughness=0.2 + 0.6 * r[4], metallic=r[5],
                           specular_tint=(1, 1, 1), sheen_tint=(1, 1, 1), interp_normals=True)
        d.add_instance(sph, T, m)
    # two more instances with per-face materials (Lambertian / Disney palette by face)
    nf = i.size // 3
    pal = [R.Material(material_idx=0, albedo=(0.8, 0.3, 0.2)), R.Material(material_idx=0, albedo=(0.2, 0.6, 0.8)),
           R.Material(material_idx=3, albedo=(0.9, 0.9, 0.3), roughness=0.4, specular_tint=(1, 1, 1),
                      sheen_tint=(1, 1, 1))]
    for k, pos in enumerate([(-0.45, 0.45, 0.3), (0.5, 0.5, -0.3)]):
        face = (uniform(nf, seed + 20 + k) * len(pal)).astype(np.uint32)
        d.add_instance(sph, translate(*pos) @ scale(0.15, 0.15, 0.15), materials=pal, face_material=face)
    return d


def instance_models(d: SceneDesc):
    """Object-space triangles (9 floats each) of every object of a scene description."""
    return [np.ascontiguousarray(v4[np.asarray(idx).reshape(-1, 3)][:, :, :3].reshape(-1, 9), np.float32)
            for v4, idx, *_ in d.objects]
