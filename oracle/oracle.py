"""ORACLE — test infrastructure only.  ctypes binding of `oracle/_build/liboracle.so` (the CPU restatement).

Used by tests/ (as the checker), by `__graft_entry__.smoke()` and by bench.py's CPU-baseline leg.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

RAY_DTYPE = np.dtype([("org", np.float32, 3), ("tmin", np.float32), ("dir", np.float32, 3), ("tmax", np.float32)])
HIT_DTYPE = np.dtype([("prim", np.uint32), ("t", np.float32), ("u", np.float32), ("v", np.float32)])
HIT64_DTYPE = np.dtype([("prim", np.uint32), ("pad", np.uint32), ("t", np.float64), ("u", np.float64),
                        ("v", np.float64)])
MISS = 0xFFFFFFFF

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        P, U32, U64, I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
        L.oracle_hw_threads.restype = I
        L.oracle_rng.argtypes = [U32, I, P, P, P]
        L.oracle_bvh_build.restype = P
        L.oracle_bvh_build.argtypes = [P, U64]
        L.oracle_bvh_destroy.argtypes = [P]
        L.oracle_raycast.argtypes = [P, P, U64, I, I, I, P, P]
        L.oracle_raycast_brute.argtypes = [P, U64, P, U64, I, I, I, P, P]
        L.oracle_test_triangle.argtypes = [P, P, P]
        L.oracle_test_triangle.restype = I
        _setup_shading(L)
        _lib = L
    return _lib


def _setup_shading(L) -> None:
    """Signatures of the shading/post-process entry points (added by later oracle modules)."""
    for name, (res, args) in _SHADING_SIGS.items():
        if hasattr(L, name):
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args


_SHADING_SIGS: dict = {}


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def hw_threads() -> int:
    return int(lib().oracle_hw_threads())


def rng(seed: int, n: int):
    """Outputs of `random()` (shaders/raytrace/shaderCommon.h.glsl:39-45) from state `seed`:
    (words u32, float32 values, float64 values)."""
    w = np.zeros(n, np.uint32)
    f = np.zeros(n, np.float32)
    d = np.zeros(n, np.float64)
    lib().oracle_rng(seed & 0xFFFFFFFF, n, _p(w), _p(f), _p(d))
    return w, f, d


_SHADING_SIGS["oracle_icosphere_counts"] = (None, [C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)])
_SHADING_SIGS["oracle_gen_icosphere"] = (None, [C.c_uint32, C.c_float, C.c_uint64, C.c_void_p, C.c_void_p])
_SHADING_SIGS["oracle_gen_rays"] = (None, [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_float, C.c_uint64,
                                           C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p])


def icosphere(level: int, amplitude: float = 0.0, seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """The synthetic displaced icosphere (oracle_gen.cpp): vertices (N, 4) and indices (3M,)."""
    nv, nt = C.c_uint64(), C.c_uint64()
    lib().oracle_icosphere_counts(level, C.byref(nv), C.byref(nt))
    v = np.zeros((nv.value, 4), np.float32)
    i = np.zeros(3 * nt.value, np.uint32)
    lib().oracle_gen_icosphere(level, float(amplitude), seed, _p(v), _p(i))
    return v, i


def raycast_rays(width: int, height: int, cam_pos, cam_target, fovy_degrees: float, n_random: int, box_min, box_max,
                 seed: int = 1) -> np.ndarray:
    """The synthetic ray set (oracle_gen.cpp): camera rays then box rays, as RAY_DTYPE records."""
    out = np.zeros(width * height + n_random, RAY_DTYPE)
    f3 = lambda a: np.ascontiguousarray(a, np.float32).reshape(3)
    cp, ct, lo, hi = f3(cam_pos), f3(cam_target), f3(box_min), f3(box_max)
    lib().oracle_gen_rays(width, height, _p(cp), _p(ct), float(fovy_degrees), n_random, _p(lo), _p(hi), seed, _p(out))
    return out


_SHADING_SIGS["oracle_bvh8_raycast"] = (None, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int,
                                               C.c_int, C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)])


def bvh8_raycast(nodes: np.ndarray, tris: np.ndarray, rays: np.ndarray, any_hit: bool = False, threads: int = 0):
    """Traverses the product's exported BVH8 (node bytes, 48-byte triangle records) on the CPU.  Returns
    (hits with unrefined t/u/v, node visits, triangle tests)."""
    nb = np.ascontiguousarray(nodes).view(np.uint8).reshape(-1)
    tb = np.ascontiguousarray(tris).view(np.float32).reshape(-1)
    r = np.ascontiguousarray(rays)
    hits = np.zeros(r.shape[0], HIT_DTYPE)
    nv, nt = C.c_uint64(0), C.c_uint64(0)
    lib().oracle_bvh8_raycast(_p(nb), nb.size // 80, _p(tb), _p(r), r.shape[0], int(any_hit), threads, _p(hits),
                              C.byref(nv), C.byref(nt))
    return hits, nv.value, nt.value


_SHADING_SIGS.update({
    "oracle_instanced_new": (C.c_void_p, []),
    "oracle_instanced_free": (None, [C.c_void_p]),
    "oracle_instanced_add_model": (C.c_uint32, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "oracle_instanced_add_instance": (None, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
    "oracle_instanced_raycast": (None, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_int, C.c_void_p]),
    "oracle_bvh8_two_level_raycast": (None, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_uint64, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_uint64),
                                             C.POINTER(C.c_uint64)]),
})


class InstancedScene:
    """The oracle's two-level restatement: models in object space (9 floats per triangle), instances as
    (model, world-to-object 3x4 row-major matrix, first global triangle id)."""

    def __init__(self):
        self._h = lib().oracle_instanced_new()

    def __del__(self):
        try:
            if self._h:
                lib().oracle_instanced_free(self._h)
                self._h = None
        except Exception:
            pass

    def add_model(self, tris9) -> int:
        t = np.ascontiguousarray(tris9, np.float32).reshape(-1, 9)
        return int(lib().oracle_instanced_add_model(self._h, _p(t), t.shape[0]))

    def add_instance(self, model: int, inv12, first_prim: int) -> None:
        m = np.ascontiguousarray(inv12, np.float32).reshape(12)
        lib().oracle_instanced_add_instance(self._h, model, _p(m), first_prim)

    def raycast(self, rays: np.ndarray, any_hit: bool = False, threads: int = 0) -> np.ndarray:
        r = np.ascontiguousarray(rays)
        hits = np.zeros(r.shape[0], HIT_DTYPE)
        lib().oracle_instanced_raycast(self._h, _p(r), r.shape[0], int(any_hit), threads, _p(hits))
        return hits


def bvh8_two_level_raycast(nodes, tris, refs, inst_records, rays, any_hit: bool = False, threads: int = 0):
    """Traverses an exported two-level BVH8 on the CPU: (hits with unrefined t/u/v, visits, tests)."""
    nb = np.ascontiguousarray(nodes).view(np.uint8).reshape(-1)
    tb = np.ascontiguousarray(tris).view(np.float32).reshape(-1)
    rf = np.ascontiguousarray(refs, np.uint32)
    ib = np.ascontiguousarray(inst_records).view(np.uint8).reshape(-1)
    r = np.ascontiguousarray(rays)
    hits = np.zeros(r.shape[0], HIT_DTYPE)
    nv, nt = C.c_uint64(0), C.c_uint64(0)
    lib().oracle_bvh8_two_level_raycast(_p(nb), nb.size // 80, _p(tb), _p(rf), _p(ib), _p(r), r.shape[0], int(any_hit),
                                        threads, _p(hits), C.byref(nv), C.byref(nt))
    return hits, nv.value, nt.value


_SHADING_SIGS["oracle_kat"] = (None, [C.c_int, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p])
_SHADING_SIGS["oracle_kat8"] = (None, [C.c_int, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p])
KAT_OFFSET, KAT_GGX_VNDF, KAT_EVAL_DISNEY, KAT_RANDOM, KAT_OFFSET_DIELECTRIC, KAT_SAMPLE_DISNEY = 0, 1, 2, 3, 4, 5
KAT_DIFFUSE_REFLECTION, KAT_RANDOM_UNIT_VEC, KAT_REFLECTANCE, KAT_PDFS = 6, 7, 10, 14


def kat(kind: int, records: np.ndarray, precision: int = 32) -> np.ndarray:
    """Single shading functions on 40-float case records (see oracle_kat.cpp): (n, 4) float64."""
    r = np.ascontiguousarray(records, np.float32).reshape(-1, 40)
    out = np.zeros((r.shape[0], 4), np.float64)
    lib().oracle_kat(kind, _p(r), r.shape[0], precision, _p(out))
    return out


def kat8(kind: int, records: np.ndarray, precision: int = 32) -> np.ndarray:
    """The same on 8 outputs per case (see oracle_kat.cpp): (n, 8) float64."""
    r = np.ascontiguousarray(records, np.float32).reshape(-1, 40)
    out = np.zeros((r.shape[0], 8), np.float64)
    lib().oracle_kat8(kind, _p(r), r.shape[0], precision, _p(out))
    return out


class Bvh:
    def __init__(self, tris9: np.ndarray):
        self.tris = np.ascontiguousarray(tris9, dtype=np.float32).reshape(-1, 9)
        self._h = lib().oracle_bvh_build(_p(self.tris), self.tris.shape[0])

    def close(self):
        if self._h:
            lib().oracle_bvh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def raycast(self, rays: np.ndarray, any_hit: bool = False, precision: int = 32, threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays)
        n = rays.shape[0]
        if precision == 64:
            out = np.zeros(n, HIT64_DTYPE)
            lib().oracle_raycast(self._h, _p(rays), n, int(any_hit), 64, threads, None, _p(out))
        else:
            out = np.zeros(n, HIT_DTYPE)
            lib().oracle_raycast(self._h, _p(rays), n, int(any_hit), 32, threads, _p(out), None)
        return out


def raycast_brute(tris9: np.ndarray, rays: np.ndarray, any_hit: bool = False, precision: int = 32,
                  threads: int = 0) -> np.ndarray:
    tris9 = np.ascontiguousarray(tris9, dtype=np.float32).reshape(-1, 9)
    rays = np.ascontiguousarray(rays)
    n = rays.shape[0]
    if precision == 64:
        out = np.zeros(n, HIT64_DTYPE)
        lib().oracle_raycast_brute(_p(tris9), tris9.shape[0], _p(rays), n, int(any_hit), 64, threads, None, _p(out))
    else:
        out = np.zeros(n, HIT_DTYPE)
        lib().oracle_raycast_brute(_p(tris9), tris9.shape[0], _p(rays), n, int(any_hit), 32, threads, _p(out), None)
    return out


class OMaterial(C.Structure):
    """Same field order as the C ABI's reina_material (src/scene/Scene.h:21-46)."""
    _fields_ = [
        ("material_idx", C.c_uint32), ("texture_id", C.c_int32), ("normal_map_id", C.c_int32),
        ("bump_map_id", C.c_int32), ("albedo", C.c_float * 3), ("emission", C.c_float * 3),
        ("roughness", C.c_float), ("ior", C.c_float), ("interp_normals", C.c_uint32),
        ("absorption", C.c_float), ("cull_backface", C.c_uint32), ("anisotropic", C.c_float),
        ("subsurface", C.c_float), ("clearcoat_gloss", C.c_float), ("sheen_tint", C.c_float * 3),
        ("specular_tint", C.c_float * 3), ("metallic", C.c_float), ("clearcoat", C.c_float),
        ("specular_transmission", C.c_float), ("sheen", C.c_float),
    ]

    @classmethod
    def from_obj(cls, m) -> "OMaterial":
        o = cls()
        for name, _ in cls._fields_:
            v = getattr(m, name)
            if isinstance(v, (tuple, list, np.ndarray)):
                arr = getattr(o, name)
                for i in range(3):
                    arr[i] = float(v[i])
            elif isinstance(v, bool):
                setattr(o, name, int(v))
            else:
                setattr(o, name, v)
        return o


class OPush(C.Structure):
    """polyglot/raytrace.h:43-54."""
    _fields_ = [("invView", C.c_float * 16), ("invProjection", C.c_float * 16), ("sampleBatch", C.c_uint32),
                ("totalEmissiveWeight", C.c_float), ("focusDist", C.c_float), ("defocusMultiplier", C.c_float),
                ("directClamp", C.c_float), ("indirectClamp", C.c_float), ("samplesPerPixel", C.c_uint32),
                ("maxBounces", C.c_uint32)]

    @classmethod
    def copy_of(cls, pc) -> "OPush":
        o = cls()
        C.memmove(C.byref(o), C.byref(pc), C.sizeof(cls))
        return o


class ORenderOptions(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("seed", C.c_uint32), ("env_mode", C.c_uint32), ("env_color", C.c_float * 3),
                ("x0", C.c_uint32), ("y0", C.c_uint32), ("x1", C.c_uint32), ("y1", C.c_uint32)]


_SHADING_SIGS.update({
    "oracle_scene_new": (C.c_void_p, []),
    "oracle_scene_free": (None, [C.c_void_p]),
    "oracle_scene_add_object": (C.c_uint32, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p,
                                             C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p,
                                             C.c_uint64]),
    "oracle_scene_add_texture": (C.c_uint32, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32]),
    "oracle_scene_add_instance": (None, [C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(OMaterial), C.c_uint32,
                                         C.c_void_p]),
    "oracle_scene_finalize": (None, [C.c_void_p]),
    "oracle_scene_emissive_weight": (C.c_float, [C.c_void_p]),
    "oracle_render": (None, [C.c_void_p, C.POINTER(OPush), C.POINTER(ORenderOptions), C.c_uint32, C.c_uint32, C.c_int,
                             C.c_int, C.c_void_p, C.c_void_p]),
    "oracle_seed_hash": (C.c_uint32, [C.c_uint32, C.c_uint32, C.c_uint32]),
})


class Scene:
    """The oracle's own scene: objects, instances (column-major transforms) and materials."""

    def __init__(self):
        self._h = lib().oracle_scene_new()
        self._keep = []

    def __del__(self):
        try:
            if self._h:
                lib().oracle_scene_free(self._h)
                self._h = None
        except Exception:
            pass

    def add_object(self, v4, idx, tbn9=None, tbn_idx=None, uv=None, uv_idx=None) -> int:
        v = np.ascontiguousarray(v4, np.float32).reshape(-1, 4)
        i = np.ascontiguousarray(idx, np.uint32).reshape(-1)
        t = None if tbn9 is None else np.ascontiguousarray(tbn9, np.float32).reshape(-1, 9)
        ti = None if tbn_idx is None else np.ascontiguousarray(tbn_idx, np.uint32).reshape(-1)
        u = None if uv is None else np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        ui = None if uv_idx is None else np.ascontiguousarray(uv_idx, np.uint32).reshape(-1)
        return int(lib().oracle_scene_add_object(self._h, _p(v), v.shape[0], _p(i), i.size, _p(t),
                                                 0 if t is None else t.shape[0], _p(ti), 0 if ti is None else ti.size,
                                                 _p(u), 0 if u is None else u.shape[0], _p(ui),
                                                 0 if ui is None else ui.size))

    def add_texture(self, rgba8) -> int:
        """An RGBA8 texture (H, W, 4) uint8, row 0 at v = 0."""
        a = np.ascontiguousarray(rgba8, np.uint8)
        self._keep.append(a)
        return int(lib().oracle_scene_add_texture(self._h, _p(a), a.shape[1], a.shape[0]))

    def add_instance(self, obj: int, transform16, materials: list, face_material=None) -> None:
        T = np.ascontiguousarray(transform16, np.float32).reshape(16)
        arr = (OMaterial * len(materials))(*[OMaterial.from_obj(m) for m in materials])
        fm = None if face_material is None else np.ascontiguousarray(face_material, np.uint32)
        lib().oracle_scene_add_instance(self._h, obj, _p(T), arr, len(materials), _p(fm))

    def finalize(self) -> None:
        lib().oracle_scene_finalize(self._h)

    @property
    def emissive_weight(self) -> float:
        return float(lib().oracle_scene_emissive_weight(self._h))

    def render(self, pc, width: int, height: int, mode: int = 0, seed: int = 1, env_mode: int = 0,
               env_color=(0.0, 0.0, 0.0), window=None, precision: int = 32, threads: int = 0, accum=None,
               want_samples: bool = False):
        o = ORenderOptions(mode, seed, env_mode)
        for k in range(3):
            o.env_color[k] = float(env_color[k])
        x0, y0, x1, y1 = window if window is not None else (0, 0, width, height)
        o.x0, o.y0, o.x1, o.y1 = x0, y0, x1, y1
        if accum is None:
            accum = np.zeros((height, width, 4), np.float32)
        accum = np.ascontiguousarray(accum, np.float32)
        samples = np.zeros((width * height, pc.samplesPerPixel, 3), np.float32) if want_samples else None
        push = OPush.copy_of(pc)
        lib().oracle_render(self._h, C.byref(push), C.byref(o), width, height, precision, threads, _p(accum),
                            _p(samples))
        return accum, samples


_SHADING_SIGS["oracle_postprocess"] = (None, [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                              C.c_float, C.c_int, C.c_void_p, C.c_void_p])


def postprocess(accum: np.ndarray, radius=5.0, threshold=1.0, intensity=0.05, exposure=1.0, precision=32):
    """Bloom + ACES tone map of accum (H, W, 4) -> (rgba8 (H, W, 4), combined HDR (H, W, 4))."""
    accum = np.ascontiguousarray(accum, np.float32)
    H, W = accum.shape[:2]
    out = np.zeros((H, W, 4), np.uint8)
    comb = np.zeros((H, W, 4), np.float32)
    lib().oracle_postprocess(_p(accum), W, H, radius, threshold, intensity, exposure, precision, _p(out), _p(comb))
    return out, comb


def seed_hash(pixel: int, sample: int, seed: int) -> int:
    return int(lib().oracle_seed_hash(pixel, sample, seed))


def test_triangle(tri9: np.ndarray, ray) -> tuple[bool, np.ndarray]:
    tri = np.ascontiguousarray(tri9, dtype=np.float32).reshape(9)
    r = np.ascontiguousarray(np.asarray(ray).reshape(1)).view(RAY_DTYPE)
    out = np.zeros(1, HIT_DTYPE)
    ok = lib().oracle_test_triangle(_p(tri), _p(r), _p(out))
    return bool(ok), out[0]
