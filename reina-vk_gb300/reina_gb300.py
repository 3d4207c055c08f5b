"""Python mirror of the trace path's C ABI (include/reina/reina_c.h) over ctypes.

It follows the reference's scene API one for one — `Scene.define_object` (src/scene/Scene.h:78),
`Scene.add_instance` (Scene.h:114), `Scene.build` (Scene.h:116), `Scene.emissive_weight`
(Scene.h:118) — plus the ray-cast entry points that replace traceRayEXT.  Errors raise `ReinaError`
carrying the library's status code and message, where the reference throws std::runtime_error.

The shared library `_build/libreina_gb300.so` must have been built (build.py); there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from dataclasses import dataclass, field, fields
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libreina_gb300.so"

REINA_OK = 0
REINA_ERR_INVALID = -1
REINA_ERR_CUDA = -2
REINA_ERR_OOM = -3
REINA_ERR_STATE = -4
REINA_ERR_IO = -5
REINA_ERR_NO_EMISSIVE = -6
REINA_ERR_DEVICE = -7
REINA_ERR_BUDGET = -8

RAY_CLOSEST = 0
RAY_ANY = 1
MISS = 0xFFFFFFFF
ACCEL_AUTO, ACCEL_FLAT, ACCEL_TWO_LEVEL = 0, 1, 2
REFILL_GRID = 255   # tuning.refill: one thread per ray (grid form); 0 = the default cooperative form

RAY_DTYPE = np.dtype([("org", np.float32, 3), ("tmin", np.float32), ("dir", np.float32, 3), ("tmax", np.float32)])
HIT_DTYPE = np.dtype([("prim", np.uint32), ("t", np.float32), ("u", np.float32), ("v", np.float32)])
NODE_BYTES = 80
TRI_BYTES = 48


class ReinaError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class _ModelData(C.Structure):
    _fields_ = [
        ("vertices", C.POINTER(C.c_float)), ("vertex_count", C.c_uint64),
        ("indices", C.POINTER(C.c_uint32)), ("index_count", C.c_uint64),
        ("tbns", C.POINTER(C.c_float)), ("tbn_count", C.c_uint64),
        ("tbn_indices", C.POINTER(C.c_uint32)), ("tbn_index_count", C.c_uint64),
        ("tex_coords", C.POINTER(C.c_float)), ("tex_coord_count", C.c_uint64),
        ("tex_indices", C.POINTER(C.c_uint32)), ("tex_index_count", C.c_uint64),
    ]


class _Material(C.Structure):
    _fields_ = [
        ("material_idx", C.c_uint32), ("texture_id", C.c_int32), ("normal_map_id", C.c_int32),
        ("bump_map_id", C.c_int32), ("albedo", C.c_float * 3), ("emission", C.c_float * 3),
        ("roughness", C.c_float), ("ior", C.c_float), ("interp_normals", C.c_uint32),
        ("absorption", C.c_float), ("cull_backface", C.c_uint32), ("anisotropic", C.c_float),
        ("subsurface", C.c_float), ("clearcoat_gloss", C.c_float), ("sheen_tint", C.c_float * 3),
        ("specular_tint", C.c_float * 3), ("metallic", C.c_float), ("clearcoat", C.c_float),
        ("specular_transmission", C.c_float), ("sheen", C.c_float),
    ]


class _SceneStats(C.Structure):
    _fields_ = [
        ("triangle_count", C.c_uint64), ("instance_count", C.c_uint64), ("node_count", C.c_uint64),
        ("node_bytes", C.c_uint64), ("triangle_bytes", C.c_uint64), ("device_bytes", C.c_uint64),
        ("max_depth", C.c_uint32), ("leaf_triangles_max", C.c_uint32), ("build_seconds", C.c_double),
        ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3), ("two_level", C.c_uint32),
        ("blas_count", C.c_uint32), ("emissive_seconds", C.c_double), ("bvh_device", C.c_uint32),
        ("pad0", C.c_uint32), ("bvh_kernel_seconds", C.c_double),
    ]


class _CtxOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_uint32)]


class _Tuning(C.Structure):
    _fields_ = [("refill", C.c_uint32), ("wave_paths", C.c_uint32), ("batch_flags", C.c_uint32),
                ("trace_block", C.c_uint32), ("trace_stack", C.c_uint32), ("trace_order", C.c_uint32),
                ("wave_lanes", C.c_uint32), ("wave_refill", C.c_uint32)]


TUNING_FIELDS = ("refill", "wave_paths", "batch_flags", "trace_block", "trace_stack", "trace_order", "wave_lanes",
                 "wave_refill")
ORDER_INPUT, ORDER_COHERENT = 0, 1


DEFAULT_WAVE_PATHS = 2097152
DEFAULT_WAVE_LANES = 8
SERVER_WAVE_PATHS = 2097152
SERVER_WAVE_LANES = 4
SERVER_DEFAULT_AGING = 0.03
BATCH_NO_GRAPHS = 1
BATCH_FAIR_SHARE = 2


# InstanceProperties (polyglot.h), 120 bytes.
INSTANCE_PROPERTIES_DTYPE = np.dtype([
    ("indicesOffset", "<u4"), ("albedo", "<f4", 3), ("emission", "<f4", 3), ("tbnsIndicesOffset", "<u4"),
    ("texIndicesOffset", "<u4"), ("roughness", "<f4"), ("ior", "<f4"), ("interpNormals", "<u4"),
    ("absorption", "<f4"), ("textureID", "<i4"), ("normalMapTexID", "<i4"), ("bumpMapTexID", "<i4"),
    ("cullBackface", "<u4"), ("anisotropic", "<f4"), ("subsurface", "<f4"), ("clearcoatGloss", "<f4"),
    ("sheenTint", "<f4", 3), ("specularTint", "<f4", 3), ("metallic", "<f4"), ("clearcoat", "<f4"),
    ("specularTransmission", "<f4"), ("sheen", "<f4")])


# EmissiveInstanceData (polyglot.h), 112 bytes.
EMISSIVE_INSTANCE_DTYPE = np.dtype([
    ("transform", "<f4", 16), ("materialOffset", "<u4"), ("cdfRangeStart", "<u4"), ("cdfRangeEnd", "<u4"),
    ("indexOffset", "<u4"), ("emission", "<f4", 3), ("weight", "<f4"), ("area", "<f4"), ("cullBackface", "<u4"),
    ("padding", "<f4", 2)])
EMISSIVE_HOST, EMISSIVE_DEVICE = 0, 1
BVH_HOST, BVH_DEVICE = 0, 1


class RtPushConsts(C.Structure):
    """polyglot/raytrace.h:43-54 (160 bytes; matrices column-major)."""
    _fields_ = [("invView", C.c_float * 16), ("invProjection", C.c_float * 16), ("sampleBatch", C.c_uint32),
                ("totalEmissiveWeight", C.c_float), ("focusDist", C.c_float), ("defocusMultiplier", C.c_float),
                ("directClamp", C.c_float), ("indirectClamp", C.c_float), ("samplesPerPixel", C.c_uint32),
                ("maxBounces", C.c_uint32)]


class RenderOptions(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("mode", C.c_uint32), ("seed", C.c_uint32),
                ("env_mode", C.c_uint32), ("env_color", C.c_float * 3), ("flags", C.c_uint32)]


RENDER_MEGAKERNEL = 1
RENDER_PASS_BY_PASS = 2


class BloomPushConsts(C.Structure):
    """polyglot/bloom.h:4-8."""
    _fields_ = [("radius", C.c_float), ("threshold", C.c_float), ("intensity", C.c_float)]


class TonemappingPushConsts(C.Structure):
    """polyglot/tonemapping.h:4-6."""
    _fields_ = [("exposure", C.c_float)]


class _RenderStats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("seconds", C.c_double),
                ("nodes_visited", C.c_uint64), ("triangles_tested", C.c_uint64), ("shadow_nodes_visited", C.c_uint64),
                ("shadow_triangles_tested", C.c_uint64), ("shaded_hits", C.c_uint64)]


def _stats_dict(st: "_RenderStats") -> dict:
    return {f[0]: getattr(st, f[0]) for f in _RenderStats._fields_}


class _ServerOptions(C.Structure):
    _fields_ = [("memory_budget_bytes", C.c_uint64), ("max_active_jobs", C.c_uint32), ("wave_paths", C.c_uint32),
                ("flags", C.c_uint32), ("wave_lanes", C.c_uint32), ("aging", C.c_float), ("reserved", C.c_uint32)]


class _Request(C.Structure):
    _fields_ = [("scene_id", C.c_uint32), ("reserved", C.c_uint32), ("image_key", C.c_uint64),
                ("push_consts", RtPushConsts), ("options", RenderOptions), ("accum", C.c_void_p)]


class _RequestStatus(C.Structure):
    _fields_ = [("state", C.c_uint32), ("error", C.c_int32), ("latency_s", C.c_double), ("queue_s", C.c_double),
                ("message", C.c_char * 160)]


_SERVER_STAT_FIELDS = ["submitted", "completed", "failed", "cancelled", "queued", "running", "latency_p50_s",
                       "latency_p99_s", "latency_mean_s", "latency_max_s", "uptime_s", "busy_s",
                       "first_submit_to_last_done_s", "rays", "shadow_rays", "waves", "scene_uploads",
                       "scene_evictions", "image_evictions", "image_restores", "resident_bytes",
                       "peak_resident_bytes", "budget_bytes", "reserved_bytes"]


class _ServerStats(C.Structure):
    _fields_ = [(n, C.c_double if n.endswith("_s") else C.c_uint64) for n in _SERVER_STAT_FIELDS]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = range(5)
SERVER_FIFO = 2
SERVER_SHORTEST = 4
SERVER_FAIR_SHARE = 8


class _TuneResult(C.Structure):
    _fields_ = [("best", _Tuning), ("best_ms", C.c_double), ("default_ms", C.c_double), ("candidates", C.c_uint32),
                ("kind", C.c_uint32), ("tri_bucket", C.c_uint32), ("size_bucket", C.c_uint32)]


TUNE_RAYCAST_CLOSEST, TUNE_RAYCAST_ANY, TUNE_RENDER, TUNE_BATCH = range(4)
AUTOTUNE_OFF, AUTOTUNE_CACHED = 0, 1


class _GltfStats(C.Structure):
    _fields_ = [("meshes", C.c_uint32), ("primitives", C.c_uint32), ("instances", C.c_uint32),
                ("skipped_primitives", C.c_uint32), ("ignored_textures", C.c_uint32)]


CONFIG_MAX_SAVES = 64


class RunConfig(C.Structure):
    """config/config.toml as the reference reads it (reina_config)."""
    _fields_ = [("focus_dist", C.c_float), ("defocus_multiplier", C.c_float), ("samples_per_pixel", C.c_uint32),
                ("max_bounces", C.c_uint32), ("direct_clamp", C.c_float), ("indirect_clamp", C.c_float),
                ("bloom", BloomPushConsts), ("tonemap", TonemappingPushConsts),
                ("save_on_samples_count", C.c_uint32), ("save_on_times_count", C.c_uint32),
                ("save_on_samples", C.c_int64 * CONFIG_MAX_SAVES), ("save_on_times", C.c_double * CONFIG_MAX_SAVES),
                ("width", C.c_uint32), ("height", C.c_uint32), ("seed", C.c_uint32), ("mode", C.c_uint32),
                ("scene_path", C.c_char * 512), ("camera_pos", C.c_float * 3), ("look_at", C.c_float * 3),
                ("fov_degrees", C.c_float)]


class _RenderJob(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("push_consts", RtPushConsts), ("options", RenderOptions),
                ("accum", C.c_void_p), ("samples", C.c_void_p)]


MODE_REINA = 0
MODE_NEE_MIS = 1
ENV_SKY = 0
ENV_CONSTANT = 1


def push_consts(inv_view, inv_proj, sample_batch=0, total_emissive_weight=0.0, focus_dist=1.0, defocus=0.0,
                direct_clamp=100.0, indirect_clamp=10.0, spp=1, max_bounces=8) -> RtPushConsts:
    pc = RtPushConsts()
    for k in range(16):
        pc.invView[k] = float(inv_view[k])
        pc.invProjection[k] = float(inv_proj[k])
    pc.sampleBatch = sample_batch
    pc.totalEmissiveWeight = total_emissive_weight
    pc.focusDist = focus_dist
    pc.defocusMultiplier = defocus
    pc.directClamp = direct_clamp
    pc.indirectClamp = indirect_clamp
    pc.samplesPerPixel = spp
    pc.maxBounces = max_bounces
    return pc


def render_options(width, height, mode=MODE_REINA, seed=1, env_mode=ENV_SKY, env_color=(0.0, 0.0, 0.0),
                   megakernel=False, pass_by_pass=False) -> RenderOptions:
    """reina_render_options.  Default form: the wave engine; megakernel=True: one thread per pixel;
    pass_by_pass=True: the wavefront one sample pass at a time with direct launches."""
    o = RenderOptions(width, height, mode, seed, env_mode)
    for k in range(3):
        o.env_color[k] = float(env_color[k])
    o.flags = (RENDER_MEGAKERNEL if megakernel else 0) | (RENDER_PASS_BY_PASS if pass_by_pass else 0)
    return o


@dataclass
class Material:
    """reina::scene::Material (src/scene/Scene.h:21-46); material_idx 0 Lambertian, 1 metal,
    2 dielectric, 3 Disney."""
    material_idx: int = 0
    texture_id: int = -1
    normal_map_id: int = -1
    bump_map_id: int = -1
    albedo: tuple = (1.0, 1.0, 1.0)
    emission: tuple = (0.0, 0.0, 0.0)
    roughness: float = 0.0
    ior: float = 1.5
    interp_normals: bool = False
    absorption: float = 0.0
    cull_backface: bool = False
    anisotropic: float = 0.0
    subsurface: float = 0.0
    clearcoat_gloss: float = 0.0
    sheen_tint: tuple = (1.0, 1.0, 1.0)
    specular_tint: tuple = (1.0, 1.0, 1.0)
    metallic: float = 0.0
    clearcoat: float = 0.0
    specular_transmission: float = 0.0
    sheen: float = 0.0

    def to_c(self) -> _Material:
        m = _Material()
        for f in fields(self):
            v = getattr(self, f.name)
            if isinstance(v, (tuple, list, np.ndarray)):
                arr = getattr(m, f.name)
                for i in range(3):
                    arr[i] = float(v[i])
            elif isinstance(v, bool):
                setattr(m, f.name, 1 if v else 0)
            else:
                setattr(m, f.name, v)
        return m


_lib = None


def library_path() -> Path:
    return Path(os.environ.get("REINA_GB300_LIB", str(LIB_PATH)))


def load_library() -> C.CDLL:
    """Loads the CUDA library; raises if it has not been built (the trace path has no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise RuntimeError(f"trace-path library not built: {path} (run reina-vk_gb300/build.py)")
    lib = C.CDLL(str(path))
    P, U32, U64, I32, F = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
    sig = {
        "reina_last_error": (C.c_char_p, []),
        "reina_version": (C.c_char_p, []),
        "reina_ctx_create": (I32, [C.POINTER(_CtxOptions), C.POINTER(P)]),
        "reina_ctx_destroy": (None, [P]),
        "reina_ctx_sm_count": (I32, [P]),
        "reina_ctx_set_tuning": (I32, [P, C.POINTER(_Tuning)]),
        "reina_ctx_get_tuning": (I32, [P, C.POINTER(_Tuning)]),
        "reina_scene_create": (I32, [P, C.POINTER(P)]),
        "reina_scene_destroy": (None, [P]),
        "reina_scene_define_object": (I32, [P, C.POINTER(_ModelData), C.POINTER(U32)]),
        "reina_scene_add_instance": (I32, [P, U32, C.POINTER(C.c_float), C.POINTER(_Material)]),
        "reina_scene_add_instance_per_face": (I32, [P, U32, C.POINTER(C.c_float), C.POINTER(_Material), U32,
                                                    C.POINTER(U32)]),
        "reina_scene_build": (I32, [P, U32]),
        "reina_scene_emissive_weight": (F, [P]),
        "reina_scene_get_stats": (I32, [P, C.POINTER(_SceneStats)]),
        "reina_scene_export_bvh": (I32, [P, P, P]),
        "reina_scene_prim_info": (I32, [P, U32, C.POINTER(U32), C.POINTER(U32)]),
        "reina_raycast": (I32, [P, P, P, U64, P, U32]),
        "reina_raycast_device": (I32, [P, P, P, U64, P, U32, P]),
        "reina_raycast_counters": (I32, [P, P, P, U64, U32, C.POINTER(U64), C.POINTER(U64), P]),
        "reina_render": (I32, [P, P, C.POINTER(RtPushConsts), C.POINTER(RenderOptions), P, P, C.POINTER(_RenderStats)]),
        "reina_render_device": (I32, [P, P, C.POINTER(RtPushConsts), C.POINTER(RenderOptions), P, P, P]),
        "reina_render_device_noalloc": (I32, [P, P, C.POINTER(RtPushConsts), C.POINTER(RenderOptions), P, P, P]),
        "reina_render_batch": (I32, [P, C.POINTER(_RenderJob), U32, C.POINTER(_RenderStats)]),
        "reina_scene_define_object_obj": (I32, [P, C.c_char_p, C.POINTER(U32)]),
        "reina_scene_add_gltf": (I32, [P, C.c_char_p, C.POINTER(_GltfStats)]),
        "reina_scene_object_count": (I32, [P, C.POINTER(U32)]),
        "reina_scene_export_object": (I32, [P, U32, P, C.POINTER(U64), P, C.POINTER(U64), P, C.POINTER(U64), P,
                                            C.POINTER(U64)]),
        "reina_config_load": (I32, [C.c_char_p, C.POINTER(RunConfig)]),
        "reina_save_schedule_create": (I32, [C.POINTER(RunConfig), C.POINTER(P)]),
        "reina_save_schedule_destroy": (None, [P]),
        "reina_save_schedule_next": (I32, [P, U64, C.c_double, C.c_char_p, C.c_size_t]),
        "reina_write_png": (I32, [C.c_char_p, P, U32, U32]),
        "reina_scene_define_texture_rgba8": (I32, [P, P, U32, U32, C.POINTER(U32)]),
        "reina_scene_define_texture_file": (I32, [P, C.c_char_p, C.POINTER(U32)]),
        "reina_scene_define_texture_encoded": (I32, [P, P, U64, C.POINTER(U32)]),
        "reina_scene_texture_count": (I32, [P, C.POINTER(U32)]),
        "reina_scene_set_accel": (I32, [P, C.c_int]),
        "reina_scene_set_emissive_build": (I32, [P, U32]),
        "reina_scene_set_bvh_build": (I32, [P, U32, U32, U32]),
        "reina_scene_export_emissive": (I32, [P, P, C.POINTER(U32), P, C.POINTER(U64), P]),
        "reina_device_kat": (I32, [P, C.c_int, P, U64, P]),
        "reina_ctx_device_error": (I32, [P, P, C.POINTER(U32)]),
        "reina_scene_export_two_level": (I32, [P, P, P, C.POINTER(U32), C.POINTER(U32)]),
        "reina_scene_export_properties": (I32, [P, P, U32, C.POINTER(U32)]),
        "reina_scene_export_texture": (I32, [P, U32, C.POINTER(U32), C.POINTER(U32), P, U64]),
        "reina_decode_image": (I32, [P, U64, C.POINTER(U32), C.POINTER(U32), P, U64]),
        "reina_autotune_raycast": (I32, [P, P, P, U64, P, U32, P, C.POINTER(_TuneResult)]),
        "reina_autotune_render": (I32, [P, P, C.POINTER(RtPushConsts), C.POINTER(RenderOptions), C.POINTER(_TuneResult)]),
        "reina_autotune_batch": (I32, [P, C.POINTER(_RenderJob), U32, C.POINTER(_TuneResult)]),
        "reina_autotune_set_mode": (I32, [P, U32]),
        "reina_autotune_lookup": (I32, [P, U32, U64, U64, C.POINTER(_Tuning), C.POINTER(C.c_int32)]),
        "reina_autotune_save": (I32, [P, C.c_char_p]),
        "reina_autotune_load": (I32, [P, C.c_char_p]),
        "reina_server_create": (I32, [P, C.POINTER(_ServerOptions), C.POINTER(P)]),
        "reina_server_destroy": (None, [P]),
        "reina_server_add_scene": (I32, [P, P, C.POINTER(U32)]),
        "reina_server_submit": (I32, [P, C.POINTER(_Request), C.POINTER(U64)]),
        "reina_server_poll": (I32, [P, U64, C.POINTER(_RequestStatus)]),
        "reina_server_wait": (I32, [P, U64, C.c_double, C.POINTER(_RequestStatus)]),
        "reina_server_cancel": (I32, [P, U64]),
        "reina_server_fetch_image": (I32, [P, U64, P, C.POINTER(U32), C.POINTER(U32)]),
        "reina_server_get_stats": (I32, [P, C.POINTER(_ServerStats)]),
        "reina_render_batch_device": (I32, [P, C.POINTER(_RenderJob), U32, P, C.POINTER(_RenderStats)]),
        "reina_postprocess": (I32, [P, P, U32, U32, C.POINTER(BloomPushConsts), C.POINTER(TonemappingPushConsts), P, P]),
        "reina_postprocess_device": (I32, [P, P, U32, U32, C.POINTER(BloomPushConsts),
                                           C.POINTER(TonemappingPushConsts), P, P, P]),
        "reina_camera_matrices": (I32, [P, P, P, F, F, F, F, P, P]),
        "reina_icosphere_counts": (I32, [U32, C.POINTER(U64), C.POINTER(U64)]),
        "reina_gen_icosphere": (I32, [U32, F, U64, P, P, P]),
        "reina_geodesic_counts": (I32, [U32, C.POINTER(U64), C.POINTER(U64)]),
        "reina_gen_geodesic": (I32, [U32, F, U64, P, P, P]),
        "reina_gen_raycast_rays": (I32, [U32, U32, P, P, F, U64, P, P, U64, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(status: int) -> None:
    if status != REINA_OK:
        msg = _lib.reina_last_error().decode("utf-8", "replace")
        raise ReinaError(status, msg)


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a, shape_last=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def transform_to_c(m) -> np.ndarray:
    """4x4 matrix in math (row, column) indexing -> 16 floats column-major (glm::mat4 memory order)."""
    m = np.asarray(m, dtype=np.float32).reshape(4, 4)
    return np.ascontiguousarray(m.T.reshape(16))


class Context:
    def __init__(self, device: int = 0):
        lib = load_library()
        opts = _CtxOptions(device, 0)
        h = C.c_void_p()
        _check(lib.reina_ctx_create(C.byref(opts), C.byref(h)))
        self._h = h
        self.device = device
        self._servers = weakref.WeakSet()

    @property
    def handle(self):
        return self._h

    @property
    def sm_count(self) -> int:
        return int(_lib.reina_ctx_sm_count(self._h))

    def tuning(self) -> dict:
        t = _Tuning()
        _check(_lib.reina_ctx_get_tuning(self._h, C.byref(t)))
        return {k: int(getattr(t, k)) for k in TUNING_FIELDS}

    def set_tuning(self, **kw) -> None:
        """reina_ctx_set_tuning with the given fields changed (TUNING_FIELDS)."""
        t = _Tuning()
        _check(_lib.reina_ctx_get_tuning(self._h, C.byref(t)))
        for k, v in kw.items():
            if k not in TUNING_FIELDS:
                raise TypeError(f"unknown tuning field {k}")
            setattr(t, k, int(v))
        _check(_lib.reina_ctx_set_tuning(self._h, C.byref(t)))

    @property
    def refill(self) -> int:
        return self.tuning()["refill"]

    @refill.setter
    def refill(self, value: int) -> None:
        self.set_tuning(refill=value)

    def close(self) -> None:
        if self._h:
            for srv in list(self._servers):
                srv._h = None   # destroyed with the context
            _lib.reina_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """reina::scene::Scene (src/scene/Scene.h:62-138)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        _check(_lib.reina_scene_create(ctx.handle, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if self._h:
            _lib.reina_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def define_object(self, vertices, indices, tbns=None, tbn_indices=None, tex_coords=None, tex_indices=None) -> int:
        """Scene::defineObject(ModelData) — vertices (N,4) or (N,3) (w = 1 added), indices (3M,)."""
        v = np.asarray(vertices, dtype=np.float32)
        if v.ndim == 2 and v.shape[1] == 3:
            v = np.concatenate([v, np.ones((v.shape[0], 1), np.float32)], axis=1)
        v = np.ascontiguousarray(v.reshape(-1, 4))
        idx = _u32(np.asarray(indices).reshape(-1))
        tb = None if tbns is None else _f32(np.asarray(tbns).reshape(-1, 9))
        tbi = None if tbn_indices is None else _u32(np.asarray(tbn_indices).reshape(-1))
        tc = None if tex_coords is None else _f32(np.asarray(tex_coords).reshape(-1, 2))
        ti = None if tex_indices is None else _u32(np.asarray(tex_indices).reshape(-1))
        md = _ModelData(
            v.ctypes.data_as(C.POINTER(C.c_float)), v.shape[0],
            idx.ctypes.data_as(C.POINTER(C.c_uint32)), idx.size,
            None if tb is None else tb.ctypes.data_as(C.POINTER(C.c_float)), 0 if tb is None else tb.shape[0],
            None if tbi is None else tbi.ctypes.data_as(C.POINTER(C.c_uint32)), 0 if tbi is None else tbi.size,
            None if tc is None else tc.ctypes.data_as(C.POINTER(C.c_float)), 0 if tc is None else tc.shape[0],
            None if ti is None else ti.ctypes.data_as(C.POINTER(C.c_uint32)), 0 if ti is None else ti.size,
        )
        out = C.c_uint32()
        _check(_lib.reina_scene_define_object(self._h, C.byref(md), C.byref(out)))
        return int(out.value)

    def add_instance(self, object_id: int, transform=None, material: Material | None = None) -> None:
        t = transform_to_c(np.eye(4) if transform is None else transform)
        m = (material or Material()).to_c()
        _check(_lib.reina_scene_add_instance(self._h, object_id, t.ctypes.data_as(C.POINTER(C.c_float)), C.byref(m)))

    def add_object(self, vertices, indices, transform=None, material: Material | None = None, **kw) -> int:
        """Scene::addObject(ModelData, transform, material) (src/scene/Scene.h:106)."""
        oid = self.define_object(vertices, indices, **kw)
        self.add_instance(oid, transform, material)
        return oid

    def add_instance_per_face(self, object_id: int, transform, materials: list, face_material) -> None:
        t = transform_to_c(np.eye(4) if transform is None else transform)
        arr = (_Material * len(materials))(*[m.to_c() for m in materials])
        fm = _u32(face_material)
        _check(_lib.reina_scene_add_instance_per_face(self._h, object_id, t.ctypes.data_as(C.POINTER(C.c_float)), arr,
                                                      len(materials), fm.ctypes.data_as(C.POINTER(C.c_uint32))))

    def define_object_obj(self, path) -> int:
        """Scene::defineObject(filepath): a Wavefront OBJ file as one model."""
        oid = C.c_uint32()
        _check(_lib.reina_scene_define_object_obj(self._h, str(path).encode(), C.byref(oid)))
        return oid.value

    def add_object_obj(self, path, transform=None, material: "Material | None" = None) -> int:
        oid = self.define_object_obj(path)
        self.add_instance(oid, transform, material)
        return oid

    def add_gltf(self, path) -> dict:
        """gltf::loadScene without the build: the default scene of a .gltf/.glb file."""
        st = _GltfStats()
        _check(_lib.reina_scene_add_gltf(self._h, str(path).encode(), C.byref(st)))
        return {f: int(getattr(st, f)) for f, _ in _GltfStats._fields_}

    def define_texture_rgba8(self, rgba8) -> int:
        """Scene::defineTexture from raw texels: (H, W, 4) uint8, row 0 at v = 0."""
        a = np.ascontiguousarray(rgba8, np.uint8)
        if a.ndim != 3 or a.shape[2] != 4:
            raise ValueError("texture must be (H, W, 4) uint8")
        out = C.c_uint32()
        _check(_lib.reina_scene_define_texture_rgba8(self._h, _ptr(a), a.shape[1], a.shape[0], C.byref(out)))
        return out.value

    def define_texture(self, path) -> int:
        """Scene::defineTexture(filepath) (src/scene/Scene.cpp:15): an image file, rows flipped vertically."""
        out = C.c_uint32()
        _check(_lib.reina_scene_define_texture_file(self._h, str(path).encode(), C.byref(out)))
        return out.value

    def define_texture_encoded(self, data: bytes) -> int:
        """Scene::defineTexture(imageData, length) (src/scene/Scene.cpp:22): image file bytes, not flipped."""
        buf = C.create_string_buffer(bytes(data), len(data))
        out = C.c_uint32()
        _check(_lib.reina_scene_define_texture_encoded(self._h, buf, len(data), C.byref(out)))
        return out.value

    def instance_properties(self) -> np.ndarray:
        """The InstanceProperties records (structured array with the polyglot.h field names)."""
        n = C.c_uint32()
        _check(_lib.reina_scene_export_properties(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value, INSTANCE_PROPERTIES_DTYPE)
        _check(_lib.reina_scene_export_properties(self._h, _ptr(out), n.value, C.byref(n)))
        return out

    def export_texture(self, texture_id: int) -> np.ndarray:
        """Texels of a defined texture, (H, W, 4) uint8, row 0 at v = 0."""
        w, h = C.c_uint32(), C.c_uint32()
        _check(_lib.reina_scene_export_texture(self._h, texture_id, C.byref(w), C.byref(h), None, 0))
        out = np.empty((h.value, w.value, 4), np.uint8)
        _check(_lib.reina_scene_export_texture(self._h, texture_id, C.byref(w), C.byref(h), _ptr(out), out.nbytes))
        return out

    def export_two_level(self):
        """(instance records (N, 16) as raw 32-bit words, top-level leaf entries); empty for flat scenes."""
        ni, nr = C.c_uint32(), C.c_uint32()
        _check(_lib.reina_scene_export_two_level(self._h, None, None, C.byref(ni), C.byref(nr)))
        rec = np.zeros((ni.value, 16), np.uint32)
        refs = np.zeros(nr.value, np.uint32)
        _check(_lib.reina_scene_export_two_level(self._h, _ptr(rec), _ptr(refs), C.byref(ni), C.byref(nr)))
        return rec, refs

    def set_accel(self, mode: int) -> None:
        """ACCEL_AUTO, ACCEL_FLAT or ACCEL_TWO_LEVEL (before build)."""
        _check(_lib.reina_scene_set_accel(self._h, mode))

    def set_emissive_build(self, where: int) -> None:
        """EMISSIVE_HOST (default) or EMISSIVE_DEVICE: where build() computes the emissive CDFs."""
        _check(_lib.reina_scene_set_emissive_build(self._h, where))

    def set_bvh_build(self, where: int, sah_bins: int = 0, median_depth: int = 0) -> None:
        """BVH_HOST (default) or BVH_DEVICE: where build() builds the triangle BVHs (same bytes either way);
        sah_bins / median_depth 0 keep the defaults (32 bins, object medians from depth 48)."""
        _check(_lib.reina_scene_set_bvh_build(self._h, where, sah_bins, median_depth))

    def export_emissive(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(EmissiveInstanceData records, concatenated triangle CDFs, instance CDF) of the built scene."""
        ni, nt = C.c_uint32(), C.c_uint64()
        _check(_lib.reina_scene_export_emissive(self._h, None, C.byref(ni), None, C.byref(nt), None))
        inst = np.zeros(ni.value, EMISSIVE_INSTANCE_DTYPE)
        tris = np.zeros(nt.value, np.float32)
        cdf_i = np.zeros(ni.value, np.float32)
        _check(_lib.reina_scene_export_emissive(self._h, _ptr(inst), C.byref(ni), _ptr(tris), C.byref(nt), _ptr(cdf_i)))
        return inst, tris, cdf_i

    def texture_count(self) -> int:
        n = C.c_uint32()
        _check(_lib.reina_scene_texture_count(self._h, C.byref(n)))
        return n.value

    def object_count(self) -> int:
        n = C.c_uint32()
        _check(_lib.reina_scene_object_count(self._h, C.byref(n)))
        return n.value

    def export_object(self, object_id: int) -> dict:
        """The model data stored for an object: vertices (N,4), indices (3M,), tbns (K,9), tex_coords (L,2)."""
        nv, ni, nt, nu = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(_lib.reina_scene_export_object(self._h, object_id, None, C.byref(nv), None, C.byref(ni), None,
                                              C.byref(nt), None, C.byref(nu)))
        v = np.zeros((nv.value, 4), np.float32)
        i = np.zeros(ni.value, np.uint32)
        t = np.zeros((nt.value, 9), np.float32)
        u = np.zeros((nu.value, 2), np.float32)
        _check(_lib.reina_scene_export_object(self._h, object_id, _ptr(v), C.byref(nv), _ptr(i), C.byref(ni), _ptr(t),
                                              C.byref(nt), _ptr(u), C.byref(nu)))
        return {"vertices": v, "indices": i, "tbns": t, "tex_coords": u}

    def build(self, require_emissive: bool = False) -> None:
        _check(_lib.reina_scene_build(self._h, 1 if require_emissive else 0))

    @property
    def emissive_weight(self) -> float:
        return float(_lib.reina_scene_emissive_weight(self._h))

    def stats(self) -> dict:
        s = _SceneStats()
        _check(_lib.reina_scene_get_stats(self._h, C.byref(s)))
        d = {f[0]: getattr(s, f[0]) for f in _SceneStats._fields_}
        d["bounds_min"] = list(s.bounds_min)
        d["bounds_max"] = list(s.bounds_max)
        return d

    def export_bvh(self) -> tuple[np.ndarray, np.ndarray]:
        st = self.stats()
        nodes = np.zeros((st["node_count"], NODE_BYTES), np.uint8)
        tris = np.zeros((st["triangle_count"], TRI_BYTES), np.uint8)
        _check(_lib.reina_scene_export_bvh(self._h, _ptr(nodes), _ptr(tris)))
        return nodes, tris

    def prim_info(self, prim: int) -> tuple[int, int]:
        a, b = C.c_uint32(), C.c_uint32()
        _check(_lib.reina_scene_prim_info(self._h, prim, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)


def raycast(ctx: Context, scene: Scene, rays: np.ndarray, flags: int = RAY_CLOSEST) -> np.ndarray:
    """Host-buffer ray cast: rays -> hits (structured arrays RAY_DTYPE / HIT_DTYPE)."""
    rays = np.ascontiguousarray(rays)
    if rays.dtype != RAY_DTYPE:
        rays = np.ascontiguousarray(rays.view(np.float32).reshape(-1, 8)).view(RAY_DTYPE).reshape(-1)
    hits = np.empty(rays.shape[0], HIT_DTYPE)
    _check(_lib.reina_raycast(ctx.handle, scene.handle, _ptr(rays), rays.shape[0], _ptr(hits), flags))
    return hits


def raycast_into(ctx: Context, scene: Scene, rays_ptr: int, count: int, hits_ptr: int, flags: int = RAY_CLOSEST) -> None:
    """Host-buffer ray cast on caller-provided (ideally pinned) host memory."""
    _check(_lib.reina_raycast(ctx.handle, scene.handle, C.c_void_p(rays_ptr), count, C.c_void_p(hits_ptr), flags))


def raycast_device(ctx: Context, scene: Scene, d_rays: int, count: int, d_hits: int, flags: int = RAY_CLOSEST,
                   stream: int = 0) -> None:
    _check(_lib.reina_raycast_device(ctx.handle, scene.handle, C.c_void_p(d_rays), count, C.c_void_p(d_hits), flags,
                                     C.c_void_p(stream)))


def raycast_counters(ctx: Context, scene: Scene, d_rays: int, count: int, flags: int = RAY_CLOSEST,
                     stream: int = 0) -> tuple[int, int]:
    a, b = C.c_uint64(), C.c_uint64()
    _check(_lib.reina_raycast_counters(ctx.handle, scene.handle, C.c_void_p(d_rays), count, flags, C.byref(a),
                                       C.byref(b), C.c_void_p(stream)))
    return int(a.value), int(b.value)


def render(ctx: Context, scene: Scene, pc: RtPushConsts, opts: RenderOptions, accum: np.ndarray | None = None,
           want_samples: bool = False):
    """One frame (Reina::traceRays): returns (accum (H, W, 4) float32, samples (H*W, spp, 3) or None, stats)."""
    n = opts.width * opts.height
    if accum is None:
        accum = np.zeros((opts.height, opts.width, 4), np.float32)
    accum = np.ascontiguousarray(accum, dtype=np.float32)
    assert accum.size == 4 * n
    samples = np.zeros((n, pc.samplesPerPixel, 3), np.float32) if want_samples else None
    st = _RenderStats()
    _check(_lib.reina_render(ctx.handle, scene.handle, C.byref(pc), C.byref(opts), _ptr(accum), _ptr(samples),
                             C.byref(st)))
    return accum, samples, _stats_dict(st)


def render_device(ctx: Context, scene: Scene, pc: RtPushConsts, opts: RenderOptions, d_accum: int, d_samples: int = 0,
                  stream: int = 0) -> None:
    _check(_lib.reina_render_device(ctx.handle, scene.handle, C.byref(pc), C.byref(opts), C.c_void_p(d_accum),
                                    C.c_void_p(d_samples or None), C.c_void_p(stream)))


def postprocess(ctx: Context, accum: np.ndarray, radius: float = 5.0, threshold: float = 1.0, intensity: float = 0.05,
                exposure: float = 1.0, want_combined: bool = False):
    """Reina::applyBloom + applyTonemapping: accum (H, W, 4) float32 -> (rgba8 (H, W, 4) uint8, combined)."""
    accum = np.ascontiguousarray(accum, np.float32)
    H, W = accum.shape[:2]
    out = np.zeros((H, W, 4), np.uint8)
    comb = np.zeros((H, W, 4), np.float32) if want_combined else None
    b = BloomPushConsts(radius, threshold, intensity)
    t = TonemappingPushConsts(exposure)
    _check(_lib.reina_postprocess(ctx.handle, _ptr(accum), W, H, C.byref(b), C.byref(t), _ptr(out), _ptr(comb)))
    return out, comb


class RenderJob:
    """One frame of a batched render: scene, push constants, options and the images it writes."""

    def __init__(self, scene: Scene, pc: RtPushConsts, opts: RenderOptions, accum: np.ndarray | None = None,
                 want_samples: bool = False):
        n = opts.width * opts.height
        self.scene, self.pc, self.opts = scene, pc, opts
        if accum is None:
            accum = np.zeros((opts.height, opts.width, 4), np.float32)
        self.accum = np.ascontiguousarray(accum, dtype=np.float32)
        assert self.accum.size == 4 * n
        self.samples = np.zeros((n, pc.samplesPerPixel, 3), np.float32) if want_samples else None


def _jobs_array(jobs, device: bool):
    arr = (_RenderJob * max(1, len(jobs)))()
    for k, j in enumerate(jobs):
        arr[k].scene = j.scene.handle
        arr[k].push_consts = j.pc
        arr[k].options = j.opts
        if device:
            arr[k].accum = j.d_accum
            arr[k].samples = j.d_samples or None
        else:
            arr[k].accum = j.accum.ctypes.data
            arr[k].samples = None if j.samples is None else j.samples.ctypes.data
    return arr


def render_batch(ctx: Context, jobs: list) -> dict:
    """reina_render_batch: every RenderJob's frame traced in shared waves; fills job.accum / job.samples."""
    arr = _jobs_array(jobs, False)
    st = _RenderStats()
    _check(_lib.reina_render_batch(ctx.handle, arr, len(jobs), C.byref(st)))
    return _stats_dict(st)


class DeviceRenderJob:
    """A batched-render job on device buffers (addresses of 16-byte aligned device memory)."""

    def __init__(self, scene: Scene, pc: RtPushConsts, opts: RenderOptions, d_accum: int, d_samples: int = 0):
        self.scene, self.pc, self.opts, self.d_accum, self.d_samples = scene, pc, opts, d_accum, d_samples


def render_batch_device(ctx: Context, jobs: list, stream: int = 0) -> dict:
    arr = _jobs_array(jobs, True)
    st = _RenderStats()
    _check(_lib.reina_render_batch_device(ctx.handle, arr, len(jobs), C.c_void_p(stream), C.byref(st)))
    return _stats_dict(st)


def _status(st: _RequestStatus) -> dict:
    return {"state": int(st.state), "error": int(st.error), "latency_s": st.latency_s, "queue_s": st.queue_s,
            "message": st.message.decode("utf-8", "replace")}


class Server:
    """reina_server_*: a request loop that admits render requests by device-memory budget, keeps scenes and
    kept images resident with LRU eviction and runs admitted requests together in shared waves."""

    def __init__(self, ctx: Context, budget_bytes: int = 0, max_active: int = 0, wave_paths: int = 0,
                 graphs: bool = True, fifo: bool = False, shortest: bool = False, fair: bool = False,
                 wave_lanes: int = 0, aging: float = 0.0):
        """Wave-slot policy: shortest remaining work first (the default, or shortest=True), fifo=True or
        fair=True (an equal share per running request); at most one may be given."""
        self.ctx = ctx
        flags = ((0 if graphs else BATCH_NO_GRAPHS) | (SERVER_FIFO if fifo else 0) | (SERVER_SHORTEST if shortest else 0)
                 | (SERVER_FAIR_SHARE if fair else 0))
        o = _ServerOptions(budget_bytes, max_active, wave_paths, flags, wave_lanes, aging, 0)
        h = C.c_void_p()
        _check(_lib.reina_server_create(ctx.handle, C.byref(o), C.byref(h)))
        self._h = h
        ctx._servers.add(self)
        self._outputs = {}   # request id -> host image kept alive until the request ends

    @property
    def handle(self):
        if not self._h:
            raise ReinaError(REINA_ERR_STATE, "server is closed")
        return self._h

    def close(self) -> None:
        # A context destroys its servers; when garbage collection finalizes the context first (its
        # weak set of servers may already be cleared then), the server's handle is gone with it.
        if self._h and self.ctx._h:
            _lib.reina_server_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, scene: Scene) -> int:
        """Hands the scene over: the server owns and destroys it; the Scene object becomes unusable."""
        sid = C.c_uint32()
        _check(_lib.reina_server_add_scene(self.handle, scene.handle, C.byref(sid)))
        scene._h = None
        return sid.value

    def submit(self, scene_id: int, pc: RtPushConsts, opts: RenderOptions, out: np.ndarray | None = None,
               image_key: int = 0) -> int:
        """Queues a request; `out` ((H, W, 4) float32, or None with an image key) receives the image."""
        if out is not None:
            assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == 4 * opts.width * opts.height
        r = _Request(scene_id, 0, image_key, pc, opts, None if out is None else out.ctypes.data)
        rid = C.c_uint64()
        _check(_lib.reina_server_submit(self.handle, C.byref(r), C.byref(rid)))
        self._outputs[rid.value] = out
        return rid.value

    def poll(self, rid: int) -> dict:
        st = _RequestStatus()
        _check(_lib.reina_server_poll(self.handle, rid, C.byref(st)))
        return _status(st)

    def wait(self, rid: int, timeout_s: float = -1.0) -> dict:
        st = _RequestStatus()
        _check(_lib.reina_server_wait(self.handle, rid, float(timeout_s), C.byref(st)))
        d = _status(st)
        if d["state"] >= REQ_DONE:
            self._outputs.pop(rid, None)
        return d

    def cancel(self, rid: int) -> None:
        _check(_lib.reina_server_cancel(self.handle, rid))

    def fetch_image(self, key: int) -> np.ndarray:
        w, h = C.c_uint32(), C.c_uint32()
        _check(_lib.reina_server_fetch_image(self.handle, key, None, C.byref(w), C.byref(h)))
        out = np.zeros((h.value, w.value, 4), np.float32)
        _check(_lib.reina_server_fetch_image(self.handle, key, _ptr(out), C.byref(w), C.byref(h)))
        return out

    def stats(self) -> dict:
        st = _ServerStats()
        _check(_lib.reina_server_get_stats(self.handle, C.byref(st)))
        return {n: getattr(st, n) for n in _SERVER_STAT_FIELDS}


def _tune_result(r: _TuneResult) -> dict:
    return {"best": {k: int(getattr(r.best, k)) for k in TUNING_FIELDS}, "best_ms": r.best_ms,
            "default_ms": r.default_ms, "candidates": int(r.candidates), "kind": int(r.kind),
            "tri_bucket": int(r.tri_bucket), "size_bucket": int(r.size_bucket)}


def autotune_raycast(ctx: Context, scene: Scene, d_rays: int, count: int, d_hits: int, flags: int = RAY_CLOSEST,
                     stream: int = 0) -> dict:
    r = _TuneResult()
    _check(_lib.reina_autotune_raycast(ctx.handle, scene.handle, C.c_void_p(d_rays), count, C.c_void_p(d_hits), flags,
                                       C.c_void_p(stream), C.byref(r)))
    return _tune_result(r)


def autotune_render(ctx: Context, scene: Scene, pc: RtPushConsts, opts: RenderOptions) -> dict:
    r = _TuneResult()
    _check(_lib.reina_autotune_render(ctx.handle, scene.handle, C.byref(pc), C.byref(opts), C.byref(r)))
    return _tune_result(r)


def autotune_batch(ctx: Context, jobs: list) -> dict:
    """Times batch configurations on (up to 32 of) the jobs; jobs are RenderJob or DeviceRenderJob."""
    arr = _jobs_array(jobs, isinstance(jobs[0], DeviceRenderJob))
    r = _TuneResult()
    _check(_lib.reina_autotune_batch(ctx.handle, arr, len(jobs), C.byref(r)))
    return _tune_result(r)


def autotune_set_mode(ctx: Context, mode: int) -> None:
    _check(_lib.reina_autotune_set_mode(ctx.handle, mode))


def autotune_lookup(ctx: Context, kind: int, triangles: int, work_size: int) -> dict | None:
    t = _Tuning()
    found = C.c_int32()
    _check(_lib.reina_autotune_lookup(ctx.handle, kind, triangles, work_size, C.byref(t), C.byref(found)))
    return {k: int(getattr(t, k)) for k in TUNING_FIELDS} if found.value else None


def autotune_save(ctx: Context, path) -> None:
    _check(_lib.reina_autotune_save(ctx.handle, str(path).encode()))


def autotune_load(ctx: Context, path) -> None:
    _check(_lib.reina_autotune_load(ctx.handle, str(path).encode()))


def load_config(path) -> RunConfig:
    """config/config.toml (reina_config_load)."""
    lib = load_library()
    c = RunConfig()
    _check(lib.reina_config_load(str(path).encode(), C.byref(c)))
    return c


class SaveSchedule:
    """SaveManager: file names due at (samples, seconds), each save point once."""

    def __init__(self, config: RunConfig):
        lib = load_library()
        h = C.c_void_p()
        _check(lib.reina_save_schedule_create(C.byref(config), C.byref(h)))
        self._h = h

    def next(self, samples: int, seconds: float) -> str:
        buf = C.create_string_buffer(128)
        _check(_lib.reina_save_schedule_next(self._h, samples, float(seconds), buf, 128))
        return buf.value.decode()

    def close(self) -> None:
        if self._h:
            _lib.reina_save_schedule_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


KAT_OFFSET, KAT_GGX_VNDF, KAT_EVAL_DISNEY, KAT_RANDOM, KAT_OFFSET_DIELECTRIC, KAT_SAMPLE_DISNEY = 0, 1, 2, 3, 4, 5
KAT_DIFFUSE_REFLECTION, KAT_RANDOM_UNIT_VEC, KAT_SAMPLE_DISNEY_LOBE = 6, 7, 15


def device_error(ctx: "Context", stream: int = 0) -> int:
    """reina_ctx_device_error: the device error bits of the asynchronous calls queued on `stream` so far
    (raises ReinaError REINA_ERR_DEVICE when any is set; the word is cleared either way)."""
    out = C.c_uint32()
    _check(_lib.reina_ctx_device_error(ctx.handle, C.c_void_p(stream), C.byref(out)))
    return int(out.value)


def device_kat(ctx: "Context", kind: int, records: np.ndarray) -> np.ndarray:
    """reina_device_kat: single device shading functions on 40-float case records -> (n, 4) float32."""
    r = np.ascontiguousarray(records, np.float32).reshape(-1, 40)
    out = np.zeros((r.shape[0], 4), np.float32)
    _check(load_library().reina_device_kat(ctx._h, kind, _ptr(r), r.shape[0], _ptr(out)))
    return out


def decode_image(data: bytes) -> np.ndarray:
    """An image file's bytes (PNG or sequential JPEG) decoded to (H, W, 4) uint8, as the texture calls decode them."""
    L = load_library()
    buf = C.create_string_buffer(bytes(data), len(data))
    w, h = C.c_uint32(), C.c_uint32()
    _check(L.reina_decode_image(buf, len(data), C.byref(w), C.byref(h), None, 0))
    out = np.empty((h.value, w.value, 4), np.uint8)
    _check(L.reina_decode_image(buf, len(data), C.byref(w), C.byref(h), _ptr(out), out.nbytes))
    return out


def write_png(path, rgba8: np.ndarray) -> None:
    rgba8 = np.ascontiguousarray(rgba8, np.uint8)
    h, w = rgba8.shape[:2]
    _check(load_library().reina_write_png(str(path).encode(), _ptr(rgba8), w, h))


NOALLOC_MAX_PIXELS = 65536


def render_device_noalloc(ctx: Context, scene: Scene, pc: RtPushConsts, opts: RenderOptions, d_accum: int,
                          d_samples: int = 0, stream: int = 0) -> None:
    """reina_render_device_noalloc: the render without any device allocation, for callers that cannot
    allocate while they run; at most NOALLOC_MAX_PIXELS pixels; overlapping calls race."""
    _check(_lib.reina_render_device_noalloc(ctx.handle, scene.handle, C.byref(pc), C.byref(opts), C.c_void_p(d_accum),
                                            C.c_void_p(d_samples or None), C.c_void_p(stream)))


def camera_matrices(pos, front, up=(0.0, 1.0, 0.0), fovy_radians=np.radians(45.0), aspect=1.0, z_near=0.1,
                    z_far=100.0) -> tuple[np.ndarray, np.ndarray]:
    """inverse(glm::lookAt) and inverse(glm::perspective), 16 floats column-major each."""
    lib = load_library()
    p, f, u = (np.asarray(x, np.float32) for x in (pos, front, up))
    iv, ip = np.zeros(16, np.float32), np.zeros(16, np.float32)
    _check(lib.reina_camera_matrices(_ptr(p), _ptr(f), _ptr(u), float(fovy_radians), float(aspect), float(z_near),
                                     float(z_far), _ptr(iv), _ptr(ip)))
    return iv, ip


def icosphere(level: int, amplitude: float = 0.0, seed: int = 1) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Level-L icosphere, vertices radially displaced by 3-octave value noise; returns (V (N,4), I (3M,), N (N,3))."""
    lib = load_library()
    nv, nt = C.c_uint64(), C.c_uint64()
    _check(lib.reina_icosphere_counts(level, C.byref(nv), C.byref(nt)))
    v = np.zeros((nv.value, 4), np.float32)
    i = np.zeros(3 * nt.value, np.uint32)
    n = np.zeros((nv.value, 3), np.float32)
    _check(lib.reina_gen_icosphere(level, float(amplitude), seed, _ptr(v), _ptr(i), _ptr(n)))
    return v, i, n


def geodesic(frequency: int, amplitude: float = 0.0, seed: int = 1) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Frequency-n geodesic sphere (20 n^2 triangles), displaced like icosphere(); returns (V, I, N)."""
    lib = load_library()
    nv, nt = C.c_uint64(), C.c_uint64()
    _check(lib.reina_geodesic_counts(frequency, C.byref(nv), C.byref(nt)))
    v = np.zeros((nv.value, 4), np.float32)
    i = np.zeros(3 * nt.value, np.uint32)
    n = np.zeros((nv.value, 3), np.float32)
    _check(lib.reina_gen_geodesic(frequency, float(amplitude), seed, _ptr(v), _ptr(i), _ptr(n)))
    return v, i, n


def raycast_rays(width: int, height: int, cam_pos, cam_target, fovy_degrees: float, n_random: int, box_min, box_max,
                 seed: int = 1) -> np.ndarray:
    lib = load_library()
    out = np.zeros(width * height + n_random, RAY_DTYPE)
    cp, ct, bmin, bmax = (np.asarray(x, np.float32) for x in (cam_pos, cam_target, box_min, box_max))
    _check(lib.reina_gen_raycast_rays(width, height, _ptr(cp), _ptr(ct), float(fovy_degrees), n_random, _ptr(bmin),
                                      _ptr(bmax), seed, _ptr(out)))
    return out


def version() -> str:
    return load_library().reina_version().decode()
