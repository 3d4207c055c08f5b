"""ORACLE — test infrastructure only.  ctypes binding of `oracle/_ref/libref_glsl.so`, the reference's own
shader source compiled for the host by oracle/glsl/build_ref.py (see glsl_runtime.cpp for the C interface).

Only tests and the golden-fixture script use this; the library can be built only where the reference's
sources are present (REINA_REFERENCE_DIR), so every caller must handle `available() == False`.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE.parent / "_ref" / "libref_glsl.so"

# known-answer kinds (ref_kat_*.inc)
KAT_OFFSET, KAT_GGX_VNDF, KAT_EVAL_DISNEY, KAT_RANDOM, KAT_OFFSET_DIELECTRIC, KAT_SAMPLE_DISNEY = 0, 1, 2, 3, 4, 5
KAT_DIFFUSE_REFLECTION, KAT_RANDOM_UNIT_VEC, KAT_RANDOM_GAUSSIAN, KAT_HEXAGON = 6, 7, 8, 9
KAT_REFLECTANCE_DIELECTRIC, KAT_REFLECTANCE_DISNEY, KAT_TONEMAP, KAT_GAUSS, KAT_PDFS = 10, 11, 12, 13, 14

_lib = None


def reference_dir() -> Path | None:
    env = os.environ.get("REINA_REFERENCE_DIR")
    p = Path(env) if env else None
    return p if p is not None and (p / "shaders").is_dir() else None


def available() -> bool:
    """True when the library is built or can be built (the reference's sources are reachable)."""
    if LIB_PATH.exists():
        return True
    return reference_dir() is not None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if reference_dir() is not None:
            import importlib.util

            spec = importlib.util.spec_from_file_location("build_ref", HERE / "build_ref.py")
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        L = C.CDLL(str(LIB_PATH))
        P, U64, I = C.c_void_p, C.c_uint64, C.c_int
        L.ref_init.restype = I
        L.ref_set_buffer.argtypes = [I, P, U64]
        L.ref_set_scene.argtypes = [P, P, P, P, U64, P, P, P, U64]
        L.ref_set_textures.argtypes = [U64, P, P, P]
        L.ref_render.argtypes = [P, U64, I, I, P, I]
        L.ref_postprocess.argtypes = [P, I, I, P, P, P, P]
        L.ref_kat.argtypes = [I, P, U64, P]
        L.ref_out_of_range.restype = U64
        L.ref_init()
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def kat(kind: int, records: np.ndarray) -> np.ndarray:
    rec = np.ascontiguousarray(records, np.float32).reshape(-1, 40)
    out = np.zeros((rec.shape[0], 8), np.float64)
    lib().ref_kat(kind, _p(rec), rec.shape[0], _p(out))
    return out


def set_buffer(binding: int, data: np.ndarray) -> None:
    a = np.ascontiguousarray(data)
    lib().ref_set_buffer(binding, _p(a), a.nbytes)


def set_scene(tris9, tri_inst, tri_prim, tri_id, o2w12, custom, sbt) -> None:
    t = np.ascontiguousarray(tris9, np.float32)
    ti, tp, tid = (np.ascontiguousarray(x, np.uint32) for x in (tri_inst, tri_prim, tri_id))
    m = np.ascontiguousarray(o2w12, np.float32)
    cu, sb = np.ascontiguousarray(custom, np.uint32), np.ascontiguousarray(sbt, np.uint32)
    lib().ref_set_scene(_p(t), _p(ti), _p(tp), _p(tid), t.shape[0], _p(m), _p(cu), _p(sb), cu.shape[0])


def set_textures(images: list[np.ndarray]) -> None:
    w = np.array([im.shape[1] for im in images], np.uint32)
    h = np.array([im.shape[0] for im in images], np.uint32)
    texels = (np.concatenate([np.ascontiguousarray(im, np.uint8).reshape(-1, 4).view(np.uint32).reshape(-1) for im in images])
              if images else np.zeros(1, np.uint32))
    lib().ref_set_textures(len(images), _p(w), _p(h), _p(texels))


def render(push_consts: np.ndarray, width: int, height: int, image: np.ndarray | None = None, threads: int = 0) -> np.ndarray:
    pc = np.ascontiguousarray(push_consts)
    img = np.zeros((height, width, 4), np.float32) if image is None else np.ascontiguousarray(image, np.float32).copy()
    lib().ref_render(_p(pc), pc.nbytes, width, height, _p(img), threads or (os.cpu_count() or 1))
    return img


def postprocess(accum: np.ndarray, radius: float, threshold: float, intensity: float, exposure: float):
    a = np.ascontiguousarray(accum, np.float32)
    H, W = a.shape[:2]
    bp = np.array([radius, threshold, intensity], np.float32)
    tp = np.array([exposure], np.float32)
    bloomed = np.zeros_like(a)
    out8 = np.zeros((H, W, 4), np.uint8)
    lib().ref_postprocess(_p(a), W, H, _p(bp), _p(tp), _p(bloomed), _p(out8))
    return bloomed, out8


def out_of_range() -> int:
    return int(lib().ref_out_of_range())
