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


def test_triangle(tri9: np.ndarray, ray) -> tuple[bool, np.ndarray]:
    tri = np.ascontiguousarray(tri9, dtype=np.float32).reshape(9)
    r = np.ascontiguousarray(np.asarray(ray).reshape(1)).view(RAY_DTYPE)
    out = np.zeros(1, HIT_DTYPE)
    ok = lib().oracle_test_triangle(_p(tri), _p(r), _p(out))
    return bool(ok), out[0]
