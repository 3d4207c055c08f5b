"""Builds the trace-path library `_build/libreina_gb300.so` from `csrc/` (CUDA for sm_103a + host C++), and
the headless renderer `_build/reina_render` from `cli/` against it.

Usage: python reina-vk_gb300/build.py [--force] [--ptxas-verbose]

The CUDA sources are compiled with `nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo`, the host
sources with g++ (-ffp-contract=off so that host floating-point results are identical on x86-64 and
aarch64), in parallel, and linked with the static CUDA runtime.  Objects are rebuilt only when a source
or any header of the package is newer than the object.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libreina_gb300.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDES = [f"-I{CSRC}", f"-I{ROOT / 'include'}", f"-I{CUDA_HOME / 'include'}"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-Wall",
            "-Wno-unused-function"]
NVCCFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
             "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include" / "reina").glob("*.h")))


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return t < src.stat().st_mtime or t < newest_header


def _compile(src: Path, obj: Path, ptxas_verbose: bool) -> tuple[Path, str]:
    if src.suffix == ".cu":
        cmd = [NVCC, *ARCH, *NVCCFLAGS, *INCLUDES, "-c", str(src), "-o", str(obj)]
        if ptxas_verbose:
            cmd[1:1] = ["-Xptxas", "-v"]
    else:
        cmd = ["g++", *CXXFLAGS, *INCLUDES, "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(force: bool = False, ptxas_verbose: bool = False, verbose: bool = False) -> Path:
    if shutil.which(NVCC) is None and not Path(NVCC).exists():
        raise RuntimeError(f"nvcc not found at {NVCC}")
    OUT.mkdir(exist_ok=True)
    sources = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    jobs = []
    objs = []
    for src in sources:
        obj = OUT / (src.name + ".o")
        objs.append(obj)
        if force or ptxas_verbose or _stale(obj, src, newest_header):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_compile, s, o, ptxas_verbose) for s, o in jobs]
            for f in cf.as_completed(futs):
                obj, err = f.result()
                if (verbose or ptxas_verbose) and err.strip():
                    print(f"[{obj.name}]\n{err}", file=sys.stderr)
    if force or jobs or not LIB.exists() or any(LIB.stat().st_mtime < o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [NVCC, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl", "-lrt"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    _build_cli(force)
    return LIB


OUT_CHECKED = PKG / "_build_checked"
LIB_CHECKED = OUT_CHECKED / "libreina_gb300.so"
OUT_WATCHDOG = PKG / "_build_watchdog"
LIB_WATCHDOG = OUT_WATCHDOG / "libreina_gb300.so"
WATCHDOG_STEPS = 2


def _build_variant(out_dir: Path, defines: list[str], force: bool) -> Path:
    """Every CUDA source again with `defines`, linked with the host objects of the normal build into
    `out_dir/libreina_gb300.so`."""
    build()
    lib = out_dir / "libreina_gb300.so"
    out_dir.mkdir(exist_ok=True)
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    objs, jobs = [], []
    for src in sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp"))):
        if src.suffix != ".cu":
            objs.append(OUT / (src.name + ".o"))
            continue
        obj = out_dir / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, src, newest_header):
            jobs.append([NVCC, *ARCH, *NVCCFLAGS, *defines, *INCLUDES, "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for res in ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs):
                if res.returncode != 0:
                    raise RuntimeError(f"variant build failed:\n{res.stdout}\n{res.stderr}")
    if force or jobs or not lib.exists() or any(lib.stat().st_mtime < o.stat().st_mtime for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lpthread", "-ldl", "-lrt"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"variant link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return lib


def build_checked(force: bool = False) -> Path:
    """The checked build: every CUDA source again with -DRT_CHECKED (the wavefront kernels check each queue
    position and path index and flag, instead of making, an out-of-bounds access), linked with the host
    objects of the normal build into `_build_checked/libreina_gb300.so`.  Not part of build()."""
    return _build_variant(OUT_CHECKED, ["-DRT_CHECKED"], force)


def build_watchdog(force: bool = False) -> Path:
    """The watchdog build: the traversal step limit lowered to WATCHDOG_STEPS, so that ordinary rays run
    past it and the device error path (flag set, ray ended, REINA_ERR_DEVICE at the C ABI) can be tested
    without a faulty scene.  `_build_watchdog/libreina_gb300.so`; not part of build()."""
    return _build_variant(OUT_WATCHDOG, [f"-DRT_MAX_TRAVERSAL_STEPS={WATCHDOG_STEPS}"], force)


CLI_SRC = PKG / "cli" / "reina_render.cpp"
CLI = OUT / "reina_render"


def _build_cli(force: bool) -> None:
    """The headless renderer (cli/reina_render.cpp), linked against the library (rpath $ORIGIN)."""
    if not force and CLI.exists() and CLI.stat().st_mtime >= max(CLI_SRC.stat().st_mtime, LIB.stat().st_mtime):
        return
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", f"-I{ROOT / 'include'}", str(CLI_SRC), "-o", str(CLI), f"-L{OUT}",
           "-lreina_gb300", "-Wl,-rpath,$ORIGIN", "-pthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, ptxas_verbose=a.ptxas_verbose, verbose=True))
