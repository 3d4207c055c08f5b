"""ORACLE — test infrastructure only.  Builds `oracle/_build/liboracle.so` from the oracle's C++ sources.

The oracle restates the reference's algorithms on the CPU and is only ever used as the checker (tests,
smoke check) and as the timed CPU baseline of bench.py; the product library never links or loads it.
Compiled with -ffp-contract=off so that float-mode results are plain IEEE binary32 on x86-64 and aarch64.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-Wall",
         "-Wno-unused-function"]


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    srcs = sorted(HERE.glob("*.cpp"))
    hdrs = sorted(HERE.glob("*.h"))
    newest = max(p.stat().st_mtime for p in srcs + hdrs)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = ["g++", *FLAGS, "-o", str(tmp), *map(str, srcs)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
