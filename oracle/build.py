"""Build recipe of the FP64 oracle (test infrastructure, see aep_oracle.cpp).

Compiles aep_oracle.cpp into oracle/_build/liboracle.so with g++ and OpenMP.
Portable flags only (the library is rebuilt on x86_64 and on aarch64 hosts).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "aep_oracle.cpp"
HDR = HERE.parent / "include" / "aep.h"
OUT = HERE / "_build" / "liboracle.so"


def build(force: bool = False) -> Path:
    if not force and OUT.exists() and OUT.stat().st_mtime >= max(SRC.stat().st_mtime, HDR.stat().st_mtime):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
