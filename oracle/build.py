"""Build recipe of the FP64 oracle (test infrastructure, see aep_oracle.cpp).

Compiles aep_oracle.cpp into oracle/_build/liboracle.so with g++ and OpenMP,
tuned for the host it is built on (the library is rebuilt on every host and
never copied between machines): -mcpu=native on aarch64 (the GPU hosts' Grace
cores), -march=native on x86_64 with FP contraction off, so that the x86 build's
results stay those the golden fixtures were made with.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "aep_oracle.cpp"
HDR = HERE.parent / "include" / "aep.h"
OUT = HERE / "_build" / "liboracle.so"


def host_flags() -> list[str]:
    m = platform.machine().lower()
    if m in ("aarch64", "arm64"):
        return ["-mcpu=native"]
    if m in ("x86_64", "amd64"):
        return ["-march=native", "-ffp-contract=off"]
    return []


def build(force: bool = False) -> Path:
    if not force and OUT.exists() and OUT.stat().st_mtime >= max(SRC.stat().st_mtime, HDR.stat().st_mtime,
                                                                 Path(__file__).stat().st_mtime):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-O3", *host_flags(), "-std=c++17", "-fopenmp", "-fPIC", "-shared", str(SRC),
           "-o", str(tmp)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
