"""Builds the CPU oracle (test infrastructure) into oracle/liboracle_pdal.so.

g++ with -ffp-contract=off so that x86 and Arm hosts give identical bits;
OpenMP when the compiler supports it (only the timed CPU baseline uses more
than one thread).
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCES = ["cpal_oracle.cpp", "facp_oracle.cpp"]
TARGET = HERE / "liboracle_pdal.so"


def build() -> Path:
    srcs = [HERE / s for s in SOURCES if (HERE / s).exists()]
    newest = max(p.stat().st_mtime for p in srcs + list((HERE.parent / "include").glob("*.h")))
    if TARGET.exists() and TARGET.stat().st_mtime > newest:
        return TARGET
    base = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(TARGET), *map(str, srcs)]
    res = subprocess.run(base[:1] + ["-fopenmp"] + base[1:], capture_output=True, text=True)
    if res.returncode != 0:
        res = subprocess.run(base, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    return TARGET


if __name__ == "__main__":
    print(build())
