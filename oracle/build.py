"""Builds the CPU oracle (test infrastructure) into oracle/liboracle_pdal.so.

g++ with -ffp-contract=off so that x86 and Arm hosts give identical bits;
OpenMP when the compiler supports it (only the timed CPU baseline uses more
than one thread).
"""
from __future__ import annotations

import shutil
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


REFERENCE = Path("/root/reference")
REF_OUT = HERE / "_ref"
SHIM = HERE / "ref_shim"
# reference MPS readers, compiled from their own sources where they lie:
# output name -> (project directory, shim macro)
REF_READERS = {
    "libref_mps_lp.so": ("LP/CP_AL", "REF_LP"),
    "libref_mps_qp.so": ("QP/FA_CP", "REF_QP"),
}


def _cuda_include() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return str(Path(nvcc).resolve().parent.parent / "include")


def build_ref() -> list[Path]:
    """Compiles the reference's own MPS readers (LP/CP_AL/src/mps_parser.c and
    QP/FA_CP/src/mps_parser.c) and its FA_CP equilibration
    (QP/FA_CP/src/preconditioner.c), unmodified and read in place, into oracle/_ref/
    with gcc, zlib and ref_shim/ (allocation helpers, the problem free
    functions and an empty PSLP_stats.h).  Their internal headers include the
    CUDA headers for declarations only; nothing of CUDA is linked.  Returns
    the built objects, or [] where the reference sources are absent."""
    if not REFERENCE.exists():
        return []
    REF_OUT.mkdir(exist_ok=True)
    out = []
    for name, (proj, macro) in REF_READERS.items():
        src = REFERENCE / proj / "src" / "mps_parser.c"
        target = REF_OUT / name
        deps = [src, *SHIM.iterdir()]
        if target.exists() and target.stat().st_mtime > max(p.stat().st_mtime for p in deps):
            out.append(target)
            continue
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-w", f"-D{macro}", "-I", str(SHIM),
               "-I", str(REFERENCE / proj / "include"), "-I", str(REFERENCE / proj / "internal"),
               "-I", _cuda_include(), str(src), str(SHIM / "ref_mps_shim.c"), "-lz", "-o", str(target)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("reference reader build failed:\n" + " ".join(cmd) + "\n" + res.stderr)
        out.append(target)
    # the FA_CP equilibration (host code in the reference)
    proj = "QP/FA_CP"
    src = REFERENCE / proj / "src" / "preconditioner.c"
    target = REF_OUT / "libref_facp_precond.so"
    deps = [src, *SHIM.iterdir()]
    if not (target.exists() and target.stat().st_mtime > max(p.stat().st_mtime for p in deps)):
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-w", "-I", str(SHIM), "-I", str(REFERENCE / proj / "include"),
               "-I", str(REFERENCE / proj / "internal"), "-I", _cuda_include(), str(src),
               str(SHIM / "ref_precond_shim.c"), str(SHIM / "ref_mps_shim.c"), "-lm", "-o", str(target)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("reference preconditioner build failed:\n" + " ".join(cmd) + "\n" + res.stderr)
    out.append(target)
    return out


if __name__ == "__main__":
    print(build())
    for p in build_ref():
        print(p)
