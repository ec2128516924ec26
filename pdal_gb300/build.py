"""In-tree build of the native libraries (no cmake): nvcc for sm_103a, g++ for
host code, translation units compiled in parallel.

    python -m pdal_gb300.build            # product libraries
    python -m pdal_gb300.build --oracle   # also the CPU oracle (test infrastructure)
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
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"

NVCC_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off"]

# library name -> sources
LIBRARIES = {
    "libcp_al_gb300.so": ["cpal_solver.cu", "common.cpp", "cp_al_api.cpp", "noalloc.cu", "batch_solver.cu",
                          "mps_reader.cpp", "cp_al_policy.cpp"],
    "libfa_cp_gb300.so": ["facp_solver.cu", "common.cpp", "fa_cp_api.cpp", "mps_reader.cpp"],
    "libpdal_learn_gb300.so": ["mlp.cu", "common.cpp"],
}
# the drop-in commands: executable name -> (source, library it links)
EXECUTABLES = {
    "cp_al": ("cli_cp_al.cpp", "libcp_al_gb300.so"),
    "fa_cp": ("cli_fa_cp.cpp", "libfa_cp_gb300.so"),
}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pdal_gb300")


def _cuda_include() -> str:
    nvcc = Path(_nvcc()).resolve()
    return str(nvcc.parent.parent / "include")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


_ZLIB: bool | None = None


def _have_zlib() -> bool:
    """zlib header and library present (then .gz MPS files can be read)."""
    global _ZLIB
    if _ZLIB is None:
        BUILD.mkdir(exist_ok=True)
        probe = BUILD / "zlib_probe.cpp"
        probe.write_text("#include <zlib.h>\nint main() { return zlibVersion() == nullptr; }\n")
        res = subprocess.run(["g++", str(probe), "-lz", "-o", str(BUILD / "zlib_probe")], capture_output=True)
        _ZLIB = res.returncode == 0
    return _ZLIB


def _compile(src: Path, obj: Path) -> Path:
    obj.parent.mkdir(parents=True, exist_ok=True)
    deps = [*CSRC.glob("*.h"), *CSRC.glob("*.cuh"), *(ROOT / "include").glob("*.h")]
    if obj.exists() and obj.stat().st_mtime > max(src.stat().st_mtime, *(p.stat().st_mtime for p in deps)):
        return obj
    if src.suffix == ".cu":
        cmd = [_nvcc(), *NVCC_ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        extra = ["-DPDAL_HAVE_ZLIB"] if src.name == "mps_reader.cpp" and _have_zlib() else []
        cmd = ["g++", *CXX_FLAGS, *extra, "-I", _cuda_include(), "-c", str(src), "-o", str(obj)]
    _run(cmd)
    return obj


def build_product(jobs: int | None = None) -> list[Path]:
    LIBDIR.mkdir(exist_ok=True)
    BUILD.mkdir(exist_ok=True)
    out = []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 2)) as ex:
        futs = {}
        for srcs in LIBRARIES.values():
            for s in srcs:
                if s not in futs:
                    src = CSRC / s
                    futs[s] = ex.submit(_compile, src, BUILD / (src.stem + ".o"))
        objs = {s: f.result() for s, f in futs.items()}
    for lib, srcs in LIBRARIES.items():
        target = LIBDIR / lib
        # -Bsymbolic: calls inside a library bind to its own definitions (both
        # libraries export set_start_values and set_default_parameters)
        cmd = [_nvcc(), "-shared", "-o", str(target), *[str(objs[s]) for s in srcs], "-Xcompiler", "-fPIC",
               "-Xlinker", "-Bsymbolic"]
        if "mps_reader.cpp" in srcs and _have_zlib():
            cmd.append("-lz")
        _run(cmd)
        out.append(target)
    for exe, (src, lib) in EXECUTABLES.items():
        target = LIBDIR / exe
        cmd = ["g++", *CXX_FLAGS, str(CSRC / src), "-o", str(target), "-L", str(LIBDIR), f"-l:{lib}",
               "-Wl,-rpath,$ORIGIN"]
        _run(cmd)
        out.append(target)
    return out


def build_oracle() -> Path:
    sys.path.insert(0, str(ROOT))
    from oracle import build as ob  # test infrastructure, built beside the product

    return ob.build()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--oracle", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    a = ap.parse_args()
    for p in build_product(a.j):
        print(p)
    if a.oracle:
        print(build_oracle())


if __name__ == "__main__":
    main()
