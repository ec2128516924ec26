"""Builds the CPU oracle (test infrastructure) into oracle/liboracle_pdal.so.

g++ with -ffp-contract=off so that x86 and Arm hosts give identical bits;
OpenMP when the compiler supports it (only the timed CPU baseline uses more
than one thread).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
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


# where the reference sources lie (read in place, never copied into the repository)
REFERENCE = Path(os.environ.get("PDAL_REFERENCE_DIR", "/root/reference"))
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
    QP/FA_CP/src/mps_parser.c), its FA_CP equilibration
    (QP/FA_CP/src/preconditioner.c) and its CP_AL command's policy layer
    (LP/CP_AL/src/cli.c, behind ref_shim/ref_cli_harness.c), unmodified and read in place, into oracle/_ref/
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
    # the CP_AL command's policy layer (LP/CP_AL/src/cli.c, host code) behind ref_cli_harness.c
    proj = "LP/CP_AL"
    src = REFERENCE / proj / "src" / "cli.c"
    target = REF_OUT / "libref_cli_policy.so"
    deps = [src, *SHIM.iterdir()]
    if not (target.exists() and target.stat().st_mtime > max(p.stat().st_mtime for p in deps)):
        cmd = ["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-w", "-DREF_LP", "-I", str(SHIM),
               "-I", str(REFERENCE / proj / "src"), "-I", str(REFERENCE / proj / "include"),
               "-I", str(REFERENCE / proj / "internal"), "-I", _cuda_include(), str(SHIM / "ref_cli_harness.c"),
               str(SHIM / "ref_mps_shim.c"), "-lm", "-o", str(target)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("reference policy layer build failed:\n" + " ".join(cmd) + "\n" + res.stderr)
    out.append(target)
    return out


# the reference solvers: executable -> (project, C sources, CUDA sources, driver macro)
REF_SOLVERS = {
    "ref_cp_al": ("LP/CP_AL", ["cp_al.c"], ["solver.cu", "utils.cu", "preconditioner.cu"], "REF_LP"),
    "ref_fa_cp": ("QP/FA_CP", ["fa_cp.c", "preconditioner.c"],
                  ["solver.cu", "utils.cu", "solver_state.cu", "fa_cp_core_op.cu"], "REF_QP"),
}
# the reference's own CP_AL command (LP/CP_AL/src/cli.c with its MPS reader and
# zlib): ref_cp_al's library objects (without the driver) plus these sources
REF_CLI = ("ref_cp_al_cli", "ref_cp_al", ["cli.c", "mps_parser.c"])
DRIVER = HERE / "ref_driver" / "ref_solve.c"


def build_ref_solvers(reference: Path | None = None, jobs: int | None = None) -> list[Path]:
    """Compiles the reference's own CP_AL and FA_CP solvers (their src/*.c and
    src/*.cu, unmodified, read where they lie) for sm_103a as the reference's
    CMake does (-O3, separable device compilation, cuSPARSE and cuBLAS), and
    links each with the driver ref_driver/ref_solve.c into oracle/_ref/; and
    the reference's CP_AL command itself (cli.c and its MPS reader with zlib
    over the same CP_AL objects) as oracle/_ref/ref_cp_al_cli.
    CP_AL's presolve library (PSLP) is absent: ref_shim/ gives its header and
    entry points, never reached with presolve off.  `reference` (default:
    PDAL_REFERENCE_DIR, else the reference's usual location) must hold
    LP/CP_AL and QP/FA_CP.  Returns the executables, or [] where the sources
    are absent.  Test infrastructure: only the fixture script
    tests/golden/make_ref_solver_golden.py runs them."""
    ref = Path(reference) if reference else REFERENCE
    if not (ref / "LP" / "CP_AL" / "src" / "solver.cu").exists():
        return []
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = _cuda_include()
    REF_OUT.mkdir(exist_ok=True)
    objdir = REF_OUT / "obj"
    objdir.mkdir(exist_ok=True)
    jobs_list = []  # (exe, object, command)
    for exe, (proj, csrcs, cusrcs, macro) in REF_SOLVERS.items():
        inc = ["-I", str(SHIM), "-I", str(ref / proj / "include"), "-I", str(ref / proj / "internal")]
        for s in cusrcs:
            obj = objdir / f"{exe}_{Path(s).stem}.o"
            jobs_list.append((exe, obj, [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-rdc=true",
                                         "-std=c++17", "-w", *inc, "-c", str(ref / proj / "src" / s), "-o",
                                         str(obj)]))
        for s in csrcs:
            obj = objdir / f"{exe}_{Path(s).stem}.o"
            jobs_list.append((exe, obj, ["gcc", "-O3", "-std=gnu99", "-w", *inc, "-I", cuda_inc, "-c",
                                         str(ref / proj / "src" / s), "-o", str(obj)]))
        extra = [SHIM / "ref_presolve_stub.c"] if macro == "REF_LP" else []
        for s in [DRIVER, *extra]:
            obj = objdir / f"{exe}_{s.stem}.o"
            jobs_list.append((exe, obj, ["gcc", "-O2", "-std=gnu99", "-w", f"-D{macro}", *inc, "-I", cuda_inc,
                                         "-c", str(s), "-o", str(obj)]))

    def run(cmd):
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("reference solver build failed:\n" + " ".join(cmd) + "\n" + res.stderr[-4000:])

    cli, base, cli_srcs = REF_CLI
    proj = REF_SOLVERS[base][0]
    inc = ["-I", str(SHIM), "-I", str(ref / proj / "include"), "-I", str(ref / proj / "internal")]
    for s in cli_srcs:
        jobs_list.append((cli, objdir / f"{cli}_{Path(s).stem}.o",
                          ["gcc", "-O3", "-std=gnu99", "-w", *inc, "-I", cuda_inc, "-c", str(ref / proj / "src" / s),
                           "-o", str(objdir / f"{cli}_{Path(s).stem}.o")]))

    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 2)) as ex:
        list(ex.map(run, [j[2] for j in jobs_list]))
    out = []
    for exe in REF_SOLVERS:
        objs = [str(o) for e, o, _ in jobs_list if e == exe]
        target = REF_OUT / exe
        run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-rdc=true", *objs, "-lcusparse", "-lcublas",
             "-lm", "-o", str(target)])
        out.append(target)
    objs = [str(o) for e, o, _ in jobs_list if e == cli or (e == base and DRIVER.stem not in o.name)]
    target = REF_OUT / cli
    run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-rdc=true", *objs, "-lcusparse", "-lcublas", "-lz",
         "-lm", "-o", str(target)])
    out.append(target)
    return out


if __name__ == "__main__":
    import sys

    print(build())
    for p in build_ref():
        print(p)
    if "--solvers" in sys.argv:
        for p in build_ref_solvers():
            print(p)
