"""Runs the reference's own CP_AL and FA_CP solvers on the seeded cases of
tests/ref_cases.py and writes their results as fixtures under
tests/golden/ref_solver/: one JSON per case (status, iteration count,
objectives and residuals at full precision, times) and, for small cases, the
primal and dual solutions (.npz).  The parity tests (tests/test_ref_parity*.py)
hold this library and the CPU oracle to these fixtures.

The reference is GPU code: this script runs where a GPU is, with the
reference solvers already built by oracle/build.py (build_ref_solvers, which
compiles the reference's sources where they lie; PDAL_REFERENCE_DIR names
their directory).  Each solve is one fresh process with every CP_AL_* and
FA_CP_* variable cleared and the case's own set, as the reference's runners do
(experiments/random_lp/run_random_lp.sbatch:64-68).

    python tests/golden/make_ref_solver_golden.py --bin oracle/_ref --out DIR [--only a,b] [--timing]

--timing also writes the reference timing rows that need no parity: the large
LP's time per iteration and a sample of the 4,096-LP batch solved one by one.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import ref_cases as RC  # noqa: E402


def _env(extra: dict) -> dict:
    env = {k: v for k, v in os.environ.items() if not (k.startswith("CP_AL_") or k.startswith("FA_CP_"))}
    env.update(extra)
    return env


def run_ref(bin_dir: Path, kind: str, data, env: dict, params: dict, vectors: bool, tmp: Path):
    exe = bin_dir / ("ref_cp_al" if kind == "lp" else "ref_fa_cp")
    prob = tmp / "problem.bin"
    prob.write_bytes(RC.problem_bytes(data))
    args = [str(exe), str(prob), *RC.driver_args(params)]
    if vectors:
        args += [f"out_x={tmp / 'x.bin'}", f"out_y={tmp / 'y.bin'}"]
    t0 = time.perf_counter()
    res = subprocess.run(args, capture_output=True, text=True, env=_env(env), timeout=3600)
    wall = time.perf_counter() - t0
    if res.returncode != 0:
        raise RuntimeError(f"{exe.name} failed ({res.returncode}):\n{res.stderr[-3000:]}")
    line = [ln for ln in res.stdout.splitlines() if ln.startswith("{")][-1]
    out = json.loads(line)
    out["process_wall_sec"] = wall
    out["controllers"] = RC.controller_events(res.stderr + "\n" + res.stdout)
    x = y = None
    if vectors:
        x = np.fromfile(tmp / "x.bin", dtype="<f8")
        y = np.fromfile(tmp / "y.bin", dtype="<f8")
    return out, x, y


def run_cli_cases(bin_dir: Path, out_dir: Path, only: set, tmp: Path, meta: dict) -> None:
    """The reference's own CP_AL command on each CLI case's MPS file: its
    summary file and what its policy layer did (RC.cli_events of its
    stderr)."""
    import hashlib

    from pdal_gb300 import mps

    exe = bin_dir / "ref_cp_al_cli"
    for case in RC.CLI_CASES:
        if only and case["name"] not in only:
            continue
        data = RC.make_instance(case["gen"])
        src = mps.write_lp(data, tmp / f"{case['name']}.mps")
        outd = tmp / f"{case['name']}_out"
        outd.mkdir(exist_ok=True)
        t0 = time.perf_counter()
        res = subprocess.run([str(exe), *case["args"], str(src), str(outd)], capture_output=True, text=True,
                             env=_env(case["env"]), timeout=3600)
        wall = time.perf_counter() - t0
        if res.returncode != 0:
            raise RuntimeError(f"{exe.name} failed ({res.returncode}):\n{res.stderr[-3000:]}")
        rec = {"name": case["name"], "mps_sha256": hashlib.sha256(src.read_bytes()).hexdigest(), "gen": case["gen"],
               "env": case["env"], "args": case["args"],
               "summary": RC.read_summary(outd / f"{case['name']}_summary.txt"),
               "events": RC.cli_events(res.stderr + "\n" + res.stdout), "process_wall_sec": wall,
               "driver": "oracle/_ref/ref_cp_al_cli (LP/CP_AL/src/cli.c)", "gpu": meta["gpu"]}
        (out_dir / f"{case['name']}.json").write_text(json.dumps(rec, indent=1) + "\n")
        print(f"{case['name']}: {rec['summary']['Termination Reason']} iters={rec['summary']['Iterations Count']} "
              f"events={rec['events']} wall={wall:.2f}s", flush=True)


def gpu_name() -> str:
    try:
        return subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader"], capture_output=True,
                              text=True, timeout=60).stdout.strip().splitlines()[0]
    except Exception:
        return "unknown"


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--bin", type=Path, default=ROOT / "oracle" / "_ref")
    ap.add_argument("--out", type=Path, default=ROOT / "tests" / "golden" / "ref_solver")
    ap.add_argument("--only", default="")
    ap.add_argument("--timing", action="store_true")
    ap.add_argument("--cli", action="store_true", help="only the reference command's cases (CLI_CASES)")
    a = ap.parse_args()
    a.out.mkdir(parents=True, exist_ok=True)
    only = set(filter(None, a.only.split(",")))
    meta = {"gpu": gpu_name(), "reference_build": "oracle/build.py build_ref_solvers (sm_103a, -O3, cuSPARSE/cuBLAS)",
            "driver": "oracle/ref_driver/ref_solve.c"}
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        if a.cli:
            run_cli_cases(a.bin, a.out, only, tmp, meta)
            return
        for case in RC.CASES:
            if only and case["name"] not in only:
                continue
            data = RC.make_instance(case["gen"], case["kind"])
            r, x, y = run_ref(a.bin, case["kind"], data, case["env"], case["params"], bool(case.get("vectors")), tmp)
            rec = {"name": case["name"], "kind": case["kind"], "instance_sha256": RC.instance_sha256(data),
                   "gen": case["gen"], "env": case["env"], "params": case["params"], "ref": r, **meta}
            (a.out / f"{case['name']}.json").write_text(json.dumps(rec, indent=1) + "\n")
            if x is not None:
                np.savez_compressed(a.out / f"{case['name']}.npz", x=x, y=y)
            print(f"{case['name']}: reason={r['termination_reason']} iters={r['iterations']} "
                  f"obj={r['primal_objective']:.12g} t={r['cumulative_time_sec']:.3f}s", flush=True)
        if not a.timing:
            return
        # the large LP: time per iteration from two iteration limits
        c = RC.C1_TIMING
        data = RC.make_instance(c["gen"])
        runs = {}
        for lim in c["limits"]:
            r, _, _ = run_ref(a.bin, "lp", data, c["env"], {**c["params"], "iteration_limit": lim}, False, tmp)
            runs[lim] = r
            print(f"{c['name']} limit {lim}: iters={r['iterations']} t={r['cumulative_time_sec']:.3f}s", flush=True)
        lo, hi = c["limits"]
        per_iter = (runs[hi]["cumulative_time_sec"] - runs[lo]["cumulative_time_sec"]) / (hi - lo)
        rec = {"name": c["name"], "kind": "lp", "instance_sha256": RC.instance_sha256(data), "gen": c["gen"],
               "env": c["env"], "params": c["params"], "runs": {str(k): v for k, v in runs.items()},
               "us_per_iteration": per_iter * 1e6, **meta}
        (a.out / f"{c['name']}.json").write_text(json.dumps(rec, indent=1) + "\n")
        del data
        # the batch, one instance at a time (the batch benchmark's parameters)
        from pdal_gb300 import instances

        items = instances.batch_lps(count=4096)
        idx = [int(i) for i in np.linspace(0, 4095, RC.C3_SAMPLE)]
        params = {"eps": 1e-6, "l_inf_ruiz_iterations": 4, "iteration_limit": 100_000}
        rows = []
        for i in idx:
            r, _, _ = run_ref(a.bin, "lp", items[i], {}, params, False, tmp)
            rows.append({"index": i, "termination_reason": r["termination_reason"], "iterations": r["iterations"],
                         "solve_sec": r["wall_sec"], "cumulative_time_sec": r["cumulative_time_sec"]})
        mean = float(np.mean([q["solve_sec"] for q in rows]))
        rec = {"name": "lp_c3_one_by_one", "kind": "lp", "params": params, "sample": rows,
               "s_per_instance": mean, "extrapolated_4096_s": mean * 4096, **meta}
        (a.out / "lp_c3_one_by_one.json").write_text(json.dumps(rec, indent=1) + "\n")
        print(f"lp_c3_one_by_one: {mean:.4f} s per instance, {mean * 4096:.1f} s for 4096", flush=True)


if __name__ == "__main__":
    main()
