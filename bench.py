"""Benchmark of the CP_AL (LP) hot path on one GB300 (or N replicas).

Workload (default): the large single LP -- m = 1,000,000 rows, n = 2,000,000
variables, ~20M nonzeros with Zipf(1.5) row lengths capped at 20,000, entries
N(0,1) * 10^U[-3,3] per row and per column, 5% free variables, planted b and c
(pdal_gb300.instances.zipf_lp, seed 1000).  A step is one full solve to
relative KKT 1e-6 (equilibration, power iteration, iteration loop, result).

  value   chosen form (FP32 iteration + FP64 reductions/refinement), inputs
          resident in HBM (session solve), seconds per solve
  e2e     the same solve through the C entry points with host buffers
          (create_lp_problem + cp_al_gb300_solve + result download)
  plain   the plain FP64 form, seconds per solve (same instance)

--impl reference times the CPU restatement of the same iteration (the
reference has no CPU solver) with every host thread, on a bounded sample: one
evaluation block of iterations, extrapolated to the iteration count of the
FP64 iteration on this instance.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    # name: (generator kwargs, description)
    "large_lp": (dict(m=1_000_000, n=2_000_000, nnz=20_000_000, seed=1000),
                 "LP 1,000,000 x 2,000,000, ~20M nnz, Zipf(1.5) rows <= 20,000, badly scaled"),
    "medium_lp": (dict(m=100_000, n=200_000, nnz=2_000_000, seed=1001),
                  "LP 100,000 x 200,000, ~2M nnz, Zipf(1.5) rows <= 20,000, badly scaled"),
}
EPS = 1e-6
# iterations of the plain FP64 iteration to relative KKT 1e-6 on each workload
# (measured on a GB300 with this code; the FP64 trajectory is the oracle's)
FP64_ITERATIONS = {"large_lp": None, "medium_lp": None}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 6]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].strip().replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[3 + i] and "Not" not in r[3 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_bytes(m, n, nnz, sv):
    """Bytes one primal and one dual launch must move (each matrix streamed
    once, every vector touched once, one gather of the other side's vector)."""
    dual = nnz * (sv + 4) + 4 * (m + 1) + sv * n + m * (6 * sv + 16)
    primal = nnz * (sv + 4) + 4 * (n + 1) + sv * m + n * (6 * sv + 8)
    return primal, dual


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_ours(args, rank, world, local):
    import torch

    from pdal_gb300 import instances, lp

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    gen_kwargs, desc = WORKLOADS[args.workload]
    data = instances.zipf_lp(**gen_kwargs)
    rp, ci, v, (m, n) = data.csr()
    nnz = int(ci.shape[0])
    params = {"eps": EPS, "l_inf_ruiz_iterations": 10}
    chosen = {"precision": "fp32_refine", "device": local, "timing": 1}
    plain = {"precision": "fp64", "device": local, "timing": 1}

    def timed(fn, k):
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = [fn() for _ in range(k)]
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if dist:
            t = torch.tensor([dt])
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dt = float(t.item())
        return dt / k, out

    sess = lp.LPSession(data, params, chosen)
    for _ in range(args.warmup):
        sess.solve()
    with Clocks(local) as clk:
        t_value, res = timed(sess.solve, args.steps)
    r = res[-1]
    sess.close()

    sess64 = lp.LPSession(data, params, plain)
    for _ in range(max(1, args.warmup // 3)):
        sess64.solve()
    t_plain, res64 = timed(sess64.solve, max(1, args.steps // 2))
    r64 = res64[-1]
    sess64.close()

    for _ in range(1):
        lp.solve(data, params, chosen)
    t_e2e, rese = timed(lambda: lp.solve(data, params, chosen), max(1, args.steps // 2))
    re = rese[-1]

    # dominant kernel (primal or dual launch) of the FP32 phase
    hbm, src = peaks()
    sv = 4
    b_primal, b_dual = algorithmic_bytes(m, n, nnz, sv)
    st = r.stats
    tp, td = st.get("avg_primal32_ms", 0.0), st.get("avg_dual32_ms", 0.0)
    if td >= tp:
        name, b, t_ms = "k_dual<float>", b_dual, td
    else:
        name, b, t_ms = "k_primal<float>", b_primal, tp
    achieved = b / (t_ms * 1e-3) / 1e9 if t_ms > 0 else None
    clocks = clk.summary()
    h2d = int(re.stats["h2d_bytes"])
    d2h = int(re.stats["d2h_bytes"])
    line = {
        "metric": "time to 1e-6 rel KKT (chosen: FP32 + FP64 refinement) on the large LP",
        "value": t_value,
        "unit": "s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_value * 1e3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": args.workload, "description": desc, "m": m, "n": n, "nnz": nnz, "eps": EPS,
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (matrices ~400 MB)"},
        "status": r.status,
        "iterations": r.iterations,
        "fp32_iterations": st["fp32_iterations"],
        "kkt": r.kkt,
        "plain_fp64": {"value": t_plain, "unit": "s", "iterations": r64.iterations, "status": r64.status,
                       "kkt": r64.kkt, "objective_rel_diff_vs_chosen":
                           abs(r64.primal_objective - r.primal_objective) / (1 + abs(r64.primal_objective))},
        "iterations_per_s": r.iterations / max(st["loop_sec"], 1e-12),
        "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(st["kernel_launches"]) * args.steps,
        "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": None,
                     "bytes_per_launch": b, "avg_launch_ms": t_ms, "peak_source": src},
        "clocks": clocks,
    }
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(data, r64.iterations, params)
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def cpu_baseline(data, iterations, params, threads=None, blocks=1):
    """CPU restatement (the oracle) on the host cores: `blocks` evaluation
    blocks of 200 iterations, extrapolated to `iterations`."""
    from oracle import oracle as O

    threads = threads or os.cpu_count() or 1
    p = dict(params)
    p["iteration_limit"] = 200 * blocks
    p["sv_max_iter"] = 20
    t0 = time.perf_counter()
    r = O.solve_lp(data, p, None, threads=threads)
    wall = time.perf_counter() - t0
    per_iter = r.solve_sec / max(r.iterations, 1)
    est = per_iter * iterations + (wall - r.solve_sec)
    return {"value": est, "unit": "s", "cores": threads, "kind": "port",
            "sample": f"{r.iterations} iterations (+ setup with 20 power steps) of the same LP with "
                      f"{threads} threads, {per_iter * 1e3:.1f} ms/iteration, extrapolated to {iterations} iterations",
            "ms_per_iteration": per_iter * 1e3}


def run_reference(args, rank, world, local):
    if rank != 0:
        return
    from pdal_gb300 import instances

    gen_kwargs, desc = WORKLOADS[args.workload]
    data = instances.zipf_lp(**gen_kwargs)
    rp, ci, v, (m, n) = data.csr()
    iters = FP64_ITERATIONS.get(args.workload) or 10000
    params = {"eps": EPS, "l_inf_ruiz_iterations": 10}
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(data, iters, params)
    for _ in range(args.steps):
        vals.append(cpu_baseline(data, iters, params))
    v = statistics.mean(x["value"] for x in vals)
    cb = dict(vals[-1])
    cb["value"] = v
    print(json.dumps({
        "impl": "reference", "metric": "time to 1e-6 rel KKT (chosen: FP32 + FP64 refinement) on the large LP",
        "value": v, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "description": desc, "m": m, "n": n, "nnz": int(ci.shape[0])},
        "cpu_baseline": cb, "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large_lp", choices=list(WORKLOADS))
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
