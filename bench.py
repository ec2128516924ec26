"""Benchmark of the CP_AL (LP) hot path on one GB300 (or N replicas).

Workload: the large single LP -- m = 1,000,000 rows, n = 2,000,000 variables,
~20M nonzeros with Zipf(1.5) row lengths capped at 20,000, entries
N(0,1) * 10^U[-3,3] per row and per column, 5% free variables, b and c from a
planted primal/dual pair (pdal_gb300.instances.zipf_lp, seed 1000).  The
algorithm settings are the reference's random-LP protocol (sigma mode, paper
sigma controller, CP_AL_LAMBDA=0, restart thresholds 0.2/0.8/0.36).

A step is ITERS_PER_STEP iterations of that solve, continued from the device
resident session (every evaluation, restart and phase decision included).

  value     iteration HBM throughput of the chosen form (FP32 iteration with
            FP64 anchors/reductions): algorithmic bytes of the iterations /
            wall time of the steps, GB/s, inputs resident in HBM
  e2e       the same metric through the C entry points with host buffers:
            each step is one cp_al_gb300_solve call of ITERS_PER_STEP
            iterations (problem copy, upload, equilibration, power iteration,
            iterations, result download inside the timed region)
  plain_fp64  the same metric for the plain FP64 form
  time_to_kkt the time to relative KKT 1e-6 of both forms on the plain CP_AL
            LP (2,000 x 5,000), which converges in seconds; the large LP needs
            minutes per solve

--impl reference times the CPU restatement of the iteration (the reference
has no CPU solver; the oracle port, every host thread) on a bounded sample:
one evaluation block (200 iterations) per step, same metric.
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

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "large_lp": (dict(m=1_000_000, n=2_000_000, nnz=20_000_000, seed=1000),
                 "LP 1,000,000 x 2,000,000, ~20M nnz, Zipf(1.5) rows <= 20,000, entries N(0,1)*10^U[-3,3] "
                 "per row and column, 5% free variables"),
    "medium_lp": (dict(m=100_000, n=200_000, nnz=2_000_000, seed=1001),
                  "LP 100,000 x 200,000, ~2M nnz, same structure at 1/10 scale"),
}
ITERS_PER_STEP = 1000
METRIC = "iteration HBM GB/s of the CP_AL iteration on the large LP (chosen form: FP32 + FP64 refinement)"
# the reference's random-LP protocol (experiments/random_lp/run_random_lp.sbatch:81-97)
SIGMA_PROTOCOL = {"sigma_mode": 1, "sigma_adaptive": 1, "sigma_init_factor": 0.5, "sigma_min_factor": 1e-4,
                  "sigma_max_factor": 100.0, "sigma_balance_gain": 0.0, "sigma_kp": 0.5, "sigma_ki": 0.0,
                  "sigma_kd": 0.0, "sigma_update_min": 1e-6, "sigma_update_max": 1e6, "lambda_factor": 2.01,
                  "al_lambda": 0.0, "restart_sufficient": 0.2, "restart_necessary": 0.8, "restart_artificial": 0.36}
PARAMS = {"eps": 1e-6, "l_inf_ruiz_iterations": 10}


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
        rows = [[c.strip() for c in r.split(",")] for r in self.f.read().strip().splitlines() if r.count(",") >= 6]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [v for v in (num(r[0]) for r in rows) if v is not None]
        mx = [v for v in (num(r[1]) for r in rows) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def iteration_bytes(m, n, nnz, sv, beta_on=True):
    """Algorithmic bytes of one primal launch and one dual launch: each matrix
    streamed once (values + int32 column indices + int32 row pointers), the
    gathered vector read once, every per-row vector read or written once.
    Anchors are 8 bytes in both forms (FP64, or an FP32 (hi, lo) pair)."""
    primal = nnz * (sv + 4) + 4 * (n + 1) + sv * m + n * (6 * sv + 8)
    dual_row = (6 * sv + 16) if beta_on else (4 * sv + 8)
    dual = nnz * (sv + 4) + 4 * (m + 1) + sv * n + m * dual_row
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
    chosen = {**SIGMA_PROTOCOL, "precision": "fp32_refine", "device": local, "timing": 1,
              "fp32_stall_evals": 1_000_000_000}
    plain = {**SIGMA_PROTOCOL, "precision": "fp64", "device": local, "timing": 1}

    def barrier():
        if dist:
            dist.barrier()

    def max_over_ranks(x):
        if not dist:
            return x
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def timed_steps(step, k):
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = [step() for _ in range(k)]
        torch.cuda.synchronize()
        return max_over_ranks(time.perf_counter() - t0), out

    # chosen form, device-resident session
    sess = lp.LPSession(data, PARAMS, chosen)
    sess.start()
    for _ in range(args.warmup):
        sess.iterate(ITERS_PER_STEP)
    it0 = sess.iterate(0).iterations
    launches0 = sess.iterate(0).stats["kernel_launches"]
    with Clocks(local) as clk:
        dt, res = timed_steps(lambda: sess.iterate(ITERS_PER_STEP), args.steps)
    r = res[-1]
    iters = r.iterations - it0
    st = r.stats
    launches = int(st["kernel_launches"] - launches0)
    sess.close()
    b_primal, b_dual = iteration_bytes(m, n, nnz, 4)
    value = (b_primal + b_dual) * iters * world / dt / 1e9

    # dominant kernel of the FP32 iteration, timed with CUDA events on the
    # library's stream inside the same steps
    tp, td = st["avg_primal32_ms"], st["avg_dual32_ms"]
    name, b, t_ms = ("k_dual<float>", b_dual, td) if td >= tp else ("k_primal<float>", b_primal, tp)
    hbm, src = peaks()
    achieved = b / (t_ms * 1e-3) / 1e9 if t_ms > 0 else None

    # plain FP64 form
    s64 = lp.LPSession(data, PARAMS, plain)
    s64.start()
    for _ in range(args.warmup):
        s64.iterate(ITERS_PER_STEP)
    i0 = s64.iterate(0).iterations
    dt64, r64s = timed_steps(lambda: s64.iterate(ITERS_PER_STEP), max(1, args.steps // 2))
    r64 = r64s[-1]
    s64.close()
    b64p, b64d = iteration_bytes(m, n, nnz, 8)
    value64 = (b64p + b64d) * (r64.iterations - i0) * world / dt64 / 1e9

    # end to end through the C entry points (host buffers)
    e2e_params = {**PARAMS, "iteration_limit": ITERS_PER_STEP}
    lp.solve(data, e2e_params, chosen)
    dte, rese = timed_steps(lambda: lp.solve(data, e2e_params, chosen), max(1, args.steps // 4))
    re = rese[-1]
    e2e_value = (b_primal + b_dual) * re.iterations * len(rese) * world / dte / 1e9

    # time to relative KKT 1e-6 on the plain CP_AL LP (2,000 x 5,000)
    small = instances.random_lp(2000, 5000, 8, seed=0)
    sp = {"eps": 1e-6, "l_inf_ruiz_iterations": 4}
    kkt = {}
    for tag, opts in (("chosen", {"precision": "fp32_refine", "device": local}), ("plain_fp64", {"device": local})):
        lp.solve(small, sp, opts)
        t0 = time.perf_counter()
        rr = lp.solve(small, sp, opts)
        kkt[tag] = {"s": time.perf_counter() - t0, "iterations": rr.iterations, "status": rr.status,
                    "objective": rr.primal_objective}

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32+f64",
            "data": "synthetic (seeded generator, shapes of the large-LP benchmark)",
            "config": {"workload": args.workload, "description": desc, "m": m, "n": n, "nnz": nnz,
                       "iterations_per_step": ITERS_PER_STEP, "algorithm": "random-LP sigma protocol",
                       "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2 (~450 MB streamed per iteration)"},
            "iterations_per_s": iters / (dt / args.steps * args.steps),
            "us_per_iteration": dt / max(iters, 1) * 1e6,
            "kkt_after_steps": r.kkt,
            "plain_fp64": {"value": value64, "unit": "GB/s",
                           "us_per_iteration": dt64 / max(r64.iterations - i0, 1) * 1e6},
            "e2e": {"value": e2e_value, "unit": "GB/s", "h2d_bytes_per_step": int(re.stats["h2d_bytes"]),
                    "d2h_bytes_per_step": int(re.stats["d2h_bytes"]), "s_per_step": dte / len(rese)},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": (achieved / hbm) if achieved else None, "traffic": None,
                         "bytes_per_launch": b, "avg_launch_ms": t_ms, "peak_source": src},
            "time_to_kkt_1e-6_small_lp": kkt,
            "clocks": clk.summary(),
        }
        line["cpu_baseline"] = cpu_baseline(data, m, n, nnz)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def cpu_baseline(data, m, n, nnz, blocks=1, warm=0):
    """The CPU restatement (oracle port) on every host core: one evaluation
    block (200 iterations) after setup, in the metric's unit."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    s = O.Session(data, {**PARAMS, "sv_max_iter": 20}, SIGMA_PROTOCOL, threads=threads)
    for _ in range(warm):
        s.iterate(200)
    t0 = time.perf_counter()
    done = sum(s.iterate(200) for _ in range(blocks))
    dt = time.perf_counter() - t0
    s.close()
    b_p, b_d = iteration_bytes(m, n, nnz, 8)
    return {"value": (b_p + b_d) * done / dt / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"{done} iterations of the same LP and settings (setup excluded) with {threads} threads, "
                      f"{dt / done * 1e3:.1f} ms/iteration",
            "ms_per_iteration": dt / done * 1e3}


def run_reference(args, rank, world, local):
    if rank != 0:
        return
    from oracle import oracle as O
    from pdal_gb300 import instances

    gen_kwargs, desc = WORKLOADS[args.workload]
    data = instances.zipf_lp(**gen_kwargs)
    rp, ci, v, (m, n) = data.csr()
    nnz = int(ci.shape[0])
    threads = os.cpu_count() or 1
    s = O.Session(data, {**PARAMS, "sv_max_iter": 20}, SIGMA_PROTOCOL, threads=threads)
    for _ in range(args.warmup):
        s.iterate(200)
    t0 = time.perf_counter()
    done = sum(s.iterate(200) for _ in range(args.steps))
    dt = time.perf_counter() - t0
    s.close()
    b_p, b_d = iteration_bytes(m, n, nnz, 8)
    val = (b_p + b_d) * done / dt / 1e9
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / max(args.steps, 1) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "description": desc, "m": m, "n": n, "nnz": nnz,
                   "iterations_per_step": 200, "algorithm": "random-LP sigma protocol"},
        "cpu_baseline": {"value": val, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{done} iterations (one evaluation block per step) with {threads} threads"},
        "e2e": {"value": val, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large_lp", choices=list(WORKLOADS))
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
