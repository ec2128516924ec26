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
            LP (2,000 x 5,000), which converges in seconds; on the large LP the
            KKT error each form reaches within --kkt-cap seconds (neither this
            library nor the reference solver gets below ~1e-5 in minutes there)

Further sections of the same JSON line (skipped with --lp-only):
  fa_cp_qp            the FA_CP convex QP at its benchmark size: time to
                      relative KKT 1e-6 / 1e-8 through the C entry points,
                      error against the planted optimum, CPU port per iteration
  batch_4096          4,096 uneven LPs in one persistent launch (chosen form
                      and FP64): solves/s, p50/p99 iterations, and the speed-up
                      over the FP64 single-instance solver run one by one
  learned_warm_start  the MLP warm start + initial sigma on the 40 x 40
                      transportation family: iterations from the learned
                      start vs the cold start on held-out instances

--learned-full runs only the learned warm start on the 200 x 200 family
(20,000 training optima, 2,000 held-out instances; about 25 minutes).

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

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "large_lp": (dict(m=1_000_000, n=2_000_000, nnz=20_000_000, seed=1000),
                 "LP 1,000,000 x 2,000,000, ~20M nnz, Zipf(1.5) rows <= 20,000, entries N(0,1)*10^U[-3,3] "
                 "per row and column, 5% free variables"),
    "medium_lp": (dict(m=100_000, n=200_000, nnz=2_000_000, seed=1001),
                  "LP 100,000 x 200,000, ~2M nnz, same structure at 1/10 scale"),
    # the size the full ncu captures run on: larger than L2, ~0.5 GB on the device
    "half_lp": (dict(m=500_000, n=1_000_000, nnz=10_000_000, seed=1000),
                "LP 500,000 x 1,000,000, ~10M nnz, same structure at 1/2 scale"),
}
ITERS_PER_STEP = 1000
METRIC = "iteration HBM GB/s of the CP_AL iteration on the large LP (chosen form: FP32 + FP64 refinement)"
# the reference's random-LP protocol (experiments/random_lp/run_random_lp.sbatch:81-97)
SIGMA_PROTOCOL = {"sigma_mode": 1, "sigma_adaptive": 1, "sigma_init_factor": 0.5, "sigma_min_factor": 1e-4,
                  "sigma_max_factor": 100.0, "sigma_balance_gain": 0.0, "sigma_kp": 0.5, "sigma_ki": 0.0,
                  "sigma_kd": 0.0, "sigma_update_min": 1e-6, "sigma_update_max": 1e6, "lambda_factor": 2.01,
                  "al_lambda": 0.0, "restart_sufficient": 0.2, "restart_necessary": 0.8, "restart_artificial": 0.36}
PARAMS = {"eps": 1e-6, "l_inf_ruiz_iterations": 10}
# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the dominant
# kernel on this workload, from the ncu captures summarised in profiles/: the
# single dual kernel measured at full size; the split dual step measured at
# half size (102.2 MB for its three kernels) and doubled with the nonzeros
# and rows it processes
NCU_TRAFFIC = {"k_dual<float>": 200_110_336 + 4_137_984,
               "dual step: k_dual_short<float> + k_dual_panels<float> + k_dual_long_finish<float>":
                   2 * (40_567_296 + 54_784 + 60_497_920 + 348_672 + 688_640)}


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


def run_profile(args, local):
    """Only the chosen-form iteration steps on the large LP (no other
    sections): the command the ncu captures in profiles/ run.  With
    --profile-section qp: 300 iterations of the full-size QP (one persistent
    k_facp launch per evaluation segment), qp_fp32 the same in FP32 segments;
    batch: one k_batch_lp launch over 304 small LPs (m log-uniform in
    [50, 400]), chosen form."""
    from pdal_gb300 import instances, lp

    if args.profile_section in ("qp", "qp_fp32"):
        from pdal_gb300 import qp

        qd, _, _ = instances.planted_qp()
        opts = {"device": local}
        if args.profile_section == "qp_fp32":
            opts["precision"] = "fp32_refine"
            opts["fp32_switch_tol"] = 0.0  # the whole run in FP32 segments
            opts["fp32_stall_evals"] = 0
        r = qp.solve(qd, {"eps": 1e-12, "verbose": 0, "iteration_limit": 300}, opts)
        print(json.dumps({"profile_run": "qp", "iterations": r.iterations, "inner_iterations": r.inner_iterations,
                          "kernel_launches": r.stats["kernel_launches"]}), flush=True)
        return
    if args.profile_section == "batch":
        items = instances.batch_lps(count=304, seed=3100, m_range=(50, 400))
        res, st = lp.solve_batch(items, {"eps": 1e-6, "l_inf_ruiz_iterations": 4, "iteration_limit": 100_000},
                                 {"precision": "fp32_refine", "device": local})
        print(json.dumps({"profile_run": "batch", "optimal": st["optimal"], "kernel_s": st["kernel_sec"],
                          "iterations_max": st["iterations_max"], "grid_blocks": st["grid_blocks"]}), flush=True)
        return
    gen_kwargs, _ = WORKLOADS[args.workload]
    data = instances.zipf_lp(**gen_kwargs)
    chosen = {**SIGMA_PROTOCOL, "precision": "fp32_refine", "device": local, "fp32_stall_evals": 1_000_000_000}
    sess = lp.LPSession(data, PARAMS, chosen)
    sess.start()
    for _ in range(args.warmup + args.steps):
        r = sess.iterate(ITERS_PER_STEP)
    sess.close()
    print(json.dumps({"profile_run": args.workload, "iterations": r.iterations, "kkt": r.kkt}), flush=True)


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
    dual_name = ("dual step: k_dual_short<float> + k_dual_panels<float> + k_dual_long_finish<float>"
                 if st["panel_rows"] > 0 else "k_dual<float>")
    name, b, t_ms = (dual_name, b_dual, td) if td >= tp else ("k_primal<float>", b_primal, tp)
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

    # time to relative KKT 1e-6 on the plain CP_AL LP (2,000 x 5,000): the
    # median of three solves of each form after one untimed, with one CUDA
    # graph per evaluation block (the default) and with the loop on the device
    # (one cooperative launch per 50 evaluation blocks)
    small = instances.random_lp(2000, 5000, 8, seed=0)
    sp = {"eps": 1e-6, "l_inf_ruiz_iterations": 4}
    kkt = {}
    for tag, opts in (("chosen", {"precision": "fp32_refine", "device": local}), ("plain_fp64", {"device": local}),
                      ("chosen_device_loop", {"precision": "fp32_refine", "device": local, "persistent_loop": 1}),
                      ("plain_fp64_device_loop", {"device": local, "persistent_loop": 1})):
        lp.solve(small, sp, opts)
        runs = []
        for _ in range(3):
            t0 = time.perf_counter()
            rr = lp.solve(small, sp, opts)
            runs.append((time.perf_counter() - t0, rr))
        runs.sort(key=lambda q: q[0])
        dt_med, rr = runs[1]
        kkt[tag] = {"s": dt_med, "s_runs": [q[0] for q in runs], "iterations": rr.iterations, "status": rr.status,
                    "objective": rr.primal_objective}

    # the large LP itself towards relative KKT 1e-6 and 1e-8, capped
    large_kkt = bench_large_lp_kkt(data, local, args.kkt_cap) if args.kkt_cap > 0 else None

    extras = {}
    if not args.lp_only:
        def gather(obj):
            out = [None] * world
            dist.all_gather_object(out, obj)
            return out

        extras["batch_4096"] = bench_batch(local, rank=rank, world=world, barrier=barrier,
                                           max_over_ranks=max_over_ranks, gather=gather if dist else None)
        if rank == 0:
            extras["fa_cp_qp"] = bench_qp(local)
            extras["learned_warm_start"] = bench_learned(local)
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
                    "d2h_bytes_per_step": int(re.stats["d2h_bytes"]), "s_per_step": dte / len(rese),
                    "phases_s": {k: re.stats[k] for k in ("prepare_sec", "upload_sec", "upload_plan_sec",
                                                          "upload_alloc_sec", "equilibration_sec", "power_sec",
                                                          "setup_sec", "loop_sec", "total_sec")},
                    "power_iterations": re.stats["power_iterations"]},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": (achieved / hbm) if achieved else None,
                         "traffic": NCU_TRAFFIC.get(name),
                         "traffic_unit": "bytes per launch (dram read + write, ncu)",
                         "bytes_per_launch": b, "avg_launch_ms": t_ms, "peak_source": src},
            "time_to_kkt_1e-6_small_lp": kkt,
            "time_to_kkt_large_lp": large_kkt,
            "reference_gpu_recorded": reference_gpu_recorded(),
            "clocks": clk.summary(),
        }
        line["cpu_baseline"] = cpu_baseline(data, m, n, nnz, single=args.cpu_single)
        line.update(extras)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def bench_large_lp_kkt(data, local, cap_s):
    """The large LP solved from the start towards relative KKT 1e-8 in each
    form (random-LP sigma protocol), in chunks of 1,000 iterations of a
    device-resident session: the wall time at which the KKT error first fell
    below 1e-6 and below 1e-8, or, at the cap, the error reached.  Setup
    (equilibration, sigma_max estimate) is inside the time."""
    from pdal_gb300 import lp

    out = {"cap_s": cap_s, "chunk_iterations": 1000}
    params = {**PARAMS, "eps": 1e-8, "iteration_limit": 10_000_000}
    for tag, opts in (("chosen_fp32_refine", {"precision": "fp32_refine"}), ("plain_fp64", {"precision": "fp64"})):
        s = lp.LPSession(data, params, {**SIGMA_PROTOCOL, **opts, "device": local})
        t0 = time.perf_counter()
        s.start()
        t_setup = time.perf_counter() - t0
        reached = {}
        trace = []
        while True:
            r = s.iterate(1000)
            t = time.perf_counter() - t0
            trace.append((r.iterations, round(t, 3), r.kkt))
            for tol in (1e-6, 1e-8):
                if r.kkt < tol and tol not in reached:
                    reached[tol] = {"s": t, "iterations": r.iterations, "primal_objective": r.primal_objective}
            # the session stops at its tolerance (OPTIMAL) or any other end
            if r.status != "ITERATION_LIMIT" or t > cap_s:
                break
        s.close()
        out[tag] = {"setup_s": t_setup, "status": r.status, "iterations": r.iterations, "kkt_reached": r.kkt,
                    "wall_s": time.perf_counter() - t0, "fp32_iterations": r.stats["fp32_iterations"],
                    "to_1e-6": reached.get(1e-6), "to_1e-8": reached.get(1e-8),
                    "trace": trace[:: max(1, len(trace) // 12)]}
    a, b = out["chosen_fp32_refine"].get("to_1e-8"), out["plain_fp64"].get("to_1e-8")
    if a and b:
        out["rel_obj_diff_chosen_vs_fp64_at_1e-8"] = abs(a["primal_objective"] - b["primal_objective"]) / (
            1 + abs(b["primal_objective"]))
    return out


def reference_gpu_recorded():
    """The reference's own solvers (cuSPARSE/cuBLAS FP64, built from source
    for sm_103a) timed on a GB300 when the parity fixtures were made
    (tests/golden/ref_solver/*.json, tests/golden/make_ref_solver_golden.py):
    recorded figures, not measured by this run.  Times are the wall time of
    the solve call after CUDA context creation."""
    d = ROOT / "tests" / "golden" / "ref_solver"
    out = {"source": "tests/golden/ref_solver (recorded, not this run)"}
    try:
        def ref(name):
            return json.loads((d / f"{name}.json").read_text())

        for name, key in (("lp_c0_sigma_protocol_1e-6", "small_lp_1e-6_sigma_protocol"),
                          ("lp_c0_default_1e-6", "small_lp_1e-6_defaults"), ("qp_c2_full_1e-6", "qp_1e-6"),
                          ("qp_c2_full_1e-8", "qp_1e-8"), ("lp_c4_transport_200x200", "transport_200x200_1e-6")):
            r = ref(name)["ref"]
            out[key] = {"s": r["wall_sec"], "iterations": r["iterations"], "status_code": r["termination_reason"]}
        c1 = ref("lp_c1_iteration_time")
        lo, hi = sorted(c1["runs"], key=int)
        out["large_lp_us_per_iteration"] = (c1["runs"][hi]["wall_sec"] - c1["runs"][lo]["wall_sec"]) / (
            int(hi) - int(lo)) * 1e6
        c3 = ref("lp_c3_one_by_one")
        out["batch_4096_one_by_one_s"] = c3["extrapolated_4096_s"]
        out["batch_sample"] = len(c3["sample"])
    except (OSError, KeyError, ValueError) as e:
        out["unavailable"] = str(e)
    return out


def bench_qp(local):
    """The FA_CP convex QP at its full benchmark size (n = 200,000, m = 100,000,
    A 10 nnz/column, Q = B'B + diag with B 50,000 x 200,000 at 5 nnz/row, box
    bounds, planted optimum): time to relative KKT 1e-6 and 1e-8 through the C
    entry points (host buffers), against the planted objective; the CPU port's
    time per iteration on a bounded sample (50 iterations, one thread)."""
    from oracle import oracle as O
    from pdal_gb300 import instances, qp

    qd, _, f_star = instances.planted_qp()
    out = {"workload": "QP n=200,000 m=100,000, A 2.0M nnz, Q=B'B+diag (sparse Q), planted optimum",
           "chosen_form": "FP32 segments to relative KKT 5e-6 (fp32_switch_tol), then FP64"}
    # the FP32 phase ends at relative KKT 5e-6 (measured on this QP, to 1e-6:
    # 1e-5 / 5e-6 / 3e-6 / 2e-6 / 1e-6 gave 0.233 / 0.212 / 0.266 / 0.267 /
    # 0.267 s; below 5e-6 the FP32 iterate reaches its rounding floor and the
    # stall rule ends the phase 250 iterations later)
    for form, opts in (("chosen_fp32_refine", {"device": local, "precision": "fp32_refine", "fp32_switch_tol": 5e-6}),
                       ("plain_fp64", {"device": local})):
        out[form] = {}
        for eps in (1e-6, 1e-8):
            prm = {"eps": eps, "verbose": 0, "iteration_limit": 200_000, "time_limit": 300.0}
            if eps == 1e-6:
                qp.solve(qd, prm, opts)
            t0 = time.perf_counter()
            r = qp.solve(qd, prm, opts)
            dt = time.perf_counter() - t0
            out[form][f"eps_{eps:g}"] = {
                "s": dt, "status": r.status, "iterations": r.iterations, "fp32_iterations": r.stats["fp32_iterations"],
                "inner_iterations": r.inner_iterations, "kkt": r.kkt,
                "rel_obj_err_vs_planted": abs(r.primal_objective - f_star) / (1 + abs(f_star)),
                "setup_s": r.stats["setup_sec"], "loop_s": r.stats["loop_sec"],
                "device_segments_ms": r.stats["device_loop_ms"], "kernel_launches": r.stats["kernel_launches"]}
    t0 = time.perf_counter()
    ro = O.solve_qp(qd, {"eps": 1e-14, "iteration_limit": 50, "sv_max_iter": 20})
    out["cpu_port_s_per_iteration"] = ro.solve_sec / max(ro.iterations, 1)
    out["cpu_port_sample"] = f"{ro.iterations} iterations ({ro.inner_iterations} BB steps), 1 thread, setup excluded"
    out["gpu_s_per_iteration"] = out["plain_fp64"]["eps_1e-06"]["loop_s"] / max(
        out["plain_fp64"]["eps_1e-06"]["iterations"], 1)
    return out


def bench_batch(local, count=4096, rank=0, world=1, barrier=None, max_over_ranks=None, gather=None):
    """4,096 uneven LPs (m log-uniform in [50, 5000], n = m*U[2,3], 3-20
    nnz/column, planted) solved to relative KKT 1e-6 in one persistent launch,
    chosen form (FP32 phase + FP64 refinement) and FP64, against the plain FP64
    single-instance solver run instance by instance on the same GPU (timed on
    48 evenly spaced instances, scaled to the batch).  With N ranks the
    instances are split by an LPT assignment (no collective on the data path)
    and the time is the maximum over ranks."""
    from pdal_gb300 import instances, lp
    from pdal_gb300.shard import assemble, instance_weight, lpt_partition

    items = instances.batch_lps(count=count)
    nnz = sum(int(d.csr()[1].shape[0]) for d in items)
    parts = lpt_partition([instance_weight(d) for d in items], world)
    mine = parts[rank]
    shard = [items[i] for i in mine]
    params = {"eps": 1e-6, "l_inf_ruiz_iterations": 4, "iteration_limit": 100_000}
    out = {"workload": f"{count} LPs, m log-uniform [50, 5000], n = m*U[2,3], 3-20 nnz/column",
           "chosen_form": "FP32 phase to relative KKT 3e-6 (fp32_switch_tol), then FP64 to 1e-6",
           "sum_nnz": nnz, "sharding": f"LPT over {world} GPU(s), no collective"}
    # chosen form with the FP32 phase ending at relative KKT 3e-6 (measured on
    # this batch: 1e-5 / 3e-6 / 1e-6 gave 20.4 / 18.6 / 22.2 s; an FP32 phase
    # run to the 1e-6 tolerance itself converges more slowly near its end)
    for tag, opts in (("chosen_fp32_refine", {"precision": "fp32_refine", "device": local, "fp32_switch_tol": 3e-6}),
                      ("fp64", {"device": local})):
        # the schedule autotuner runs once per batch shape (its choice is
        # remembered): timed here, outside the solve it serves
        sched = lp.tune_batch(shard, params, opts)
        if barrier:
            barrier()
        t0 = time.perf_counter()
        res, st = lp.solve_batch(shard, params, opts)
        wall = time.perf_counter() - t0
        if max_over_ranks:
            wall = max_over_ranks(wall)
        rows = [(r.status == "OPTIMAL", r.iterations, r.kkt) for r in res]
        if gather is not None and world > 1:
            # every rank's per-instance results, back in the batch's order
            rows = assemble(parts, gather(rows))
        its = np.array([q[1] for q in rows])
        out[tag] = {"total_s": wall, "kernel_s": st["kernel_sec"], "solves_per_s": count / wall,
                    "optimal": int(sum(q[0] for q in rows)), "iterations_p50": float(np.percentile(its, 50)),
                    "iterations_p99": float(np.percentile(its, 99)), "iterations_max": int(its.max()),
                    "max_kkt": max(q[2] for q in rows), "grid_blocks": st["grid_blocks"],
                    "schedule": {"block_nnz": st["block_nnz"], "blocks_per_sm": st["blocks_per_sm"],
                                 "tune_s": sched["tune_sec"], "tuned_before_solve": st["tune_sec"] == 0.0}}
    if rank != 0:
        return out
    idx = [int(i) for i in np.linspace(0, count - 1, 48)]
    lp.solve(items[idx[0]], params, {"device": local})
    t0 = time.perf_counter()
    seq_its = [lp.solve(items[i], params, {"device": local}).iterations for i in idx]
    dt = time.perf_counter() - t0
    out["sequential_fp64"] = {"sample": len(idx), "s_per_instance": dt / len(idx),
                              "extrapolated_s": dt / len(idx) * count, "mean_iterations": float(np.mean(seq_its))}
    out["speedup_vs_sequential"] = out["sequential_fp64"]["extrapolated_s"] / out["chosen_fp32_refine"]["total_s"]
    return out


def bench_learned(local, S=40, D=40, n_train=4096, n_test=256, epochs=100, label_eps=1e-6, batch=128):
    """Learned warm start + initial sigma on the transportation family (costs
    U[1,100] x (1 + 0.2 N(0,1)), supplies/demands U[10,100] rebalanced,
    capacities U[20,200]): an MLP (3 layers, width 256, trained by the
    library's kernels on solver-generated optima, BF16 tensor-core inference,
    features, decoding and the predicted point's KKT on the GPU) predicts the
    start; held-out instances are solved to relative KKT 1e-6 from it and from
    the cold start (both as batch launches).  The default run uses the 40 x 40
    graph; --learned-full runs the 200 x 200 family with 20,000 training
    optima (solved to 1e-4: ~5,800 iterations and 0.034 s of batch time per
    instance, against ~20,000 iterations and 0.15 s to 1e-6) and 2,000
    held-out instances, ~25 minutes of GPU time."""
    from pdal_gb300.instances import transport_family
    from pdal_gb300.learn import WarmStart

    base = np.random.default_rng(4000).uniform(1, 100, S * D)
    train = transport_family(S, D, range(10_000, 10_000 + n_train), base)
    test = transport_family(S, D, range(900_000, 900_000 + n_test), base)
    params = {"eps": 1e-6, "l_inf_ruiz_iterations": 10, "iteration_limit": 100_000}
    t0 = time.perf_counter()
    solved, _ = WarmStart.solve_family(train, {**params, "eps": label_eps})
    t_label = time.perf_counter() - t0
    ws = WarmStart.fit(train, S, D, params, hidden=256, epochs=epochs, batch=batch, lr=1e-3, solved=solved)
    cold, cst = WarmStart.solve_family(test, params)
    t0 = time.perf_counter()
    xs, ys, sig, used, kkt = ws.predict(test)
    t_pred = time.perf_counter() - t0
    for d, x, y in zip(test, xs, ys):
        d.primal_start, d.dual_start = x, y
    warm, wst = WarmStart.solve_family(test, params, sigma0=sig)
    ic = float(np.mean([r.iterations for r in cold]))
    iw = float(np.mean([r.iterations for r in warm]))
    return {"workload": f"transportation LPs {S}x{D} ({S * D} arcs); {n_train} training optima "
                        f"(relative KKT {label_eps:g}), {n_test} held-out instances solved to 1e-6",
            "epochs": epochs, "batch": batch,
            "label_solve_s": t_label, "train_s": ws.train_sec, "train_loss": ws.train_loss,
            "predict_s": t_pred, "predictions_used": float(np.mean(used)),
            "predicted_point_kkt_median": float(np.median(kkt)),
            "cold_mean_iterations": ic, "warm_mean_iterations": iw, "iteration_ratio": iw / ic,
            "cold_batch_s": sum(s["total_sec"] for s in cst), "warm_batch_s": sum(s["total_sec"] for s in wst),
            "all_optimal": all(r.status == "OPTIMAL" for r in cold + warm)}


def cpu_baseline(data, m, n, nnz, blocks=1, warm=0, single=False):
    """The CPU restatement (oracle port) on every host core: one evaluation
    block (200 iterations) after setup, in the metric's unit; with single,
    also one more block of the same session on one thread."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    s = O.Session(data, {**PARAMS, "sv_max_iter": 20}, SIGMA_PROTOCOL, threads=threads)
    for _ in range(warm):
        s.iterate(200)
    t0 = time.perf_counter()
    done = sum(s.iterate(200) for _ in range(blocks))
    dt = time.perf_counter() - t0
    b_p, b_d = iteration_bytes(m, n, nnz, 8)
    out = {"value": (b_p + b_d) * done / dt / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
           "sample": f"{done} iterations of the same LP and settings (setup excluded) with {threads} threads, "
                     f"{dt / done * 1e3:.1f} ms/iteration",
           "ms_per_iteration": dt / done * 1e3}
    if single:
        s.set_threads(1)
        t0 = time.perf_counter()
        d1 = s.iterate(200)
        dt1 = time.perf_counter() - t0
        out["single_thread"] = {"value": (b_p + b_d) * d1 / dt1 / 1e9, "unit": "GB/s", "cores": 1,
                                "ms_per_iteration": dt1 / d1 * 1e3, "iterations": d1}
    s.close()
    return out


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


def spawn_ranks(n: int) -> int:
    """--gpus N without a launcher: start N local ranks of this same command
    (RANK = LOCAL_RANK = i, WORLD_SIZE = N, rendezvous on 127.0.0.1), one per
    GPU, as torchrun would; rank 0 prints the line.  Returns the worst exit
    code."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    procs = []
    for i in range(n):
        env = {**os.environ, "RANK": str(i), "LOCAL_RANK": str(i), "WORLD_SIZE": str(n),
               "LOCAL_WORLD_SIZE": str(n), "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)}
        procs.append(subprocess.Popen([sys.executable, str(Path(__file__).resolve()), *sys.argv[1:]], env=env))
    return max(abs(p.wait()) for p in procs)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large_lp", choices=list(WORKLOADS))
    ap.add_argument("--lp-only", action="store_true", help="skip the QP, batch and learned-start sections")
    ap.add_argument("--kkt-cap", type=float, default=40.0,
                    help="seconds per form for the large LP's time to relative KKT 1e-6 / 1e-8 (0: skip)")
    ap.add_argument("--cpu-single", action="store_true",
                    help="also time the CPU port on one thread (one more 200-iteration block, ~30 s)")
    ap.add_argument("--learned-full", action="store_true",
                    help="only the learned warm start on the 200 x 200 family: 20,000 training optima, "
                         "2,000 held-out instances (~25 minutes)")
    ap.add_argument("--learned-size", type=int, nargs=4, default=None, metavar=("S", "D", "TRAIN", "TEST"),
                    help="with --learned-full: another family size and split (a quick check of the run)")
    ap.add_argument("--profile", action="store_true", help="only the chosen-form iteration steps (for ncu)")
    ap.add_argument("--profile-section", default="lp", choices=["lp", "qp", "qp_fp32", "batch"],
                    help="with --profile: which solver's kernels to run")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(spawn_ranks(args.gpus))
    rank, world, local = dist_env()
    if args.learned_full:
        S, D, n_train, n_test = args.learned_size or (200, 200, 20_000, 2_000)
        out = bench_learned(local, S, D, n_train, n_test, epochs=60, label_eps=1e-4, batch=256)
        print(json.dumps({"learned_warm_start_full": out}), flush=True)
    elif args.profile:
        run_profile(args, local)
    elif args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
