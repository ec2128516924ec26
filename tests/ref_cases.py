"""Seeded cases on which the reference's own CP_AL and FA_CP solvers were run
(tests/golden/make_ref_solver_golden.py writes their results to
tests/golden/ref_solver/), and the helpers that rebuild each instance, the
problem file the reference driver reads (oracle/ref_driver/ref_solve.c), and
the parameters and environment of a case in this library's vocabulary.

Each case:
  name      fixture file stem
  kind      "lp" (CP_AL) or "qp" (FA_CP)
  gen       (generator in pdal_gb300.instances, keyword arguments)
  env       CP_AL_* / FA_CP_* variables set for the run (all others cleared)
  params    solver parameters (pdal_gb300.lp / qp apply_params keys)
  parity    compared with this library (and, if "oracle", with the CPU oracle)
  vectors   the reference's x and y are stored too (small cases)
  timing    what the case measures when it is a reference timing row
"""
from __future__ import annotations

import hashlib
import io
import struct

import numpy as np

# the reference's random-LP protocol (experiments/random_lp/run_random_lp.sbatch:81-97)
SIGMA_PROTOCOL_ENV = {
    "CP_AL_SIGMA_MODE": "1", "CP_AL_SIGMA_ADAPTIVE": "1", "CP_AL_SIGMA_INIT_FACTOR": "0.5",
    "CP_AL_SIGMA_MIN_FACTOR": "1e-4", "CP_AL_SIGMA_MAX_FACTOR": "100", "CP_AL_SIGMA_BALANCE_GAIN": "0",
    "CP_AL_SIGMA_KP": "0.5", "CP_AL_SIGMA_KI": "0", "CP_AL_SIGMA_KD": "0", "CP_AL_SIGMA_UPDATE_MIN": "1e-6",
    "CP_AL_SIGMA_UPDATE_MAX": "1e6", "CP_AL_LAMBDA_FACTOR": "2.01", "CP_AL_LAMBDA": "0",
    "CP_AL_RESTART_SUFFICIENT": "0.2", "CP_AL_RESTART_NECESSARY": "0.8", "CP_AL_RESTART_ARTIFICIAL": "0.36",
    "CP_AL_PROGRESS_LOG_FREQ": "0",
}
LAMBDA0_ENV = {"CP_AL_LAMBDA": "0"}

C0 = ("random_lp", {"m": 2000, "n": 5000, "nnz_per_col": 8, "seed": 0})
SMALL = ("random_lp", {"m": 300, "n": 800, "nnz_per_col": 6, "seed": 17})
P8 = {"eps": 1e-8, "l_inf_ruiz_iterations": 4, "termination_evaluation_frequency": 200}
NOSCALE = ("random_lp", {"m": 200, "n": 500, "nnz_per_col": 5, "seed": 5})
NOSCALE_PARAMS = {"l_inf_ruiz_iterations": 0, "has_pock_chambolle_alpha": False, "bound_objective_rescaling": False}
# the alpha pulse, its gate forced open as the structural tail's rescue solve sets it (LP/CP_AL/src/cli.c:760-763)
PULSE_ENV = {"CP_AL_ALPHA_DIRECT_PULSE": "1", "CP_AL_DETERMINISTIC_PULSE_FORCE": "1"}
# the sigma trigger with thresholds that always hold: it fires at the first evaluation after 2,000 iterations
TRIGGER_ENV = {"CP_AL_SIGMA_TRIGGER": "1", "CP_AL_SIGMA_TRIGGER_MIN_ITERS": "2000", "CP_AL_SIGMA_TRIGGER_PRIMAL": "0",
               "CP_AL_SIGMA_TRIGGER_DUAL": "1", "CP_AL_SIGMA_TRIGGER_RATIO": "0"}

CASES = [
    # CP_AL, the plain FP64 form: status, objective and iteration parity at KKT 1e-8
    dict(name="lp_c0_sigma_protocol", kind="lp", gen=C0, env=SIGMA_PROTOCOL_ENV, params=P8, parity=True,
         vectors=True),
    dict(name="lp_c0_lambda0", kind="lp", gen=C0, env=LAMBDA0_ENV, params=P8, parity=True, vectors=True),
    dict(name="lp_c0_default", kind="lp", gen=C0, env={}, params=P8, parity=True, vectors=True),
    dict(name="lp_small_default", kind="lp", gen=SMALL, env={}, params=P8, parity=True, vectors=True,
         oracle=True),
    dict(name="lp_small_sigma_protocol", kind="lp", gen=SMALL, env=SIGMA_PROTOCOL_ENV, params=P8, parity=True,
         vectors=True, oracle=True),
    dict(name="lp_small_linf_reflect", kind="lp", gen=SMALL, env=LAMBDA0_ENV,
         params={**P8, "linf": True, "reflection_coefficient": 0.7}, parity=True, vectors=True, oracle=True),
    dict(name="lp_small_no_scaling", kind="lp", gen=("random_lp", {"m": 200, "n": 500, "nnz_per_col": 5, "seed": 5}),
         env=LAMBDA0_ENV, params={**P8, "l_inf_ruiz_iterations": 0, "has_pock_chambolle_alpha": False,
                                  "bound_objective_rescaling": False}, parity=True, vectors=True, oracle=True),
    dict(name="lp_small_polish", kind="lp", gen=SMALL, env=LAMBDA0_ENV,
         params={**P8, "eps": 1e-4, "feasibility_polishing": True, "eps_feas_polish": 1e-8}, parity=True,
         vectors=True, oracle=True),
    dict(name="lp_docs_example", kind="lp", gen=("docs_example_lp", {}), env={}, params=P8, parity=True,
         vectors=True, oracle=True),
    dict(name="lp_transport_20x20", kind="lp", gen=("transport_lp", {"supplies": 20, "demands": 20, "seed": 4001}),
         env=SIGMA_PROTOCOL_ENV, params=P8, parity=True, vectors=True, oracle=True),
    dict(name="lp_zipf_20k_lambda0", kind="lp",
         gen=("zipf_lp", {"m": 20000, "n": 40000, "nnz": 400000, "seed": 1000}), env=LAMBDA0_ENV,
         params={**P8, "iteration_limit": 100000}, parity=True),
    dict(name="lp_zipf_20k_sigma_protocol", kind="lp",
         gen=("zipf_lp", {"m": 20000, "n": 40000, "nnz": 400000, "seed": 1000}), env=SIGMA_PROTOCOL_ENV,
         params={**P8, "iteration_limit": 100000}, parity=True),
    dict(name="lp_c4_transport_200x200", kind="lp",
         gen=("transport_lp", {"supplies": 200, "demands": 200, "seed": 4000}), env=SIGMA_PROTOCOL_ENV,
         params={"eps": 1e-6, "l_inf_ruiz_iterations": 4}, parity=True, timing="C4 cold start to 1e-6"),
    # the benchmark controllers (LP/CP_AL/src/solver.cu:885-1032 alpha pulse, 1496-1527 sigma trigger): the
    # iteration at which each acted is read from the reference's own log lines ("controllers" in the fixture)
    dict(name="lp_noscale_pulse", kind="lp", gen=NOSCALE, env={**LAMBDA0_ENV, **PULSE_ENV},
         params={**NOSCALE_PARAMS, "eps": 1e-14, "iteration_limit": 12000}, parity=True, vectors=True, oracle=True,
         controllers=True),
    dict(name="lp_noscale_pulse_gate", kind="lp", gen=NOSCALE,
         env={**LAMBDA0_ENV, "CP_AL_ALPHA_DIRECT_PULSE": "1"},
         params={**NOSCALE_PARAMS, "eps": 1e-14, "iteration_limit": 12000}, parity=True, vectors=True, oracle=True,
         controllers=True),
    dict(name="lp_c0_pulse", kind="lp", gen=C0, env={**LAMBDA0_ENV, **PULSE_ENV},
         params={"eps": 1e-14, "iteration_limit": 13000, "l_inf_ruiz_iterations": 4}, parity=True, vectors=True,
         controllers=True),
    dict(name="lp_c0_pulse_1e-8", kind="lp", gen=C0, env={**LAMBDA0_ENV, **PULSE_ENV}, params=P8, parity=True,
         vectors=True, controllers=True),
    dict(name="lp_small_sigma_trigger", kind="lp", gen=SMALL, env={**LAMBDA0_ENV, **TRIGGER_ENV},
         params={**P8, "verbose": True}, parity=True, vectors=True, oracle=True, controllers=True),
    # the dynamic evaluation frequency (solver.cu:1229-1255, 1529-1583): by the residual test, by the
    # iteration gate, and the bootstrap's short blocks
    dict(name="lp_small_dynamic_eval", kind="lp", gen=SMALL,
         env={**LAMBDA0_ENV, "CP_AL_DYNAMIC_EVAL": "1", "CP_AL_DYNAMIC_EVAL_RATIO": "3",
              "CP_AL_DYNAMIC_EVAL_LARGE_RES": "1e-6"},
         params={**P8, "verbose": True}, parity=True, vectors=True, oracle=True, controllers=True),
    dict(name="lp_small_dynamic_eval_iters", kind="lp", gen=SMALL,
         env={**LAMBDA0_ENV, "CP_AL_DYNAMIC_EVAL_AFTER_ITERS": "1500"}, params=P8, parity=True, vectors=True,
         oracle=True, controllers=True),
    dict(name="lp_small_dynamic_eval_bootstrap", kind="lp", gen=SMALL,
         env={**LAMBDA0_ENV, "CP_AL_DYNAMIC_EVAL": "1", "CP_AL_DYNAMIC_EVAL_BOOTSTRAP_ITERS": "1000"}, params=P8,
         parity=True, vectors=True, oracle=True, controllers=True),
    # reference timing rows (time to relative KKT 1e-6, and per-iteration time on the large LP)
    dict(name="lp_c0_sigma_protocol_1e-6", kind="lp", gen=C0, env=SIGMA_PROTOCOL_ENV,
         params={"eps": 1e-6, "l_inf_ruiz_iterations": 4}, parity=True, timing="C0 to 1e-6"),
    dict(name="lp_c0_default_1e-6", kind="lp", gen=C0, env={}, params={"eps": 1e-6, "l_inf_ruiz_iterations": 4},
         parity=True, timing="C0 to 1e-6 (reference defaults)"),
    # FA_CP (defaults: guarded sigma rule, L-infinity norm)
    dict(name="qp_sparse_small", kind="qp",
         gen=("planted_qp", {"n": 400, "m": 200, "b_rows": 100, "seed": 23, "q_form": "sparse"}),
         env={}, params={"eps": 1e-8}, parity=True, vectors=True, oracle=True),
    dict(name="qp_lowrank_small", kind="qp",
         gen=("planted_qp", {"n": 400, "m": 200, "b_rows": 100, "seed": 29, "q_form": "lowrank"}),
         env={}, params={"eps": 1e-8}, parity=True, vectors=True, oracle=True),
    dict(name="qp_sparse_fixed_sigma", kind="qp",
         gen=("planted_qp", {"n": 400, "m": 200, "b_rows": 100, "seed": 31, "q_form": "sparse"}),
         env={}, params={"eps": 1e-8, "sigma_update_rule": "fixed"}, parity=True, vectors=True, oracle=True),
    dict(name="qp_lp_through_facp", kind="qp", gen=("random_lp", {"m": 300, "n": 800, "nnz_per_col": 6, "seed": 17}),
         env={}, params={"eps": 1e-8}, parity=True, vectors=True, oracle=True),
    # FA_CP feasibility polishing on LPs solved through FA_CP (fa_cp_core_op.cu:1241-1735)
    dict(name="qp_lp_polish", kind="qp", gen=("random_lp", {"m": 300, "n": 800, "nnz_per_col": 6, "seed": 17}),
         env={}, params={"eps": 1e-4, "feasibility_polishing": True, "eps_feas_polish": 1e-8}, parity=True,
         vectors=True, oracle=True),
    dict(name="qp_transport_polish", kind="qp",
         gen=("transport_lp", {"supplies": 20, "demands": 20, "seed": 4001}),
         env={}, params={"eps": 1e-4, "feasibility_polishing": True, "eps_feas_polish": 1e-8}, parity=True,
         vectors=True, oracle=True),
    dict(name="qp_c2_20k", kind="qp",
         gen=("planted_qp", {"n": 20000, "m": 10000, "b_rows": 5000, "seed": 2000, "q_form": "sparse"}),
         env={}, params={"eps": 1e-8}, parity=True),
    dict(name="qp_c2_full_1e-6", kind="qp", gen=("planted_qp", {}), env={}, params={"eps": 1e-6}, parity=True,
         timing="C2 to 1e-6"),
    dict(name="qp_c2_full_1e-8", kind="qp", gen=("planted_qp", {}), env={}, params={"eps": 1e-8}, parity=True,
         timing="C2 to 1e-8"),
]

# The reference's own CP_AL command (oracle/_ref/ref_cp_al_cli) under the paper protocol's one switch
# (LP/CP_AL/run_unified_full856.sbatch:87-89 environment, 110-113 arguments), on MPS files written by
# pdal_gb300.mps.write_lp: one case per route of the unified decision list.  The tail case's iteration limit
# ends the base solve long before its time share, so both phases are deterministic, and its rescue runs
# the forced alpha pulse.
UNIFIED_ENV = {"CP_AL_UNIFIED_POLICY": "1", "CP_AL_ALPHA_DIRECT_PULSE_TRACE": "1", "CP_AL_PROGRESS_LOG_FREQ": "0"}


def _cli_args(eps: float, iters: int) -> list[str]:
    return ["--time_limit", "3600", "--iter_limit", str(iters), "--eps_opt", repr(eps), "--eps_feas", repr(eps),
            "--eval_freq", "200", "--no_presolve"]


CLI_CASES = [
    dict(name="cli_unified_tail_pulse", gen=("transport_lp", {"supplies": 200, "demands": 200, "seed": 4000}),
         env=UNIFIED_ENV, args=_cli_args(1e-10, 12000)),
    dict(name="cli_unified_base_c0", gen=C0, env=UNIFIED_ENV, args=_cli_args(1e-6, 100000)),
    dict(name="cli_unified_zero_equality",
         gen=("random_lp", {"m": 2000, "n": 5000, "nnz_per_col": 8, "seed": 7, "eq_fraction": 0.0}), env=UNIFIED_ENV,
         args=_cli_args(1e-6, 100000)),
    dict(name="cli_unified_lowobj", gen=("sparse_objective_lp", {}), env=UNIFIED_ENV, args=_cli_args(1e-6, 100000)),
    # the feature policy alone, variant trigger_select: the sigma trigger, the dynamic evaluation frequency
    # (which switches to short blocks at 5,200 iterations on this LP) and three-point restart selection at
    # lambda = 0.  The policy's 50 Curtis-Reid passes leave this LP ill-conditioned: rounding differences
    # between any two implementations grow (1e-13 at 1,000 iterations, 1e-9 at 6,000) until a restart decision
    # flips near 20,000, so the case stops at 6,000.
    dict(name="cli_feature_trigger_select", gen=("zipf_lp", {"m": 2000, "n": 4000, "nnz": 40000, "seed": 1000}),
         env={"CP_AL_FEATURE_AUTO_POLICY": "1", "CP_AL_FEATURE_POLICY_VARIANT": "trigger_select",
              "CP_AL_PROGRESS_LOG_FREQ": "0"}, args=_cli_args(1e-6, 6000)),
]
CLI_BY_NAME = {c["name"]: c for c in CLI_CASES}


def cli_events(text: str) -> dict:
    """What the policy layer did, from a CP_AL command's stderr: the unified
    route, the Curtis-Reid effort of each feature-policy application, the
    structural tail's phases (status and iterations of each) and the alpha
    pulse's events."""
    import re

    out = {"route": None, "cr_selected": [int(v) for v in re.findall(r"\[feature-auto-policy\] .*? cr_selected=(\d+)", text)]}
    m = re.search(r"\[unified-policy\] version=2 route=(\S+)", text)
    if m:
        out["route"] = m.group(1)
    for tag in ("base", "rescue"):
        m = re.search(r"\[structural-tail-%s\] status=(\S+) .*? iterations=(\d+)" % tag, text)
        out[tag] = [m.group(1), int(m.group(2))] if m else None
    m = re.search(r"\[structural-tail-final\] phases=(\d) tail_started=(\d) status=(\S+) .*? total_iterations=(\d+)",
                  text)
    out["final"] = [int(m.group(1)), int(m.group(2)), m.group(3), int(m.group(4))] if m else None
    out.update(controller_events(text))
    return out


def read_summary(path) -> dict:
    """A CP_AL command's <name>_summary.txt (LP/CP_AL/src/cli.c:526-586)."""
    from pathlib import Path

    out = {}
    for line in Path(path).read_text().splitlines():
        k, v = line.split(": ", 1)
        out[k] = v
    return out


# the large LP, reference time per iteration: two runs that differ only in the
# iteration limit; (t[hi] - t[lo]) / (hi - lo) removes the setup
C1_TIMING = dict(name="lp_c1_iteration_time", gen=("zipf_lp", {}), env=SIGMA_PROTOCOL_ENV,
                 params={"eps": 1e-12, "l_inf_ruiz_iterations": 4}, limits=(200, 1200))
# the batch, reference one instance at a time: this many evenly spaced instances
C3_SAMPLE = 32

BY_NAME = {c["name"]: c for c in CASES}


def make_instance(gen, kind: str = "lp"):
    """The case's instance: LPData, or QPData for planted_qp (whose extra
    returns are dropped) and for an LP solved by FA_CP (kind "qp")."""
    from pdal_gb300 import instances
    from pdal_gb300.lp import LPData
    from pdal_gb300.qp import QPData

    fn, kw = gen
    out = getattr(instances, fn)(**kw)
    out = out[0] if isinstance(out, tuple) else out
    if kind == "qp" and isinstance(out, LPData):
        out = QPData(c=out.c, A=out.A, con_lb=out.con_lb, con_ub=out.con_ub, var_lb=out.var_lb, var_ub=out.var_ub,
                     c0=out.c0)
    return out


def _csr_arrays(M):
    from pdal_gb300.qp import _csr

    rp, ci, v, shape = _csr(M)
    return rp, ci, v, shape


def problem_bytes(data) -> bytes:
    """The problem file of oracle/ref_driver/ref_solve.c for an LPData or a
    QPData (infinite bounds kept as IEEE infinities)."""
    A = getattr(data, "A", None)
    Q = getattr(data, "Q", None)
    R = getattr(data, "R", None)
    if A is not None:
        arp, aci, av, (m, n) = _csr_arrays(A)
    else:
        m = 0
        n = _csr_arrays(Q if Q is not None else R)[3][1]
        arp, aci, av = np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0)
    f = lambda a, k, fill: (np.ascontiguousarray(a, dtype="<f8") if a is not None else np.full(k, fill, dtype="<f8"))
    buf = io.BytesIO()
    q = _csr_arrays(Q) if Q is not None else None
    r = _csr_arrays(R) if R is not None else None
    buf.write(b"PDALPRB1")
    buf.write(struct.pack("<8i", m, n, len(aci), int(q is not None), len(q[1]) if q else 0, int(r is not None),
                          r[3][0] if r else 0, len(r[1]) if r else 0))
    buf.write(struct.pack("<d", float(data.c0)))
    for a, k, fill in ((data.c, n, 0.0), (data.var_lb, n, -np.inf), (data.var_ub, n, np.inf),
                       (data.con_lb, m, -np.inf), (data.con_ub, m, np.inf)):
        buf.write(f(a, k, fill).tobytes())
    for M in ((arp, aci, av), q, r):
        if M is None:
            continue
        buf.write(np.ascontiguousarray(M[0], dtype="<i4").tobytes())
        buf.write(np.ascontiguousarray(M[1], dtype="<i4").tobytes())
        buf.write(np.ascontiguousarray(M[2], dtype="<f8").tobytes())
    return buf.getvalue()


def instance_sha256(data) -> str:
    return hashlib.sha256(problem_bytes(data)).hexdigest()


_LP_KEYS = {"eps": "eps", "l_inf_ruiz_iterations": "ruiz", "termination_evaluation_frequency": "eval_freq",
            "iteration_limit": "iter_limit", "reflection_coefficient": "reflection",
            "pock_chambolle_alpha": "pc_alpha", "eps_feas_polish": "eps_polish", "sv_max_iter": "sv_max_iter",
            "sv_tol": "sv_tol", "necessary_reduction_for_restart": "necessary", "time_limit": "time_limit"}
SIGMA_RULES = {"fixed": 0, "residual": 1, "kkt": 2, "displacement": 3, "progress": 4, "greedy": 5, "guarded": 6,
               "balanced_guarded": 7}


def driver_args(params: dict) -> list[str]:
    """key=value arguments of the reference driver for a params dict."""
    out = []
    for k, v in params.items():
        if k in _LP_KEYS:
            out.append(f"{_LP_KEYS[k]}={v!r}" if isinstance(v, float) else f"{_LP_KEYS[k]}={v}")
        elif k == "linf":
            out.append(f"linf={int(bool(v))}")
        elif k == "feasibility_polishing":
            out.append(f"polish={int(bool(v))}")
        elif k == "has_pock_chambolle_alpha":
            out.append(f"no_pc={int(not v)}")
        elif k == "bound_objective_rescaling":
            out.append(f"no_bo={int(not v)}")
        elif k == "sigma_update_rule":
            out.append(f"sigma_rule={SIGMA_RULES[v]}")
        elif k == "al_sigma":
            out.append(f"al_sigma={v!r}")
        elif k == "verbose":
            out.append(f"verbose={int(bool(v))}")
        else:
            raise KeyError(f"no driver key for {k!r}")
    return out


def controller_events(text: str) -> dict:
    """The benchmark controllers' actions in a CP_AL log (the reference's
    stderr and stdout, or this library's): the iteration at which the alpha
    pulse started (-1: never), whether its gate was evaluated and passed
    (None: not evaluated), and the iteration at which the sigma trigger fired
    (0: never; printed with verbose output only) and the dynamic evaluation
    frequency switched to short blocks (0: never; printed with verbose output
    or an iteration or time gate)."""
    import re

    out = {"pulse_start": -1, "pulse_gate_pass": None, "pulse_gate_iteration": -1, "sigma_trigger": 0,
           "dynamic_eval": 0}
    m = re.search(r"\[alpha-direct-pulse-start\] charged_iter=(\d+)", text)
    if m:
        out["pulse_start"] = int(m.group(1))
    m = re.search(r"\[alpha-deterministic-tail-anchor\] charged_iter=(\d+).* pass=(\d)", text)
    if m:
        out["pulse_gate_iteration"] = int(m.group(1))
        out["pulse_gate_pass"] = m.group(2) == "1"
    m = re.search(r"sigma-trigger iter (\d+)", text)
    if m:
        out["sigma_trigger"] = int(m.group(1))
    m = re.search(r"\[dynamic-eval\] iter=(\d+)", text)
    if m:
        out["dynamic_eval"] = int(m.group(1))
    return out


def load_fixture(name: str):
    """(result dict, x or None, y or None) of a committed fixture."""
    import json
    from pathlib import Path

    d = Path(__file__).resolve().parent / "golden" / "ref_solver"
    js = json.loads((d / f"{name}.json").read_text())
    x = y = None
    npz = d / f"{name}.npz"
    if npz.exists():
        z = np.load(npz)
        x, y = z["x"], z["y"]
    return js, x, y
