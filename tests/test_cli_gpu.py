"""The drop-in commands end to end on the GPU: an LP written as MPS through
`cp_al` and a QP written as QPS through `fa_cp` give the same solution files
as the library called directly on the same data (the kernels' reductions are
deterministic, so the files match to the last printed digit), in the
reference's output formats (LP/CP_AL/src/cli.c:472-586,
QP/FA_CP/src/cli.c:112-170)."""
import os
import subprocess

import numpy as np
import pytest

from pdal_gb300 import _native as N
from pdal_gb300 import instances, lp, mps, qp

pytestmark = pytest.mark.gpu

LP_KEYS = ["Termination Reason", "Precondition time (sec)", "Runtime (sec)", "Iterations Count",
           "Primal Objective Value", "Dual Objective Value", "Relative Primal Residual", "Relative Dual Residual",
           "Absolute Objective Gap", "Relative Objective Gap", "Rows", "Columns", "Nonzeros"]
QP_KEYS = ["Termination Reason", "Runtime (sec)", "Iterations Count", "Inner Iterations Count",
           "Primal Objective Value", "Dual Objective Value", "Relative Primal Residual", "Relative Dual Residual",
           "Absolute Objective Gap", "Relative Objective Gap", "Final AL Sigma", "Sigma Update Rule",
           "Sigma Update Count", "Rows", "Columns", "Nonzeros"]


def clean_env():
    env = {k: v for k, v in os.environ.items() if not k.startswith(("CP_AL_", "FA_CP_"))}
    return env


def summary(path):
    out = {}
    for line in path.read_text().splitlines():
        k, v = line.split(": ", 1)
        out[k] = v
    return out


def fmt(v):
    return ["%.10g" % x for x in v]


def test_cp_al_command_matches_library(tmp_path, lp_lib):
    data = instances.batch_lps(count=1, seed=77, m_range=(600, 601))[0]
    src = mps.write_lp(data, tmp_path / "planted_lp.mps")
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(N.LIBDIR / "cp_al"), "--eps_opt", "1e-7", "--eps_feas", "1e-7", "--l_inf_ruiz_iter", "4",
                        "--no_presolve", str(src), str(out)], capture_output=True, text=True, env=clean_env(),
                       timeout=300)
    assert r.returncode == 0, r.stderr
    s = summary(out / "planted_lp_summary.txt")
    assert list(s) == LP_KEYS
    assert s["Termination Reason"] == "OPTIMAL"
    d = mps.read_lp(src)
    prm = {"eps": 1e-7, "l_inf_ruiz_iterations": 4, "presolve": False}
    res = lp.solve(d, prm, lp.default_options(lp_lib, from_env=True))
    assert int(s["Iterations Count"]) == res.iterations
    assert s["Primal Objective Value"] == "%e" % res.primal_objective
    x = (out / "planted_lp_primal_solution.txt").read_text().split()
    y = (out / "planted_lp_dual_solution.txt").read_text().split()
    assert x == fmt(res.x) and y == fmt(res.y)
    m, n = d.csr()[3]
    assert int(s["Rows"]) == m and int(s["Columns"]) == n


def test_fa_cp_command_matches_library(tmp_path, qp_lib):
    data, _, f_star = instances.planted_qp(n=400, m=200, b_rows=100, seed=29, q_form="sparse")
    src = mps.write_qp(data, tmp_path / "planted_qp.qps")
    back = mps.read_qp(src)
    out = tmp_path / "out"
    out.mkdir()
    traj = tmp_path / "traj.csv"
    r = subprocess.run([str(N.LIBDIR / "fa_cp"), "-v", "0", "--eps_opt", "1e-8", "--eps_feas", "1e-8",
                        "--trajectory_csv", str(traj), str(src), str(out)], capture_output=True, text=True,
                       env=clean_env(), timeout=300)
    assert r.returncode == 0, r.stderr
    s = summary(out / "planted_qp_summary.txt")
    assert list(s) == QP_KEYS
    assert s["Termination Reason"] == "OPTIMAL" and s["Sigma Update Rule"] == "guarded"
    res = qp.solve(back, {"eps": 1e-8, "verbose": 0})
    assert int(s["Iterations Count"]) == res.iterations
    assert abs(res.primal_objective - f_star) <= 1e-6 * (1 + abs(f_star))
    x = (out / "planted_qp_primal_solution.txt").read_text().split()
    assert x == fmt(res.x)
    rows = traj.read_text().splitlines()
    assert rows[0] == ("iteration,time_sec,rel_primal,rel_dual,rel_gap,kkt_residual,fixed_point_residual,restart,"
                       "al_sigma,sigma_update_count")
    body = [r.split(",") for r in rows[1:]]
    assert body[0][0] == "0" and body[0][6] == "nan"
    assert int(body[-1][0]) == res.iterations
    its = [int(b[0]) for b in body]
    assert its == sorted(its)
    kkt = [float(b[5]) for b in body]
    assert kkt[-1] <= 1e-8


def test_cp_al_command_feasibility_polishing(tmp_path, lp_lib):
    data = instances.random_lp(300, 800, 6, seed=17)
    src = mps.write_lp(data, tmp_path / "loose.mps")
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(N.LIBDIR / "cp_al"), "-f", "--eps_opt", "1e-3", "--eps_feas", "1e-3", "--eps_feas_polish",
                        "1e-8", "--l_inf_ruiz_iter", "4", str(src), str(out)], capture_output=True, text=True,
                       env=clean_env(), timeout=300)
    assert r.returncode == 0, r.stderr
    s = summary(out / "loose_summary.txt")
    assert list(s) == LP_KEYS + ["Feasibility Polishing Time (sec)", "Feasibility Polishing Iteration Count"]
    assert float(s["Relative Primal Residual"]) <= 1e-8 and float(s["Relative Dual Residual"]) <= 1e-8
    assert int(s["Feasibility Polishing Iteration Count"]) > 0
