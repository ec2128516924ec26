"""Parity of the plain FP64 form with the reference's own solvers.

The fixtures under tests/golden/ref_solver/ are the reference's CP_AL and
FA_CP solvers (LP/CP_AL/src/solver.cu:1175-1736, QP/FA_CP/src/solver.cu:
74-165, built from their sources and run on a GB300 by
tests/golden/make_ref_solver_golden.py) on the seeded cases of
tests/ref_cases.py.  Each test rebuilds the case's instance, checks that it is
byte for byte the instance the reference solved, solves it through this
library's C entry points with the same parameters and the same CP_AL_*
environment, and asserts the bar the plain form is held to: the same
termination status, primal objective within 1e-8 relative, iteration count
within 2%.  Where the fixture holds the reference's solution vectors, they
are compared too.
"""
from __future__ import annotations

import numpy as np
import pytest

import ref_cases as RC

pytestmark = pytest.mark.gpu

OBJ_TOL = 1e-8      # relative objective difference
ITER_TOL = 0.02     # relative iteration-count difference
VEC_TOL = 1e-6      # solution vectors, relative to 1 + max |x_ref| (solves stop at KKT 1e-8)
CTL_VEC_TOL = 1e-11  # the controller cases' vectors (measured: 1e-14 from the reference's)

LP_CASES = [c["name"] for c in RC.CASES if c["kind"] == "lp" and c.get("parity")]
QP_CASES = [c["name"] for c in RC.CASES if c["kind"] == "qp" and c.get("parity")]


def _fixture(name):
    try:
        return RC.load_fixture(name)
    except FileNotFoundError:
        pytest.fail(f"fixture {name} missing: run tests/golden/make_ref_solver_golden.py")


def _rel(a, b):
    return abs(a - b) / (1.0 + abs(b))


def lp_options_for(env: dict, monkeypatch):
    """This library's options for a case's CP_AL_* environment, read by
    cp_al_gb300_options_from_env exactly as solve_lp_problem reads them."""
    import os

    from pdal_gb300 import _native as N
    from pdal_gb300 import lp

    for k in list(os.environ):
        if k.startswith("CP_AL_") or k.startswith("FA_CP_"):
            monkeypatch.delenv(k)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    o = lp.default_options(from_env=True)
    for k in list(env):
        monkeypatch.delenv(k)
    return o


def _check_vectors(x, y, xr, yr):
    if xr is None:
        return
    ex = np.max(np.abs(x - xr)) / (1.0 + np.max(np.abs(xr))) if xr.size else 0.0
    ey = np.max(np.abs(y - yr)) / (1.0 + np.max(np.abs(yr))) if yr.size else 0.0
    assert ex <= VEC_TOL and ey <= VEC_TOL, (ex, ey)


def _quiet(params: dict) -> dict:
    """A case's parameters without its verbose switch (the reference's log is
    read for the controllers' iterations; this library reports them in its
    statistics)."""
    return {k: v for k, v in params.items() if k != "verbose"}


GATE = {None: 0, True: 1, False: 2}


@pytest.mark.parametrize("name", [c["name"] for c in RC.CASES if c.get("controllers")])
def test_controllers_act_where_the_reference_does(lp_lib, name, monkeypatch, capfd):
    """The alpha pulse (LP/CP_AL/src/solver.cu:885-1032), the sigma trigger
    (1496-1527) and the dynamic evaluation frequency (1529-1583) act at the
    iterations where the reference's acted, as its log lines record them: the
    pulse's gate evaluation and pass/reject, the start of its positive block,
    the trigger's iteration, the switch to short blocks.  This library's
    own pulse lines say the same.  The solution vectors agree with the
    reference's to CTL_VEC_TOL: with the controllers off the same runs end
    1e-10 to 1e-6 away from them, so the check sees what the controllers did.
    Status, objective and iterations are held to the reference by
    test_lp_matches_reference_solver."""
    from pdal_gb300 import lp

    fx, xr, yr = _fixture(name)
    case = RC.BY_NAME[name]
    data = RC.make_instance(case["gen"], case["kind"])
    opts = lp_options_for(case["env"], monkeypatch)
    opts.device = 0
    capfd.readouterr()
    g = lp.solve(data, _quiet(case["params"]), opts)
    err = capfd.readouterr().err
    ev = fx["ref"]["controllers"]
    assert g.stats["pulse_start_iteration"] == ev["pulse_start"], (g.stats["pulse_start_iteration"], ev)
    assert g.stats["pulse_gate"] == GATE[ev["pulse_gate_pass"]], (g.stats["pulse_gate"], ev)
    assert g.stats["sigma_trigger_iteration"] == ev["sigma_trigger"], (g.stats["sigma_trigger_iteration"], ev)
    assert g.stats["dynamic_eval_iteration"] == ev.get("dynamic_eval", 0), (g.stats["dynamic_eval_iteration"], ev)
    if case["env"].get("CP_AL_ALPHA_DIRECT_PULSE") == "1":
        mine = RC.controller_events(err)
        for k in ("pulse_start", "pulse_gate_pass", "pulse_gate_iteration"):
            assert mine[k] == ev[k], (k, mine, ev)
    ex = np.max(np.abs(g.x - xr)) / (1.0 + np.max(np.abs(xr)))
    ey = np.max(np.abs(g.y - yr)) / (1.0 + np.max(np.abs(yr)))
    assert ex <= CTL_VEC_TOL and ey <= CTL_VEC_TOL, (ex, ey)


@pytest.mark.parametrize("name", LP_CASES)
def test_lp_matches_reference_solver(lp_lib, name, monkeypatch):
    from pdal_gb300 import lp

    fx, xr, yr = _fixture(name)
    case = RC.BY_NAME[name]
    data = RC.make_instance(case["gen"], case["kind"])
    assert RC.instance_sha256(data) == fx["instance_sha256"], "instance generator differs from the fixture's"
    opts = lp_options_for(case["env"], monkeypatch)
    opts.device = 0
    g = lp.solve(data, _quiet(case["params"]), opts)
    ref = fx["ref"]
    assert g.status_code == ref["termination_reason"], (g.status, ref["termination_reason"])
    assert _rel(g.primal_objective, ref["primal_objective"]) <= OBJ_TOL, (g.primal_objective, ref["primal_objective"])
    assert abs(g.iterations - ref["iterations"]) <= ITER_TOL * ref["iterations"], (g.iterations, ref["iterations"])
    _check_vectors(g.x, g.y, xr, yr)


@pytest.mark.parametrize("name", QP_CASES)
def test_qp_matches_reference_solver(qp_lib, name, monkeypatch):
    import os

    from pdal_gb300 import qp

    for k in list(os.environ):
        if k.startswith("FA_CP_"):
            monkeypatch.delenv(k)
    fx, xr, yr = _fixture(name)
    case = RC.BY_NAME[name]
    data = RC.make_instance(case["gen"], case["kind"])
    assert RC.instance_sha256(data) == fx["instance_sha256"], "instance generator differs from the fixture's"
    g = qp.solve(data, {**case["params"], "verbose": 0}, {"device": 0})
    ref = fx["ref"]
    assert g.status_code == ref["termination_reason"], (g.status, ref["termination_reason"])
    assert _rel(g.primal_objective, ref["primal_objective"]) <= OBJ_TOL, (g.primal_objective, ref["primal_objective"])
    assert abs(g.iterations - ref["iterations"]) <= ITER_TOL * ref["iterations"], (g.iterations, ref["iterations"])
    _check_vectors(g.x, g.y, xr, yr)


def _cli_fixture(name):
    import json
    from pathlib import Path

    f = Path(__file__).resolve().parent / "golden" / "ref_solver" / f"{name}.json"
    if not f.exists():
        pytest.fail(f"fixture {name} missing: run tests/golden/make_ref_solver_golden.py --cli")
    return json.loads(f.read_text())


@pytest.mark.parametrize("name", [c["name"] for c in RC.CLI_CASES])
def test_cp_al_command_policy_matches_reference_command(tmp_path, lp_lib, name):
    """The paper protocol end to end: this library's `cp_al` command and the
    reference's own command (LP/CP_AL/src/cli.c, built from its sources, run
    on a GB300; fixture) on the same MPS file with CP_AL_UNIFIED_POLICY=1 and
    the runner's arguments take the same route of the unified decision list,
    the same Curtis-Reid effort, the same structural-tail phases (status of
    each, iterations within 2%) and alpha pulse (start iteration), and write
    the same summary (status, iterations within 2%, objective to the printed
    six digits, sizes)."""
    import os
    import subprocess

    from pdal_gb300 import _native as N
    from pdal_gb300 import mps

    fx = _cli_fixture(name)
    case = RC.CLI_BY_NAME[name]
    src = mps.write_lp(RC.make_instance(case["gen"]), tmp_path / f"{name}.mps")
    import hashlib

    assert hashlib.sha256(src.read_bytes()).hexdigest() == fx["mps_sha256"], "MPS text differs from the fixture's"
    out = tmp_path / "out"
    out.mkdir()
    env = {k: v for k, v in os.environ.items() if not k.startswith(("CP_AL_", "FA_CP_"))}
    env.update(case["env"])
    r = subprocess.run([str(N.LIBDIR / "cp_al"), *case["args"], str(src), str(out)], capture_output=True, text=True,
                       env=env, timeout=1800)
    assert r.returncode == 0, r.stderr[-3000:]
    ev, ref = RC.cli_events(r.stderr + "\n" + r.stdout), fx["events"]
    assert ev["route"] == ref["route"] and ev["cr_selected"] == ref["cr_selected"], (ev, ref)
    for tag in ("base", "rescue"):
        assert (ev[tag] is None) == (ref[tag] is None), (tag, ev, ref)
        if ref[tag]:
            assert ev[tag][0] == ref[tag][0], (tag, ev, ref)
            assert abs(ev[tag][1] - ref[tag][1]) <= ITER_TOL * ref[tag][1], (tag, ev, ref)
    assert (ev["final"] is None) == (ref["final"] is None)
    if ref["final"]:
        assert ev["final"][:3] == ref["final"][:3], (ev, ref)
    for k in ("pulse_start", "pulse_gate_pass", "pulse_gate_iteration"):
        assert ev[k] == ref[k], (k, ev, ref)
    s, sr = RC.read_summary(out / f"{name}_summary.txt"), fx["summary"]
    assert s["Termination Reason"] == sr["Termination Reason"]
    it, itr = int(s["Iterations Count"]), int(sr["Iterations Count"])
    assert abs(it - itr) <= ITER_TOL * itr, (it, itr)
    assert _rel(float(s["Primal Objective Value"]), float(sr["Primal Objective Value"])) <= 1e-5
    for k in ("Rows", "Columns", "Nonzeros"):
        assert s[k] == sr[k]
