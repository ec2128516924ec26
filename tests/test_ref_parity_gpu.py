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
    """The alpha pulse (LP/CP_AL/src/solver.cu:885-1032) and the sigma
    trigger (1496-1527) act at the iterations where the reference's acted, as
    its log lines record them: the pulse's gate evaluation and pass/reject,
    the start of its positive block, the trigger's iteration.  This library's
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
