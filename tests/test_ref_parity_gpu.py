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


@pytest.mark.parametrize("name", LP_CASES)
def test_lp_matches_reference_solver(lp_lib, name, monkeypatch):
    from pdal_gb300 import lp

    fx, xr, yr = _fixture(name)
    case = RC.BY_NAME[name]
    data = RC.make_instance(case["gen"], case["kind"])
    assert RC.instance_sha256(data) == fx["instance_sha256"], "instance generator differs from the fixture's"
    opts = lp_options_for(case["env"], monkeypatch)
    opts.device = 0
    g = lp.solve(data, case["params"], opts)
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
