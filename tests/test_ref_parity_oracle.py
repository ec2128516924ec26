"""The CPU oracle pinned on the reference's own solvers.

The fixtures under tests/golden/ref_solver/ hold what the reference's CP_AL
and FA_CP solvers (built from their sources, run on a GB300 by
tests/golden/make_ref_solver_golden.py) returned on the seeded cases of
tests/ref_cases.py.  Here the oracle (oracle/cpal_oracle.cpp,
oracle/facp_oracle.cpp) solves the small cases on the CPU and must agree with
the reference on termination status, primal objective (1e-8 relative) and
iteration count (2%), so the restatement the GPU tests are checked against is
itself checked against the reference, not only against known optima.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import ref_cases as RC

ORACLE_LP = [c["name"] for c in RC.CASES if c["kind"] == "lp" and c.get("oracle")]
ORACLE_QP = [c["name"] for c in RC.CASES if c["kind"] == "qp" and c.get("oracle")]


def _rel(a, b):
    return abs(a - b) / (1.0 + abs(b))


def _options_from_env(env: dict, monkeypatch) -> dict:
    """The options a CP_AL_* environment means (cp_al_gb300_options_from_env
    of the library; only its parsing is used, no device call)."""
    from pdal_gb300 import _native as N
    from pdal_gb300 import lp

    for k in list(os.environ):
        if k.startswith("CP_AL_") or k.startswith("FA_CP_"):
            monkeypatch.delenv(k)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    o = lp.default_options(from_env=True)
    for k in env:
        monkeypatch.delenv(k)
    d = {f: getattr(o, f) for f, _ in N.CpalOptions._fields_}
    # apply_options reads a "sigma" / "lambda_param" key as an explicit value
    if not o.sigma_set:
        del d["sigma"]
    if not o.lambda_param_set:
        del d["lambda_param"]
    return d


@pytest.mark.parametrize("name", [c["name"] for c in RC.CASES if c.get("parity")])
def test_fixture_instance_is_the_generated_one(name):
    """Every fixture records the sha256 of the problem the reference solved;
    the generators must still produce it (checked for the cheap cases)."""
    fx, _, _ = RC.load_fixture(name)
    case = RC.BY_NAME[name]
    if case["gen"][0] in ("zipf_lp", "planted_qp") and case["gen"][1].get("n", 200_000) > 20000:
        pytest.skip("large instance: checked by the GPU parity test")
    assert RC.instance_sha256(RC.make_instance(case["gen"], case["kind"])) == fx["instance_sha256"]


def _quiet(params: dict) -> dict:
    return {k: v for k, v in params.items() if k != "verbose"}


@pytest.mark.parametrize("name", [c["name"] for c in RC.CASES if c.get("oracle") and c.get("controllers")])
def test_oracle_controllers_act_where_the_reference_does(lp_lib, name, monkeypatch):
    """The oracle's alpha pulse, sigma trigger and dynamic evaluation frequency
    act at the iterations where the reference's did (its log lines, recorded in the fixture), and its
    solution vectors agree with the reference's to 1e-11 (1e-10 to 1e-6 apart
    with the controllers off)."""
    from oracle import oracle as O

    fx, xr, yr = RC.load_fixture(name)
    case = RC.BY_NAME[name]
    data = RC.make_instance(case["gen"], case["kind"])
    o = O.solve_lp(data, _quiet(case["params"]), _options_from_env(case["env"], monkeypatch))
    ev = fx["ref"]["controllers"]
    assert o.stats["pulse_start_iteration"] == ev["pulse_start"], (o.stats, ev)
    assert o.stats["pulse_gate"] == {None: 0, True: 1, False: 2}[ev["pulse_gate_pass"]], (o.stats, ev)
    assert o.stats["sigma_trigger_iteration"] == ev["sigma_trigger"], (o.stats, ev)
    assert o.stats["dynamic_eval_iteration"] == ev.get("dynamic_eval", 0), (o.stats, ev)
    assert np.max(np.abs(o.x - xr)) / (1.0 + np.max(np.abs(xr))) <= 1e-11
    assert np.max(np.abs(o.y - yr)) / (1.0 + np.max(np.abs(yr))) <= 1e-11


@pytest.mark.parametrize("name", ORACLE_LP)
def test_oracle_lp_matches_reference_solver(lp_lib, name, monkeypatch):
    from oracle import oracle as O

    fx, xr, yr = RC.load_fixture(name)
    case = RC.BY_NAME[name]
    data = RC.make_instance(case["gen"], case["kind"])
    o = O.solve_lp(data, _quiet(case["params"]), _options_from_env(case["env"], monkeypatch))
    ref = fx["ref"]
    assert o.status_code == ref["termination_reason"], (o.status, ref["termination_reason"])
    assert _rel(o.primal_objective, ref["primal_objective"]) <= 1e-8, (o.primal_objective, ref["primal_objective"])
    assert abs(o.iterations - ref["iterations"]) <= 0.02 * ref["iterations"], (o.iterations, ref["iterations"])
    if xr is not None:
        assert np.max(np.abs(o.x - xr)) / (1.0 + np.max(np.abs(xr))) <= 1e-6


@pytest.mark.parametrize("name", ORACLE_QP)
def test_oracle_qp_matches_reference_solver(name):
    from oracle import oracle as O

    fx, xr, yr = RC.load_fixture(name)
    case = RC.BY_NAME[name]
    data = RC.make_instance(case["gen"], case["kind"])
    o = O.solve_qp(data, case["params"])
    ref = fx["ref"]
    assert o.status_code == ref["termination_reason"], (o.status, ref["termination_reason"])
    assert _rel(o.primal_objective, ref["primal_objective"]) <= 1e-8, (o.primal_objective, ref["primal_objective"])
    assert abs(o.iterations - ref["iterations"]) <= 0.02 * ref["iterations"], (o.iterations, ref["iterations"])
    if xr is not None:
        assert np.max(np.abs(o.x - xr)) / (1.0 + np.max(np.abs(xr))) <= 1e-6


@pytest.mark.parametrize("name", [c["name"] for c in RC.CASES if c.get("oracle") and c["params"].get("feasibility_polishing")])
def test_oracle_polishing_iterations_match_reference(lp_lib, name):
    """The polishing phases' iteration count (result feasibility_iteration)
    equals the reference's."""
    from oracle import oracle as O

    fx, _, _ = RC.load_fixture(name)
    case = RC.BY_NAME[name]
    data = RC.make_instance(case["gen"], case["kind"])
    if case["kind"] == "qp":
        o = O.solve_qp(data, case["params"])
    else:
        o = O.solve_lp(data, case["params"])
    assert o.stats["feasibility_iteration"] == fx["ref"]["feasibility_iteration"]
