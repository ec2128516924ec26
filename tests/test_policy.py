"""The CP_AL command's benchmark policy layer (include/cp_al_policy.h,
pdal_gb300/csrc/cp_al_policy.cpp) against the reference's own: the feature,
unified and structural-tail functions of LP/CP_AL/src/cli.c, compiled
unmodified behind oracle/ref_shim/ref_cli_harness.c (oracle/build.py
build_ref).  Both run in this process on the same inputs:

  * the twelve anonymous features of an LP, bit for bit;
  * the unified decision list and the feature policy: the same CP_AL_*
    environment afterwards, the same solver parameters, the same stderr line;
  * the structural tail with its solves scripted (no GPU): the same sequence
    of solves (time limits, evaluation frequency, reflection, the variables
    each solve sees, the warm start), the same combined result and the same
    stderr lines.

No GPU is used; the end-to-end command on a GPU is tests/test_cli_gpu.py.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np
import pytest

from pdal_gb300 import _native as N
from pdal_gb300 import instances as I
from pdal_gb300 import lp

ROOT = Path(__file__).resolve().parents[1]

# every variable a policy reads or sets (LP/CP_AL/src/cli.c:216-470, 588-833)
POLICY_VARS = [
    "CP_AL_UNIFIED_POLICY", "CP_AL_FEATURE_AUTO_POLICY", "CP_AL_FEATURE_POLICY_VARIANT", "CP_AL_FEATURE_CR_ITERS",
    "CP_AL_UNIFIED_EVAL_FREQ", "CP_AL_STRUCTURAL_TAIL_CUT", "CP_AL_TAIL_ONLY_PULSE", "CP_AL_LAMBDA",
    "CP_AL_LAMBDA_FACTOR", "CP_AL_ADAPTIVE_LAMBDA", "CP_AL_LAMBDA_PROFILE", "CP_AL_LAMBDA_GRID", "CP_AL_CR_ITERS",
    "CP_AL_CR_SCALING", "CP_AL_FEATURE_SIGMA_INIT_FACTOR", "CP_AL_FEATURE_SIGMA_TRIGGER_MIN_ITERS",
    "CP_AL_FEATURE_SIGMA_TRIGGER_PRIMAL", "CP_AL_FEATURE_SIGMA_TRIGGER_DUAL", "CP_AL_FEATURE_SIGMA_TRIGGER_RATIO",
    "CP_AL_SIGMA_MODE", "CP_AL_SIGMA_ADAPTIVE", "CP_AL_SIGMA_INIT_FACTOR", "CP_AL_SIGMA_TRIGGER",
    "CP_AL_SIGMA_TRIGGER_MIN_ITERS", "CP_AL_SIGMA_TRIGGER_PRIMAL", "CP_AL_SIGMA_TRIGGER_DUAL",
    "CP_AL_SIGMA_TRIGGER_RATIO", "CP_AL_FEATURE_DYNAMIC_EVAL_FAST", "CP_AL_DYNAMIC_EVAL", "CP_AL_DYNAMIC_EVAL_FAST",
    "CP_AL_DYNAMIC_EVAL_MIN_ITERS", "CP_AL_DYNAMIC_EVAL_SMALL_RES", "CP_AL_DYNAMIC_EVAL_LARGE_RES",
    "CP_AL_DYNAMIC_EVAL_RATIO", "CP_AL_RESTART_SELECT", "CP_AL_RESTART_SELECT_PROFILE", "CP_AL_RESTART_SELECT_MARGIN",
    "CP_AL_RESTART_SUFFICIENT", "CP_AL_RESTART_NECESSARY", "CP_AL_RESTART_ARTIFICIAL", "CP_AL_STEP_MARGIN",
    "CP_AL_ALPHA_DIRECT_PULSE", "CP_AL_DETERMINISTIC_PULSE_FORCE",
]

_libc = C.CDLL(None)
_libc.getenv.restype = C.c_char_p
_libc.getenv.argtypes = [C.c_char_p]
_libc.setenv.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
_libc.unsetenv.argtypes = [C.c_char_p]
_libc.calloc.restype = C.c_void_p
_libc.calloc.argtypes = [C.c_size_t, C.c_size_t]


def c_env() -> dict:
    """The process environment as C code sees it (setenv from a library
    bypasses os.environ)."""
    return {k: _libc.getenv(k.encode()) for k in POLICY_VARS}


def clear_env(preset: dict | None = None):
    import os

    for k in POLICY_VARS:
        os.environ.pop(k, None)
        _libc.unsetenv(k.encode())
    for k, v in (preset or {}).items():
        _libc.setenv(k.encode(), v.encode(), 1)


@pytest.fixture(autouse=True)
def _clean_env():
    clear_env()
    yield
    clear_env()


@pytest.fixture(scope="module")
def ref():
    sys.path.insert(0, str(ROOT))
    from oracle import build as ob

    try:
        built = {p.name: p for p in ob.build_ref()}
    except RuntimeError as e:  # the reference is present but did not compile here
        pytest.skip(str(e))
    if "libref_cli_policy.so" not in built:
        pytest.skip("reference sources absent")
    L = C.CDLL(str(built["libref_cli_policy.so"]))
    _dp = C.POINTER(C.c_double)
    L.ref_cli_feature_stats.argtypes = [C.POINTER(N.LpProblem), _dp]
    L.ref_cli_unified_policy.argtypes = [_dp]
    L.ref_cli_feature_policy.argtypes = [C.POINTER(N.LpProblem), C.POINTER(N.CpalParameters), _dp]
    L.ref_cli_structural_tail.argtypes = [C.POINTER(N.LpProblem), C.POINTER(N.CpalParameters), _dp, C.c_int]
    L.ref_cli_structural_tail.restype = C.POINTER(N.CpalResult)
    L.ref_cli_set_solver.argtypes = [N.SOLVE_FN]
    return L


def stats_array(st: N.FeatureStats) -> np.ndarray:
    return np.array([getattr(st, f) for f, _ in N.FeatureStats._fields_])


def to_stats(a) -> N.FeatureStats:
    st = N.FeatureStats()
    for (f, _), v in zip(N.FeatureStats._fields_, a):
        setattr(st, f, float(v))
    return st


def _dp_of(st: N.FeatureStats):
    return C.cast(C.pointer(st), C.POINTER(C.c_double))


def _crafted_lp() -> lp.LPData:
    """Empty rows and columns, stored zeros, mixed scales and signs, one-sided
    and infinite bounds, zero costs."""
    rng = np.random.default_rng(7)
    m, n = 60, 90
    rows, cols, vals = [], [], []
    for i in range(m):
        if i % 11 == 3:
            continue  # empty row
        k = 1 + (i % 7)
        cs = rng.choice(n - 5, size=k, replace=False)  # the last 5 columns stay empty
        for c in cs:
            rows.append(i)
            cols.append(int(c))
            vals.append(0.0 if (i + c) % 13 == 0 else rng.standard_normal() * 10.0 ** rng.integers(-4, 5))
    import scipy.sparse as sp

    A = sp.csr_matrix((vals, (rows, cols)), shape=(m, n))
    A.sort_indices()
    con_lb = np.where(np.arange(m) % 3 == 0, 1.0, -np.inf)
    con_ub = np.where(np.arange(m) % 3 == 0, 1.0, np.where(np.arange(m) % 3 == 1, 2.0, np.inf))
    var_lb = np.where(np.arange(n) % 4 == 0, -np.inf, 0.0)
    var_ub = np.where(np.arange(n) % 5 == 0, np.inf, 3.0)
    c = np.where(np.arange(n) % 6 == 0, 0.0, rng.standard_normal(n))
    return lp.LPData(c, (A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data, (m, n)), con_lb, con_ub,
                     var_lb, var_ub)


FEATURE_CASES = {
    "random_lp": lambda: I.random_lp(300, 800, 6, seed=17),
    "transport": lambda: I.transport_lp(20, 30, seed=4001),
    "zipf": lambda: I.zipf_lp(2000, 4000, 40000, seed=1000),
    "crafted": _crafted_lp,
}


@pytest.mark.parametrize("case", list(FEATURE_CASES))
def test_feature_stats_match_reference(lp_lib, ref, case):
    """cli.c:90-214: the same twelve features, bit for bit."""
    prob = lp._CProblem(lp_lib, FEATURE_CASES[case]())
    try:
        mine = N.FeatureStats()
        assert lp_lib.cp_al_feature_stats(prob.ptr, C.byref(mine)) == 0
        theirs = (C.c_double * 12)()
        ref.ref_cli_feature_stats(prob.ptr, theirs)
        a, b = stats_array(mine), np.array(theirs[:])
        assert np.array_equal(a, b), np.c_[a, b]
    finally:
        prob.close()


def test_feature_stats_of_an_empty_matrix(lp_lib):
    data = lp.LPData(np.ones(3), (np.zeros(3, np.int32), np.zeros(0, np.int32), np.zeros(0), (2, 3)),
                     np.zeros(2), np.ones(2), np.zeros(3), np.ones(3))
    prob = lp._CProblem(lp_lib, data)
    try:
        st = N.FeatureStats()
        assert lp_lib.cp_al_feature_stats(prob.ptr, C.byref(st)) == 0
        assert not stats_array(st).any()
    finally:
        prob.close()


def _stats(**kw):
    base = dict(coeff_log_range=2.0, row_logmax_std=0.3, col_logmax_std=0.4, row_logspan_mean=0.5,
                col_logspan_mean=0.6, row_span2_fraction=0.1, col_span2_fraction=0.2, row_nnz_cv=0.7, col_nnz_cv=0.3,
                equality_fraction=0.5, two_sided_variable_fraction=0.8, objective_density=0.9)
    base.update(kw)
    return to_stats([base[f] for f, _ in N.FeatureStats._fields_])


UNIFIED_CASES = {
    "lowobj_highcv": _stats(objective_density=0.005, col_nnz_cv=6.0, equality_fraction=0.0),
    "lowobj_highcv_edges": _stats(objective_density=0.01, col_nnz_cv=5.0),
    "zero_equality": _stats(equality_fraction=0.0),
    "tail_route": _stats(equality_fraction=1.0, objective_density=1.0, row_logmax_std=0.0),
    "base_route": _stats(equality_fraction=0.4),
}


@pytest.mark.parametrize("case", list(UNIFIED_CASES))
@pytest.mark.parametrize("preset", [{}, {"CP_AL_FEATURE_CR_ITERS": "9", "CP_AL_UNIFIED_EVAL_FREQ": "300",
                                         "CP_AL_STRUCTURAL_TAIL_CUT": "1"}], ids=["clean", "preset"])
def test_unified_policy_matches_reference(lp_lib, ref, case, preset, capfd):
    """cli.c:401-470: the route and the variables it sets or clears."""
    st = UNIFIED_CASES[case]
    clear_env({"CP_AL_UNIFIED_POLICY": "1", **preset})
    capfd.readouterr()
    ref.ref_cli_unified_policy(_dp_of(st))
    env_ref, err_ref = c_env(), capfd.readouterr().err
    clear_env({"CP_AL_UNIFIED_POLICY": "1", **preset})
    route = lp_lib.cp_al_unified_policy(C.byref(st))
    env_mine, err_mine = c_env(), capfd.readouterr().err
    assert env_mine == env_ref
    assert err_mine == err_ref and route.decode() in err_mine
    clear_env()
    assert lp_lib.cp_al_unified_policy(C.byref(st)) is None  # switched off: nothing set
    assert not any(c_env().values())


FEATURE_POLICY_STATS = {
    "cr5_low_cv": _stats(col_nnz_cv=0.19012745),
    "cr50": _stats(col_nnz_cv=0.3),
    "cr5_narrow_range": _stats(col_nnz_cv=0.5, coeff_log_range=3.222854),
    "cr20": _stats(col_nnz_cv=0.5, coeff_log_range=4.0),
}
FEATURE_POLICY_ENVS = {
    "safe0": {},
    "probe": {"CP_AL_FEATURE_POLICY_VARIANT": "probe"},
    "always_select": {"CP_AL_FEATURE_POLICY_VARIANT": "always_select"},
    "always_noselect": {"CP_AL_FEATURE_POLICY_VARIANT": "always_noselect"},
    "trigger": {"CP_AL_FEATURE_POLICY_VARIANT": "trigger", "CP_AL_FEATURE_SIGMA_TRIGGER_MIN_ITERS": "500"},
    "trigger_select_overrides": {"CP_AL_FEATURE_POLICY_VARIANT": "trigger_select", "CP_AL_FEATURE_CR_ITERS": "-3",
                                 "CP_AL_UNIFIED_EVAL_FREQ": "100", "CP_AL_FEATURE_SIGMA_INIT_FACTOR": "0.5",
                                 "CP_AL_FEATURE_DYNAMIC_EVAL_FAST": "20", "CP_AL_LAMBDA_PROFILE": "mp_race",
                                 "CP_AL_STEP_MARGIN": "0.9"},
    "cr_override_bad_freq": {"CP_AL_FEATURE_CR_ITERS": "7", "CP_AL_UNIFIED_EVAL_FREQ": "abc"},
}


@pytest.mark.parametrize("stats", list(FEATURE_POLICY_STATS))
@pytest.mark.parametrize("envname", list(FEATURE_POLICY_ENVS))
def test_feature_policy_matches_reference(lp_lib, ref, stats, envname, capfd):
    """cli.c:216-399: evaluation frequency and reflection coefficient, the
    Curtis-Reid effort, the variant's sigma / trigger / dynamic-evaluation /
    restart-selection variables and the [feature-auto-policy] line."""
    st = FEATURE_POLICY_STATS[stats]
    env = {"CP_AL_FEATURE_AUTO_POLICY": "1", **FEATURE_POLICY_ENVS[envname]}
    prob = lp._CProblem(lp_lib, I.random_lp(50, 120, 4, seed=3))
    try:
        out = []
        for call in (lambda p: ref.ref_cli_feature_policy(prob.ptr, C.byref(p), _dp_of(st)),
                     lambda p: lp_lib.cp_al_feature_policy(prob.ptr, C.byref(p), C.byref(st))):
            clear_env(env)
            p = lp.default_parameters(lp_lib)
            p.termination_evaluation_frequency, p.reflection_coefficient = 64, 0.4
            capfd.readouterr()
            call(p)
            out.append((p.termination_evaluation_frequency, p.reflection_coefficient, c_env(), capfd.readouterr().err))
        assert out[1] == out[0]
        assert "[feature-auto-policy] version=2" in out[1][3]
        clear_env()
        p = lp.default_parameters(lp_lib)
        assert lp_lib.cp_al_feature_policy(prob.ptr, C.byref(p), C.byref(st)) == 0  # switched off
        assert p.termination_evaluation_frequency == 200 and not any(c_env().values())
    finally:
        prob.close()


# ------------------------------------------------------------ structural tail
TAIL_WATCH = ["CP_AL_ALPHA_DIRECT_PULSE", "CP_AL_DETERMINISTIC_PULSE_FORCE", "CP_AL_FEATURE_CR_ITERS",
              "CP_AL_CR_ITERS", "CP_AL_CR_SCALING", "CP_AL_SIGMA_MODE", "CP_AL_LAMBDA", "CP_AL_RESTART_SELECT"]


class ScriptedSolver:
    """A solve callback that returns the next scripted result and records
    what each solve was given."""

    def __init__(self, script, m, n):
        self.script, self.m, self.n = list(script), m, n
        self.calls = []
        self.fn = N.SOLVE_FN(self._solve)

    def _solve(self, prob, params):
        P, pr = params.contents, prob.contents
        start = None
        if pr.primal_start:
            start = (tuple(pr.primal_start[j] for j in range(self.n)), tuple(pr.dual_start[i] for i in range(self.m)))
        env = c_env()
        self.calls.append((P.termination_criteria.time_sec_limit, P.termination_evaluation_frequency,
                           P.reflection_coefficient, tuple(env[k] for k in TAIL_WATCH), start))
        item = self.script.pop(0) if self.script else None  # an exception must not cross into C
        if item is None:
            return None
        status, sec, iters = item
        addr = _libc.calloc(1, C.sizeof(N.CpalResult))
        r = N.CpalResult.from_address(addr)
        r.termination_reason = status
        r.cumulative_time_sec = sec
        r.rescaling_time_sec = 0.25
        r.total_count = iters
        r.feasibility_polishing_time = 0.0
        k = len(self.calls)
        x = _libc.calloc(self.n, 8)
        y = _libc.calloc(self.m, 8)
        for j in range(self.n):
            C.c_double.from_address(x + 8 * j).value = k + 0.001 * j
        for i in range(self.m):
            C.c_double.from_address(y + 8 * i).value = -k - 0.002 * i
        r.primal_solution = C.cast(x, C.POINTER(C.c_double))
        r.dual_solution = C.cast(y, C.POINTER(C.c_double))
        return addr


OPT, TIME, ITER = 1, 5, 6  # termination_reason_t
TAIL_STATS = {
    "high_equality": _stats(objective_density=1.0, row_logmax_std=0.0, equality_fraction=1.0),
    "low_equality": _stats(objective_density=0.995, row_logmax_std=0.05, equality_fraction=0.0),
    "no_match": _stats(objective_density=1.0, row_logmax_std=0.2, equality_fraction=1.0),
}
TAIL_SCENARIOS = [
    ("no_match", 1, 100.0, [(ITER, 30.0, 5000)]),
    ("high_equality", 1, 100.0, [(OPT, 1.0, 800)]),
    ("high_equality", 1, 100.0, [(TIME, 5.0, 9000), (OPT, 20.0, 12000)]),
    ("high_equality", 0, 100.0, [(ITER, 2.0, 9000), (ITER, 40.0, 30000)]),
    ("low_equality", 1, 80.0, [(ITER, 50.0, 7000), (OPT, 3.0, 400)]),
    ("low_equality", 1, 80.0, [(TIME, 81.0, 7000)]),
    ("high_equality", 1, 60.0, [(TIME, 3.0, 9000), None]),
    ("high_equality", 1, float("inf"), [(OPT, 1.0, 800)]),
]


@pytest.mark.parametrize("sc", range(len(TAIL_SCENARIOS)))
def test_structural_tail_matches_reference(lp_lib, ref, sc, capfd):
    """cli.c:607-831 with scripted solves: which solves run with which time
    limit, evaluation frequency, reflection, controller variables and warm
    start, the combined result, and the stderr lines (the rescue's policy
    time, a clock reading, masked)."""
    import re

    stats_name, pulse, limit, script = TAIL_SCENARIOS[sc]
    st = TAIL_STATS[stats_name]
    data = I.random_lp(8, 12, 3, seed=11)
    m, n = 8, 12
    outcomes = []
    for impl in ("ref", "mine"):
        clear_env({"CP_AL_FEATURE_AUTO_POLICY": "1", "CP_AL_UNIFIED_EVAL_FREQ": "100"})
        prob = lp._CProblem(lp_lib, data)
        solver = ScriptedSolver(script, m, n)
        p = lp.default_parameters(lp_lib)
        p.termination_criteria.time_sec_limit = limit
        p.termination_evaluation_frequency = 100
        capfd.readouterr()
        try:
            if impl == "ref":
                ref.ref_cli_set_solver(solver.fn)
                rp = ref.ref_cli_structural_tail(prob.ptr, C.byref(p), _dp_of(st), pulse)
            else:
                lp_lib.cp_al_policy_set_solver(solver.fn)
                rp = lp_lib.cp_al_structural_tail(prob.ptr, C.byref(p), C.byref(st), pulse)
            err = re.sub(r"policy_sec=\S+", "policy_sec=*", capfd.readouterr().err)
            res = None
            if rp:
                r = rp.contents
                res = (r.termination_reason, r.total_count, r.cumulative_time_sec, r.rescaling_time_sec,
                       r.presolve_time, r.feasibility_polishing_time, r.primal_solution[0], r.dual_solution[m - 1])
                lp_lib.cp_al_result_free(rp)
            outcomes.append((solver.calls, res, err, c_env()))
        finally:
            lp_lib.cp_al_policy_set_solver(N.SOLVE_FN(0))
            ref.ref_cli_set_solver(N.SOLVE_FN(0))
            prob.close()
    assert outcomes[1][0] == outcomes[0][0]  # the solves and what each was given
    assert outcomes[1][1] == outcomes[0][1]  # the result
    assert outcomes[1][2] == outcomes[0][2]  # the log lines
    assert outcomes[1][3] == outcomes[0][3]  # the environment left behind
    calls = outcomes[1][0]
    if len(calls) == 2:  # a rescue: warm-started at the base point, the pulse as requested
        assert calls[1][4] is not None and calls[1][4][0][0] == 1.0
        assert calls[1][3][0] == (b"1" if pulse else b"0") and calls[1][1] == 200
