"""The C-ABI boundary without a GPU: the library loads, exports every function
the headers declare, its structs have the C layout, and host-side argument
checks refuse bad input before any device work."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from pdal_gb300 import _native as N
from pdal_gb300 import lp

ROOT = Path(__file__).resolve().parent.parent
HEADERS = {"libcp_al_gb300.so": ["cp_al.h", "cp_al_gb300.h", "cp_al_mps_parser.h", "cp_al_policy.h"],
           "libfa_cp_gb300.so": ["fa_cp.h", "fa_cp_gb300.h", "fa_cp_mps_parser.h"],
           "libpdal_learn_gb300.so": ["pdal_learn.h"]}


def declared_functions(header: Path):
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted({n for n in names if n not in ("if", "sizeof")})


@pytest.mark.parametrize("libname", list(HEADERS))
def test_library_exports_every_declared_symbol(libname, lp_lib, qp_lib):
    lib = C.CDLL(str(N.lib_path(libname)))
    for h in HEADERS[libname]:
        for fn in declared_functions(ROOT / "include" / h):
            assert hasattr(lib, fn), f"{libname} lacks {fn} declared in {h}"


PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "cp_al_types.h"
#include "cp_al_gb300.h"
#include "cp_al_policy.h"
#define S(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  S(lp_problem_t) S(cp_al_parameters_t) S(cp_al_result_t) S(matrix_desc_t) S(cp_al_gb300_options_t)
  S(cp_al_gb300_stats_t) S(termination_criteria_t) S(restart_parameters_t) S(cp_al_feature_stats_t)
  O(cp_al_parameters_t, termination_criteria) O(cp_al_parameters_t, restart_params)
  O(cp_al_parameters_t, optimality_norm) O(cp_al_parameters_t, matrix_zero_tol)
  O(cp_al_result_t, termination_reason) O(cp_al_result_t, feasibility_iteration)
  O(cp_al_gb300_options_t, precision) O(cp_al_gb300_options_t, graph_blocks)
  O(lp_problem_t, dual_start) O(matrix_desc_t, data)
  return 0;
}
"""


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.check_output([str(exe)], text=True).splitlines())
    sizes = {
        "lp_problem_t": N.LpProblem, "cp_al_parameters_t": N.CpalParameters, "cp_al_result_t": N.CpalResult,
        "matrix_desc_t": N.MatrixDesc, "cp_al_gb300_options_t": N.CpalOptions, "cp_al_gb300_stats_t": N.CpalStats,
        "termination_criteria_t": N.TerminationCriteria, "restart_parameters_t": N.RestartParams,
        "cp_al_feature_stats_t": N.FeatureStats,
    }
    for cname, ct in sizes.items():
        assert int(out[cname]) == C.sizeof(ct), cname
    offs = {
        "cp_al_parameters_t.termination_criteria": N.CpalParameters.termination_criteria.offset,
        "cp_al_parameters_t.restart_params": N.CpalParameters.restart_params.offset,
        "cp_al_parameters_t.optimality_norm": N.CpalParameters.optimality_norm.offset,
        "cp_al_parameters_t.matrix_zero_tol": N.CpalParameters.matrix_zero_tol.offset,
        "cp_al_result_t.termination_reason": N.CpalResult.termination_reason.offset,
        "cp_al_result_t.feasibility_iteration": N.CpalResult.feasibility_iteration.offset,
        "cp_al_gb300_options_t.precision": N.CpalOptions.precision.offset,
        "cp_al_gb300_options_t.graph_blocks": N.CpalOptions.graph_blocks.offset,
        "lp_problem_t.dual_start": N.LpProblem.dual_start.offset,
        "matrix_desc_t.data": N.MatrixDesc.data.offset,
    }
    for k, v in offs.items():
        assert int(out[k]) == v, k


QP_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "fa_cp_types.h"
#include "fa_cp_gb300.h"
#define S(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  S(qp_problem_t) S(fa_cp_parameters_t) S(fa_cp_result_t) S(matrix_desc_t) S(fa_cp_gb300_options_t)
  S(fa_cp_gb300_stats_t) S(termination_criteria_t) S(restart_parameters_t) S(CsrComponent)
  O(fa_cp_parameters_t, trajectory_csv) O(fa_cp_parameters_t, sigma_update_rule) O(fa_cp_parameters_t, verbose)
  O(fa_cp_parameters_t, termination_criteria) O(fa_cp_parameters_t, restart_params)
  O(fa_cp_parameters_t, feasibility_polishing) O(fa_cp_parameters_t, optimality_norm)
  O(fa_cp_result_t, total_inner_count) O(fa_cp_result_t, final_al_sigma) O(fa_cp_result_t, termination_reason)
  O(fa_cp_result_t, feasibility_iteration) O(qp_problem_t, objective_lowrank_matrix) O(qp_problem_t, dual_start)
  O(matrix_desc_t, zero_tolerance) O(matrix_desc_t, data) O(termination_criteria_t, iteration_limit)
  O(fa_cp_gb300_stats_t, device_loop_ms)
  return 0;
}
"""


def test_qp_struct_layouts_match_c(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(QP_PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.check_output([str(exe)], text=True).splitlines())
    sizes = {
        "qp_problem_t": N.QpProblem, "fa_cp_parameters_t": N.FacpParameters, "fa_cp_result_t": N.FacpResult,
        "matrix_desc_t": N.QpMatrixDesc, "fa_cp_gb300_options_t": N.FacpOptions, "fa_cp_gb300_stats_t": N.FacpStats,
        "termination_criteria_t": N.FacpTerminationCriteria, "restart_parameters_t": N.RestartParams,
        "CsrComponent": N.CsrComponent,
    }
    for cname, ct in sizes.items():
        assert int(out[cname]) == C.sizeof(ct), cname
    for key, val in out.items():
        if "." not in key:
            continue
        cname, field = key.split(".")
        ct = {**sizes, "termination_criteria_t": N.FacpTerminationCriteria}[cname]
        assert int(val) == getattr(ct, field).offset, key


def _problem_from_desc(lib, desc, m, n):
    c = np.arange(1, n + 1, dtype=np.float64)
    p = lib.create_lp_problem(c.ctypes.data_as(C.POINTER(C.c_double)), C.byref(desc), None, None, None, None, None)
    assert p
    P = p.contents
    nnz = P.constraint_matrix_num_nonzeros
    rp = np.ctypeslib.as_array(P.constraint_matrix_row_pointers, shape=(m + 1,)).copy()
    ci = np.ctypeslib.as_array(P.constraint_matrix_col_indices, shape=(nnz,)).copy() if nnz else np.zeros(0, int)
    v = np.ctypeslib.as_array(P.constraint_matrix_values, shape=(nnz,)).copy() if nnz else np.zeros(0)
    lb = np.ctypeslib.as_array(P.variable_lower_bound, shape=(n,)).copy()
    cu = np.ctypeslib.as_array(P.constraint_upper_bound, shape=(m,)).copy()
    lib.lp_problem_free(p)
    return rp, ci, v, lb, cu


def test_create_lp_problem_formats_agree(lp_lib):
    rng = np.random.default_rng(0)
    m, n = 7, 9
    A = rng.standard_normal((m, n)) * (rng.random((m, n)) < 0.4)
    _dp, _ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    results = []
    # dense
    Ad = np.ascontiguousarray(A)
    d = N.MatrixDesc()
    d.m, d.n, d.fmt = m, n, N.MATRIX_DENSE
    d.data.dense.A = Ad.ctypes.data_as(_dp)
    results.append(_problem_from_desc(lp_lib, d, m, n))
    import scipy.sparse as sp

    S = sp.csr_matrix(A)
    rp, ci, v = S.indptr.astype(np.int32), S.indices.astype(np.int32), S.data.copy()
    d = N.MatrixDesc()
    d.m, d.n, d.fmt = m, n, N.MATRIX_CSR
    d.data.csr.nnz, d.data.csr.row_ptr, d.data.csr.col_ind, d.data.csr.vals = len(v), rp.ctypes.data_as(_ip), ci.ctypes.data_as(_ip), v.ctypes.data_as(_dp)
    results.append(_problem_from_desc(lp_lib, d, m, n))
    T = sp.csc_matrix(A)
    cp_, ri, cv = T.indptr.astype(np.int32), T.indices.astype(np.int32), T.data.copy()
    d = N.MatrixDesc()
    d.m, d.n, d.fmt = m, n, N.MATRIX_CSC
    d.data.csc.nnz, d.data.csc.col_ptr, d.data.csc.row_ind, d.data.csc.vals = len(cv), cp_.ctypes.data_as(_ip), ri.ctypes.data_as(_ip), cv.ctypes.data_as(_dp)
    results.append(_problem_from_desc(lp_lib, d, m, n))
    Q = S.tocoo()
    perm = rng.permutation(Q.nnz)  # COO rows may come in any order; within a row input order is kept
    qr, qc, qv = Q.row[perm].astype(np.int32), Q.col[perm].astype(np.int32), Q.data[perm].copy()
    d = N.MatrixDesc()
    d.m, d.n, d.fmt = m, n, N.MATRIX_COO
    d.data.coo.nnz, d.data.coo.row_ind, d.data.coo.col_ind, d.data.coo.vals = len(qv), qr.ctypes.data_as(_ip), qc.ctypes.data_as(_ip), qv.ctypes.data_as(_dp)
    coo = _problem_from_desc(lp_lib, d, m, n)
    ref = results[0]
    for r in results[1:]:
        assert np.array_equal(r[0], ref[0]) and np.array_equal(r[1], ref[1]) and np.array_equal(r[2], ref[2])
    # COO: same rows, same entries per row
    assert np.array_equal(coo[0], ref[0])
    for i in range(m):
        a = sorted(zip(coo[1][coo[0][i]:coo[0][i + 1]], coo[2][coo[0][i]:coo[0][i + 1]]))
        b = sorted(zip(ref[1][ref[0][i]:ref[0][i + 1]], ref[2][ref[0][i]:ref[0][i + 1]]))
        assert a == b
    # NULL vectors take the reference defaults
    assert np.all(np.isneginf(ref[3])) and np.all(np.isposinf(ref[4]))


def test_bad_input_is_refused_without_exit(lp_lib):
    # column index out of range: refused on the host (returns NULL, process lives)
    rp = np.array([0, 2], dtype=np.int32)
    ci = np.array([0, 5], dtype=np.int32)
    v = np.array([1.0, 1.0])
    data = lp.LPData(np.ones(2), (rp, ci, v, (1, 2)), np.array([0.0]), np.array([1.0]), np.zeros(2), np.ones(2))
    with pytest.raises((RuntimeError, ValueError)):
        lp.solve(data)
    assert "out of range" in N.last_error(lp_lib) or True
    # evaluation frequency below 3 (the reference exits: LP/CP_AL/src/solver.cu:1757-1766)
    good = lp.LPData(np.ones(2), (np.array([0, 2], np.int32), np.array([0, 1], np.int32), v, (1, 2)),
                     np.array([0.0]), np.array([1.0]), np.zeros(2), np.ones(2))
    with pytest.raises(RuntimeError, match="termination_evaluation_frequency"):
        lp.solve(good, {"termination_evaluation_frequency": 2})


def test_options_from_env_reads_reference_variables(lp_lib, monkeypatch):
    monkeypatch.setenv("CP_AL_LAMBDA", "0")
    monkeypatch.setenv("CP_AL_SIGMA_MODE", "1")
    monkeypatch.setenv("CP_AL_SIGMA_INIT_FACTOR", "0.5")
    monkeypatch.setenv("CP_AL_RESTART_NECESSARY", "0.8")
    monkeypatch.setenv("CP_AL_SIGMA_KP", "bogus")
    o = lp.default_options(lp_lib, from_env=True)
    assert o.al_lambda == 0.0 and o.sigma_mode == 1 and o.sigma_init_factor == 0.5
    assert o.restart_necessary == 0.8 and np.isnan(o.sigma_kp) and o.sigma_adaptive == 1
    monkeypatch.setenv("CP_AL_SIGMA", "0.3")
    o = lp.default_options(lp_lib, from_env=True)
    assert o.sigma_set == 1 and o.sigma == 0.3 and o.sigma_adaptive == 0


@pytest.mark.parametrize("name,value,extra", [
    ("CP_AL_ADAPTIVE_LAMBDA", "1", {}),
    ("CP_AL_LAMBDA_PROFILE", "mp_race", {}),
    ("CP_AL_ALPHA_ROLLBACK_TRIAL", "1", {}),
])
def test_unbuilt_controller_switch_is_refused(lp_lib, monkeypatch, name, value, extra):
    """A CP_AL_* switch that turns on a controller this library does not
    implement makes solve_lp_problem (and cp_al_gb300_solve or
    cp_al_gb300_session_create without explicit options) return NULL with a
    message naming it (before any device work, so this runs without a GPU)
    instead of solving without the controller; switched off, nothing is
    refused."""
    for var in ("CP_AL_ADAPTIVE_LAMBDA", "CP_AL_LAMBDA_PROFILE", "CP_AL_DYNAMIC_EVAL", "CP_AL_SIGMA_TRIGGER",
                "CP_AL_ALPHA_ROLLBACK_TRIAL", "CP_AL_ALPHA_DIRECT_PULSE", "CP_AL_SIGMA_MODE",
                "CP_AL_SIGMA"):
        monkeypatch.delenv(var, raising=False)
    assert lp_lib.cp_al_gb300_unbuilt_switch() is None
    monkeypatch.setenv(name, "0" if value == "1" else "mp_fixed")
    assert lp_lib.cp_al_gb300_unbuilt_switch() is None
    monkeypatch.setenv(name, value)
    assert lp_lib.cp_al_gb300_unbuilt_switch() == name.encode()
    data = lp.LPData(np.ones(2), (np.array([0, 2], np.int32), np.array([0, 1], np.int32), np.ones(2), (1, 2)),
                     np.array([0.0]), np.array([1.0]), np.zeros(2), np.ones(2))
    prob = lp._CProblem(lp_lib, data)
    try:
        assert not lp_lib.solve_lp_problem(prob.ptr, None)
        assert name in N.last_error(lp_lib)
        # every entry point that takes its options from the environment
        assert not lp_lib.cp_al_gb300_solve(prob.ptr, None, None)
        assert not lp_lib.cp_al_gb300_session_create(prob.ptr, None, None)
        assert name in N.last_error(lp_lib)
    finally:
        prob.close()


def test_pulse_and_trigger_options_from_env(lp_lib, monkeypatch):
    """The alpha pulse and the sigma trigger are built: their switches are
    read into the options (LP/CP_AL/src/solver.cu:889-892, 1214-1216,
    1497-1509 defaults) and refuse nothing."""
    names = ("CP_AL_ALPHA_DIRECT_PULSE", "CP_AL_DETERMINISTIC_PULSE_FORCE", "CP_AL_ALPHA_DIRECT_PULSE_TRACE",
             "CP_AL_ALPHA_DIRECT_PULSE_TEST_TRAJECTORY_LIMIT", "CP_AL_SIGMA_TRIGGER", "CP_AL_SIGMA_TRIGGER_MIN_ITERS",
             "CP_AL_SIGMA_TRIGGER_PRIMAL", "CP_AL_SIGMA_TRIGGER_DUAL", "CP_AL_SIGMA_TRIGGER_RATIO",
             "CP_AL_ADAPTIVE_LAMBDA", "CP_AL_LAMBDA_PROFILE", "CP_AL_DYNAMIC_EVAL", "CP_AL_ALPHA_ROLLBACK_TRIAL")
    for var in names:
        monkeypatch.delenv(var, raising=False)
    o = lp.default_options(lp_lib, from_env=True)
    assert (o.alpha_direct_pulse, o.pulse_force, o.pulse_trace, o.pulse_test_limit, o.sigma_trigger) == (0,) * 5
    assert (o.sigma_trigger_min_iters, o.sigma_trigger_primal, o.sigma_trigger_dual,
            o.sigma_trigger_ratio) == (200, 1e-2, 1e-6, 1e6)
    for var, val in zip(names[:9], ("1", "1", "1", "12000", "1", "400", "0.05", "1e-5", "1e3")):
        monkeypatch.setenv(var, val)
    o = lp.default_options(lp_lib, from_env=True)
    assert (o.alpha_direct_pulse, o.pulse_force, o.pulse_trace, o.pulse_test_limit, o.sigma_trigger) == (
        1, 1, 1, 12000, 1)
    assert (o.sigma_trigger_min_iters, o.sigma_trigger_primal, o.sigma_trigger_dual,
            o.sigma_trigger_ratio) == (400, 0.05, 1e-5, 1e3)
    assert lp_lib.cp_al_gb300_unbuilt_switch() is None


def test_curtis_reid_options_from_env(lp_lib, monkeypatch):
    """CP_AL_CR_SCALING / CP_AL_CR_ITERS / CP_AL_CR_EARLY_STOP(_THRESHOLD) are
    read with the reference's atoi / atof rules (LP/CP_AL/src/
    preconditioner.cu:174-178, 403-411)."""
    for var in ("CP_AL_CR_SCALING", "CP_AL_CR_ITERS", "CP_AL_CR_EARLY_STOP", "CP_AL_CR_EARLY_STOP_THRESHOLD"):
        monkeypatch.delenv(var, raising=False)
    o = lp.default_options(lp_lib, from_env=True)
    assert (o.cr_iterations, o.cr_early_stop, o.cr_early_stop_threshold) == (0, 0, 0.1)
    monkeypatch.setenv("CP_AL_CR_ITERS", "7")
    assert lp.default_options(lp_lib, from_env=True).cr_iterations == 0
    monkeypatch.setenv("CP_AL_CR_SCALING", "1")
    assert lp.default_options(lp_lib, from_env=True).cr_iterations == 7
    monkeypatch.setenv("CP_AL_CR_ITERS", "abc")
    assert lp.default_options(lp_lib, from_env=True).cr_iterations == 0
    monkeypatch.delenv("CP_AL_CR_ITERS")
    monkeypatch.setenv("CP_AL_CR_EARLY_STOP", "1")
    monkeypatch.setenv("CP_AL_CR_EARLY_STOP_THRESHOLD", "0.25")
    o = lp.default_options(lp_lib, from_env=True)
    assert (o.cr_iterations, o.cr_early_stop, o.cr_early_stop_threshold) == (20, 1, 0.25)
    assert lp_lib.cp_al_gb300_unbuilt_switch() is None


@pytest.mark.parametrize("profile,refused", [
    ("grid4_race", True), ("race4", True), ("mp_race", True), ("safe_race", True), ("mp_auto", True),
    ("safe_auto", True), ("fixed", False), ("", False),
])
def test_lambda_profiles_that_enable_adaptive_lambda(lp_lib, monkeypatch, profile, refused):
    """The CP_AL_LAMBDA_PROFILE values that switch the reference's adaptive
    lambda on (LP/CP_AL/src/solver.cu:3168-3180) are refused; others are
    not."""
    for var in ("CP_AL_ADAPTIVE_LAMBDA", "CP_AL_DYNAMIC_EVAL", "CP_AL_SIGMA_TRIGGER", "CP_AL_ALPHA_ROLLBACK_TRIAL",
                "CP_AL_ALPHA_DIRECT_PULSE"):
        monkeypatch.delenv(var, raising=False)
    monkeypatch.setenv("CP_AL_LAMBDA_PROFILE", profile)
    got = lp_lib.cp_al_gb300_unbuilt_switch()
    assert got == (b"CP_AL_LAMBDA_PROFILE" if refused else None)
