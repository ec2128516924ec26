"""Native core of the FA_CP Python interface over libfa_cp_gb300.so: the
functions the reference's pybind11 module exports
(QP/FA_CP/python_bindings/_core_bindings.cpp:229-601), with the same
arguments, parameter keys, result keys and errors."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .. import _native as N
from ..qp import default_parameters

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

# termination reason -> (Status, StatusCode), _core_bindings.cpp:180-226
_STATUS = {
    0: ("UNSPECIFIED", -1),
    1: ("OPTIMAL", 0),
    2: ("PRIMAL_INFEASIBLE", 1),
    3: ("DUAL_INFEASIBLE", 2),
    4: ("INFEASIBLE_OR_UNBOUNDED", 5),
    5: ("TIME_LIMIT", 3),
    6: ("ITERATION_LIMIT", 4),
    7: ("FEAS_POLISH_SUCCESS", -1),
}

_TERM = ("eps_optimal_relative", "eps_feasible_relative", "time_sec_limit", "iteration_limit",
         "eps_feas_polish_relative", "eps_infeasible")
_RESTART = ("artificial_restart_threshold", "sufficient_reduction_for_restart", "necessary_reduction_for_restart",
            "k_p", "k_i", "k_d", "i_smooth")
_INT_KEYS = ("verbose", "termination_evaluation_frequency", "iteration_limit", "l_inf_ruiz_iterations", "sv_max_iter")
_BOOL_KEYS = ("has_pock_chambolle_alpha", "bound_objective_rescaling", "feasibility_polishing", "use_al_qp")


def get_default_params() -> dict:
    """The parameter dictionary of _core_bindings.cpp:229-272."""
    p = default_parameters()
    t, r = p.termination_criteria, p.restart_params
    return {
        "verbose": p.verbose,
        "termination_evaluation_frequency": p.termination_evaluation_frequency,
        "eps_optimal_relative": t.eps_optimal_relative,
        "eps_feasible_relative": t.eps_feasible_relative,
        "time_sec_limit": t.time_sec_limit,
        "iteration_limit": t.iteration_limit,
        "l_inf_ruiz_iterations": p.l_inf_ruiz_iterations,
        "has_pock_chambolle_alpha": bool(p.has_pock_chambolle_alpha),
        "pock_chambolle_alpha": p.pock_chambolle_alpha,
        "bound_objective_rescaling": bool(p.bound_objective_rescaling),
        "artificial_restart_threshold": r.artificial_restart_threshold,
        "sufficient_reduction_for_restart": r.sufficient_reduction_for_restart,
        "necessary_reduction_for_restart": r.necessary_reduction_for_restart,
        "k_p": r.k_p,
        "reflection_coefficient": p.reflection_coefficient,
        "feasibility_polishing": bool(p.feasibility_polishing),
        "eps_feas_polish_relative": t.eps_feas_polish_relative,
        "optimality_norm": "linf" if p.optimality_norm == N.NORM_LINF else "l2",
        "sv_max_iter": p.sv_max_iter,
        "sv_tol": p.sv_tol,
    }


def _parse_params(d, p: N.FacpParameters) -> None:
    """_core_bindings.cpp:276-338; the sigma controls of fa_cp_parameters_t
    (use_al_qp, al_sigma, sigma_*) are accepted as well."""
    if d is None:
        return
    for k, v in dict(d).items():
        if k == "optimality_norm":
            if not isinstance(v, str):
                raise ValueError("optimality_norm must be a string ('l2'/'linf')")
            low = v.lower()
            if low not in ("l2", "linf"):
                raise ValueError(f"Unknown norm type: {v}. Use 'l2' or 'linf'.")
            p.optimality_norm = N.NORM_LINF if low == "linf" else N.NORM_L2
            continue
        conv = int if k in _INT_KEYS else (bool if k in _BOOL_KEYS else float)
        if k in _TERM:
            setattr(p.termination_criteria, k, conv(v))
        elif k in _RESTART:
            setattr(p.restart_params, k, float(v))
        elif k == "sigma_update_rule":
            p.sigma_update_rule = N.SIGMA_RULES[v] if isinstance(v, str) else int(v)
        elif k.startswith("sigma_") or k in ("al_sigma", "use_al_qp", "verbose", "termination_evaluation_frequency",
                                             "l_inf_ruiz_iterations", "has_pock_chambolle_alpha",
                                             "pock_chambolle_alpha", "bound_objective_rescaling",
                                             "reflection_coefficient", "feasibility_polishing", "sv_max_iter",
                                             "sv_tol"):
            setattr(p, k, conv(v))
        # other keys are ignored, as in the reference binding


def _desc(M, zero_tolerance: float, keep: list):
    """matrix_desc_t of a numpy array (dense) or a scipy csr/csc/coo matrix
    (_core_bindings.cpp:340-428)."""
    if not hasattr(M, "shape") or len(M.shape) != 2:
        raise ValueError("matrix A must be 2D")
    d = N.QpMatrixDesc()
    d.m, d.n = int(M.shape[0]), int(M.shape[1])
    d.zero_tolerance = float(zero_tolerance)
    if isinstance(M, np.ndarray):
        a = np.ascontiguousarray(M, dtype=np.float64)
        keep.append(a)
        d.fmt = N.MATRIX_DENSE
        d.data.dense.A = a.ctypes.data_as(_dp)
        return d
    fmt = getattr(M, "format", "unknown")
    i32 = lambda x: np.ascontiguousarray(x, dtype=np.int32)
    f64 = lambda x: np.ascontiguousarray(x, dtype=np.float64)
    if fmt == "csr":
        rp, ci, v = i32(M.indptr), i32(M.indices), f64(M.data)
        keep += [rp, ci, v]
        d.fmt = N.MATRIX_CSR
        d.data.csr.nnz, d.data.csr.row_ptr, d.data.csr.col_ind, d.data.csr.vals = (
            v.size, rp.ctypes.data_as(_ip), ci.ctypes.data_as(_ip), v.ctypes.data_as(_dp))
    elif fmt == "csc":
        cp, ri, v = i32(M.indptr), i32(M.indices), f64(M.data)
        keep += [cp, ri, v]
        d.fmt = N.MATRIX_CSC
        d.data.csc.nnz, d.data.csc.col_ptr, d.data.csc.row_ind, d.data.csc.vals = (
            v.size, cp.ctypes.data_as(_ip), ri.ctypes.data_as(_ip), v.ctypes.data_as(_dp))
    elif fmt == "coo":
        r, c, v = i32(M.row), i32(M.col), f64(M.data)
        keep += [r, c, v]
        d.fmt = N.MATRIX_COO
        d.data.coo.nnz, d.data.coo.row_ind, d.data.coo.col_ind, d.data.coo.vals = (
            v.size, r.ctypes.data_as(_ip), c.ctypes.data_as(_ip), v.ctypes.data_as(_dp))
    else:
        raise ValueError("Unsupported matrix A: expected numpy.ndarray or scipy.sparse (csr/csc/coo)")
    return d


def _vec(obj, name: str, n: int, keep: list):
    if obj is None:
        return None
    a = np.asarray(obj, dtype=np.float64)
    if a.ndim != 1:
        raise ValueError(f"{name} must be 1D.")
    if a.size != n:
        raise ValueError(f"{name} length mismatch: expect {n}, got {a.size}")
    a = np.ascontiguousarray(a)
    keep.append(a)
    return a.ctypes.data_as(_dp)


def solve_once(Q, R, A, objective_vector, objective_constant=None, variable_lower_bound=None,
               variable_upper_bound=None, constraint_lower_bound=None, constraint_upper_bound=None,
               zero_tolerance: float = 0.0, params=None, primal_start=None, dual_start=None) -> dict:
    """One solve; returns the info dictionary of _core_bindings.cpp:431-582."""
    lib = N.load_qp()
    keep: list = []
    dA = _desc(A, zero_tolerance, keep) if A is not None else None
    dQ = _desc(Q, zero_tolerance, keep) if Q is not None else None
    dR = _desc(R, zero_tolerance, keep) if R is not None else None
    n = m = 0
    for d in (dA, dQ, dR):
        if d is not None and d.n > 0:
            n = d.n
            break
    if dA is not None and dA.m > 0:
        m = dA.m
    c = _vec(objective_vector, "objective_vector", n, keep)
    lb = _vec(variable_lower_bound, "variable_lower_bound", n, keep)
    ub = _vec(variable_upper_bound, "variable_upper_bound", n, keep)
    cl = _vec(constraint_lower_bound, "constraint_lower_bound", m, keep)
    cu = _vec(constraint_upper_bound, "constraint_upper_bound", m, keep)
    c0 = C.c_double(float(objective_constant)) if objective_constant is not None else None
    ref = lambda d: C.byref(d) if d is not None else None
    prob = lib.create_qp_problem(c, ref(dQ), ref(dR), ref(dA), cl, cu, lb, ub, C.byref(c0) if c0 is not None else None)
    if not prob:
        raise RuntimeError("create_qp_problem failed.")
    try:
        if primal_start is not None or dual_start is not None:
            lib.set_start_values(prob, _vec(primal_start, "primal_start", n, keep),
                                 _vec(dual_start, "dual_start", m, keep))
        p = default_parameters(lib)
        _parse_params(params, p)
        o = N.FacpOptions()
        lib.fa_cp_gb300_options_from_env(C.byref(o))
        res = lib.fa_cp_gb300_solve(prob, C.byref(p), C.byref(o))
    finally:
        lib.qp_problem_free(prob)
    if not res:
        raise RuntimeError("solve_qp_problem returned NULL.")
    try:
        r = res.contents
        vec = lambda ptr, k: np.ctypeslib.as_array(ptr, shape=(k,)).copy() if k > 0 else np.zeros(0)
        status, code = _STATUS.get(r.termination_reason, ("UNKNOWN", -1))
        return {
            "X": vec(r.primal_solution, r.num_variables),
            "Pi": vec(r.dual_solution, r.num_constraints),
            "PrimalObj": r.primal_objective_value,
            "DualObj": r.dual_objective_value,
            "ObjectiveGap": r.objective_gap,
            "RelativeObjectiveGap": r.relative_objective_gap,
            "Status": status,
            "StatusCode": code,
            "Iterations": r.total_count,
            "RescalingTimeSec": r.rescaling_time_sec,
            "RuntimeSec": r.cumulative_time_sec,
            "RelativePrimalResidual": r.relative_primal_residual,
            "RelativeDualResidual": r.relative_dual_residual,
            "MaxPrimalRayInfeas": r.max_primal_ray_infeasibility,
            "MaxDualRayInfeas": r.max_dual_ray_infeasibility,
            "PrimalRayLinObj": r.primal_ray_linear_objective,
            "DualRayObj": r.dual_ray_objective,
        }
    finally:
        lib.fa_cp_result_free(res)
