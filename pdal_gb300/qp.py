"""Python front end of the FA_CP (convex QP) solver: numpy / scipy arrays in,
the C entry points of libfa_cp_gb300.so underneath (create_qp_problem,
set_start_values, fa_cp_gb300_solve, fa_cp_result_free, qp_problem_free).

    from pdal_gb300 import qp
    res = qp.solve(qp.QPData(c, A=A_csr, con_lb=l, con_ub=u, Q=Q_csr), params={"eps": 1e-6})

The reference-shaped interface (fa_cp.Model) is pdal_gb300.fa_cp.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import _native as N

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _csr(M, shape_hint=None):
    """(row_ptr int32, col_ind int32, vals float64, (rows, cols)) of a scipy
    sparse matrix, a dense 2-D array or an (rp, ci, v, shape) tuple."""
    if M is None:
        return None
    if isinstance(M, tuple):
        rp, ci, v, shape = M
    elif hasattr(M, "tocsr"):
        M = M.tocsr()
        M.sort_indices()
        rp, ci, v, shape = M.indptr, M.indices, M.data, M.shape
    else:
        D = np.asarray(M, dtype=np.float64)
        rows, cols = np.nonzero(D)
        rp = np.zeros(D.shape[0] + 1, dtype=np.int32)
        np.add.at(rp, rows + 1, 1)
        rp = np.cumsum(rp).astype(np.int32)
        ci, v, shape = cols, D[rows, cols], D.shape
    return (
        np.ascontiguousarray(rp, dtype=np.int32),
        np.ascontiguousarray(ci, dtype=np.int32),
        np.ascontiguousarray(v, dtype=np.float64),
        (int(shape[0]), int(shape[1])),
    )


@dataclass
class QPData:
    """min 1/2 x'(Q + R'R)x + c'x + c0  s.t.  con_lb <= A x <= con_ub,
    var_lb <= x <= var_ub.  A, Q and R are each optional (CSR tuple, scipy
    sparse or dense); missing bounds are infinite."""

    c: np.ndarray
    A: Any = None
    con_lb: np.ndarray | None = None
    con_ub: np.ndarray | None = None
    var_lb: np.ndarray | None = None
    var_ub: np.ndarray | None = None
    Q: Any = None
    R: Any = None
    c0: float = 0.0
    primal_start: np.ndarray | None = None
    dual_start: np.ndarray | None = None

    def dims(self) -> tuple[int, int]:
        for M in (self.A, self.Q, self.R):
            if M is not None:
                n = _csr(M)[3][1]
                break
        else:
            raise ValueError("QPData needs at least one of A, Q, R")
        m = _csr(self.A)[3][0] if self.A is not None else 0
        return m, n


@dataclass
class QPResult:
    status: str
    status_code: int
    iterations: int
    inner_iterations: int
    x: np.ndarray
    y: np.ndarray
    reduced_cost: np.ndarray
    primal_objective: float
    dual_objective: float
    relative_primal_residual: float
    relative_dual_residual: float
    relative_gap: float
    absolute_primal_residual: float
    absolute_dual_residual: float
    max_primal_ray_infeasibility: float
    max_dual_ray_infeasibility: float
    primal_ray_linear_objective: float
    dual_ray_objective: float
    final_al_sigma: float
    sigma_update_count: int
    setup_sec: float
    solve_sec: float
    stats: dict = field(default_factory=dict)

    @property
    def kkt(self) -> float:
        return max(self.relative_primal_residual, self.relative_dual_residual, self.relative_gap)


def _ptr(a, ctype=_dp):
    return None if a is None else a.ctypes.data_as(ctype)


def default_parameters(lib=None) -> N.FacpParameters:
    lib = lib or N.load_qp()
    p = N.FacpParameters()
    lib.set_default_parameters(C.byref(p))
    return p


def default_options(lib=None) -> N.FacpOptions:
    lib = lib or N.load_qp()
    o = N.FacpOptions()
    lib.fa_cp_gb300_default_options(C.byref(o))
    return o


_TERM_KEYS = ("eps_optimal_relative", "eps_feasible_relative", "eps_feas_polish_relative", "eps_infeasible",
              "time_sec_limit", "iteration_limit")
_RESTART_KEYS = ("k_p", "k_i", "k_d", "i_smooth", "artificial_restart_threshold",
                 "sufficient_reduction_for_restart", "necessary_reduction_for_restart")


def apply_params(p: N.FacpParameters, d: dict | None) -> N.FacpParameters:
    """Keys: any field of fa_cp_parameters_t (nested termination and restart
    fields by their own names), plus 'eps' (both relative tolerances),
    'time_limit', 'linf' (bool) or optimality_norm 'l2'/'linf', and
    sigma_update_rule by name."""
    for k, v in (d or {}).items():
        if k == "eps":
            p.termination_criteria.eps_optimal_relative = v
            p.termination_criteria.eps_feasible_relative = v
        elif k == "time_limit":
            p.termination_criteria.time_sec_limit = float(v)
        elif k == "eps_feas_polish":
            p.termination_criteria.eps_feas_polish_relative = float(v)
        elif k == "linf":
            p.optimality_norm = N.NORM_LINF if v else N.NORM_L2
        elif k == "optimality_norm":
            if isinstance(v, str):
                low = v.lower()
                if low not in ("l2", "linf"):
                    raise ValueError(f"Unknown norm type: {v}. Use 'l2' or 'linf'.")
                v = N.NORM_LINF if low == "linf" else N.NORM_L2
            p.optimality_norm = int(v)
        elif k == "sigma_update_rule" and isinstance(v, str):
            p.sigma_update_rule = N.SIGMA_RULES[v]
        elif k in _TERM_KEYS:
            setattr(p.termination_criteria, k, int(v) if k == "iteration_limit" else float(v))
        elif k in _RESTART_KEYS:
            setattr(p.restart_params, k, float(v))
        else:
            if not hasattr(p, k):
                raise KeyError(f"unknown parameter {k!r}")
            setattr(p, k, v)
    return p


def apply_options(o: N.FacpOptions, d: dict | None) -> N.FacpOptions:
    """Keys: any field of fa_cp_gb300_options_t; 'precision' also takes
    "fp64" / "fp32_refine"."""
    for k, v in (d or {}).items():
        if k == "precision":
            v = {"fp64": 0, "fp32_refine": 1}.get(v, v)
        if not hasattr(o, k):
            raise KeyError(f"unknown option {k!r}")
        setattr(o, k, v)
    return o


def _desc(M, zero_tolerance: float = 0.0):
    """QpMatrixDesc in CSR form over arrays kept alive by the returned tuple."""
    rp, ci, v, (r, c) = _csr(M)
    d = N.QpMatrixDesc()
    d.m, d.n, d.fmt, d.zero_tolerance = r, c, N.MATRIX_CSR, zero_tolerance
    d.data.csr.nnz = int(ci.shape[0])
    d.data.csr.row_ptr = _ptr(rp, _ip)
    d.data.csr.col_ind = _ptr(ci, _ip)
    d.data.csr.vals = _ptr(v)
    return d, (rp, ci, v)


class _CProblem:
    """A qp_problem_t built by create_qp_problem (deep copy, freed on close)."""

    def __init__(self, lib, data: QPData):
        self.lib = lib
        m, n = data.dims()
        keep = []
        descs = []
        for M in (data.Q, data.R, data.A):
            if M is None:
                descs.append(None)
            else:
                d, k = _desc(M)
                keep.append(k)
                descs.append(d)
        arr = lambda a: np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
        c = arr(data.c)
        cl, cu, vl, vu = arr(data.con_lb), arr(data.con_ub), arr(data.var_lb), arr(data.var_ub)
        c0 = C.c_double(float(data.c0))
        ref = lambda d: C.byref(d) if d is not None else None
        self.ptr = lib.create_qp_problem(_ptr(c), ref(descs[0]), ref(descs[1]), ref(descs[2]), _ptr(cl), _ptr(cu),
                                         _ptr(vl), _ptr(vu), C.byref(c0))
        if not self.ptr:
            raise ValueError("create_qp_problem failed: " + N.last_error(lib))
        if data.primal_start is not None or data.dual_start is not None:
            lib.set_start_values(self.ptr, _ptr(arr(data.primal_start)), _ptr(arr(data.dual_start)))
        self.m, self.n = m, n

    def close(self):
        if self.ptr:
            self.lib.qp_problem_free(self.ptr)
            self.ptr = None

    def __del__(self):
        self.close()


def result_from_c(r: N.FacpResult, m: int, n: int, stats: dict | None = None) -> QPResult:
    vec = lambda p, k: np.ctypeslib.as_array(p, shape=(k,)).copy() if (p and k > 0) else np.zeros(0)
    return QPResult(
        status=N.TERMINATION_REASONS.get(r.termination_reason, str(r.termination_reason)),
        status_code=r.termination_reason,
        iterations=r.total_count,
        inner_iterations=r.total_inner_count,
        x=vec(r.primal_solution, n),
        y=vec(r.dual_solution, m),
        reduced_cost=vec(r.reduced_cost, n),
        primal_objective=r.primal_objective_value,
        dual_objective=r.dual_objective_value,
        relative_primal_residual=r.relative_primal_residual,
        relative_dual_residual=r.relative_dual_residual,
        relative_gap=r.relative_objective_gap,
        absolute_primal_residual=r.absolute_primal_residual,
        absolute_dual_residual=r.absolute_dual_residual,
        max_primal_ray_infeasibility=r.max_primal_ray_infeasibility,
        max_dual_ray_infeasibility=r.max_dual_ray_infeasibility,
        primal_ray_linear_objective=r.primal_ray_linear_objective,
        dual_ray_objective=r.dual_ray_objective,
        final_al_sigma=r.final_al_sigma,
        sigma_update_count=r.sigma_update_count,
        setup_sec=r.rescaling_time_sec,
        solve_sec=r.cumulative_time_sec,
        stats={"feasibility_iteration": r.feasibility_iteration,
               "feasibility_polishing_time": r.feasibility_polishing_time, **(stats or {})},
    )


def last_stats(lib=None) -> dict:
    lib = lib or N.load_qp()
    st = N.FacpStats()
    lib.fa_cp_gb300_last_stats(C.byref(st))
    return {f: getattr(st, f) for f, _ in N.FacpStats._fields_}


def solve(data: QPData, params: dict | N.FacpParameters | None = None,
          options: dict | N.FacpOptions | None = None) -> QPResult:
    """One solve through the C entry points (host buffers in and out)."""
    lib = N.load_qp()
    p = params if isinstance(params, N.FacpParameters) else apply_params(default_parameters(lib), params)
    o = options if isinstance(options, N.FacpOptions) else apply_options(default_options(lib), options)
    prob = _CProblem(lib, data)
    try:
        rp = lib.fa_cp_gb300_solve(prob.ptr, C.byref(p), C.byref(o))
        if not rp:
            raise RuntimeError("solve failed: " + N.last_error(lib))
        try:
            return result_from_c(rp.contents, prob.m, prob.n, last_stats(lib))
        finally:
            lib.fa_cp_result_free(rp)
    finally:
        prob.close()


def scaling(data: QPData, params: dict | N.FacpParameters | None = None,
            options: dict | N.FacpOptions | None = None):
    """The device equilibration alone (fa_cp_gb300_scaling): column scales,
    row scales, cbr, ovr."""
    lib = N.load_qp()
    p = params if isinstance(params, N.FacpParameters) else apply_params(default_parameters(lib), params)
    o = options if isinstance(options, N.FacpOptions) else apply_options(default_options(lib), options)
    prob = _CProblem(lib, data)
    try:
        d, r, f = np.zeros(max(prob.n, 1)), np.zeros(max(prob.m, 1)), np.zeros(2)
        if lib.fa_cp_gb300_scaling(prob.ptr, C.byref(p), C.byref(o), _ptr(d), _ptr(r), _ptr(f)) != 0:
            raise RuntimeError("scaling failed: " + N.last_error(lib))
        return d[:prob.n], r[:prob.m], float(f[0]), float(f[1])
    finally:
        prob.close()
