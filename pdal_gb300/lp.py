"""Python front end of the CP_AL (LP) solver: numpy / scipy arrays in, the
C entry points of libcp_al_gb300.so underneath (create_lp_problem,
set_start_values, cp_al_gb300_solve, cp_al_result_free, lp_problem_free).

    from pdal_gb300 import lp
    res = lp.solve(lp.LPData(c, A_csr, con_lb, con_ub, var_lb, var_ub),
                   params={"eps": 1e-6}, options={"precision": "fp32_refine"})
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import _native as N

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


@dataclass
class LPData:
    """min c'x + c0  s.t.  con_lb <= A x <= con_ub,  var_lb <= x <= var_ub.
    A is CSR: (row_ptr, col_ind, vals, shape) or any scipy sparse matrix."""

    c: np.ndarray
    A: Any
    con_lb: np.ndarray
    con_ub: np.ndarray
    var_lb: np.ndarray
    var_ub: np.ndarray
    c0: float = 0.0
    primal_start: np.ndarray | None = None
    dual_start: np.ndarray | None = None

    def csr(self):
        A = self.A
        if isinstance(A, tuple):
            rp, ci, v, shape = A
        else:
            A = A.tocsr()
            rp, ci, v, shape = A.indptr, A.indices, A.data, A.shape
        return (
            np.ascontiguousarray(rp, dtype=np.int32),
            np.ascontiguousarray(ci, dtype=np.int32),
            np.ascontiguousarray(v, dtype=np.float64),
            (int(shape[0]), int(shape[1])),
        )


@dataclass
class LPResult:
    status: str
    status_code: int
    iterations: int
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
    setup_sec: float
    solve_sec: float
    stats: dict = field(default_factory=dict)

    @property
    def kkt(self) -> float:
        return max(self.relative_primal_residual, self.relative_dual_residual, self.relative_gap)


def _ptr(a: np.ndarray | None, ctype=_dp):
    if a is None:
        return None
    return a.ctypes.data_as(ctype)


def default_parameters(lib=None) -> N.CpalParameters:
    lib = lib or N.load_lp()
    p = N.CpalParameters()
    lib.set_default_parameters(C.byref(p))
    return p


def default_options(lib=None, from_env: bool = False) -> N.CpalOptions:
    lib = lib or N.load_lp()
    o = N.CpalOptions()
    (lib.cp_al_gb300_options_from_env if from_env else lib.cp_al_gb300_default_options)(C.byref(o))
    return o


def apply_params(p: N.CpalParameters, d: dict | None) -> N.CpalParameters:
    """Keys: any field of cp_al_parameters_t, plus 'eps' (sets both relative
    tolerances), 'iteration_limit', 'time_limit', 'eps_optimal', 'eps_feasible',
    'eps_feas_polish', 'linf' (optimality norm)."""
    for k, v in (d or {}).items():
        if k == "eps":
            p.termination_criteria.eps_optimal_relative = v
            p.termination_criteria.eps_feasible_relative = v
        elif k == "eps_optimal":
            p.termination_criteria.eps_optimal_relative = v
        elif k == "eps_feasible":
            p.termination_criteria.eps_feasible_relative = v
        elif k == "iteration_limit":
            p.termination_criteria.iteration_limit = int(v)
        elif k == "eps_feas_polish":
            p.termination_criteria.eps_feas_polish_relative = v
        elif k == "time_limit":
            p.termination_criteria.time_sec_limit = float(v)
        elif k == "linf":
            p.optimality_norm = N.NORM_LINF if v else N.NORM_L2
        elif k in ("k_p", "k_i", "k_d", "i_smooth", "artificial_restart_threshold",
                   "sufficient_reduction_for_restart", "necessary_reduction_for_restart"):
            setattr(p.restart_params, k, v)
        else:
            if not hasattr(p, k):
                raise KeyError(f"unknown parameter {k!r}")
            setattr(p, k, v)
    return p


def apply_options(o: N.CpalOptions, d: dict | None) -> N.CpalOptions:
    for k, v in (d or {}).items():
        if k == "precision":
            v = {"fp64": N.PRECISION_FP64, "fp32_refine": N.PRECISION_FP32_REFINE}.get(v, v)
        if k == "sigma" and v is not None:
            o.sigma_set = 1
        if k == "lambda_param" and v is not None:
            o.lambda_param_set = 1
        if not hasattr(o, k):
            raise KeyError(f"unknown option {k!r}")
        setattr(o, k, v)
    return o


class _CProblem:
    """An lp_problem_t built by create_lp_problem (deep copy, freed on close)."""

    def __init__(self, lib, data: LPData):
        self.lib = lib
        rp, ci, v, (m, n) = data.csr()
        desc = N.MatrixDesc()
        desc.m, desc.n, desc.fmt = m, n, N.MATRIX_CSR
        desc.data.csr.nnz = int(ci.shape[0])
        desc.data.csr.row_ptr = _ptr(rp, _ip)
        desc.data.csr.col_ind = _ptr(ci, _ip)
        desc.data.csr.vals = _ptr(v)
        arr = lambda a, k: np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
        c = arr(data.c, n)
        cl, cu, vl, vu = arr(data.con_lb, m), arr(data.con_ub, m), arr(data.var_lb, n), arr(data.var_ub, n)
        c0 = C.c_double(float(data.c0))
        self.ptr = lib.create_lp_problem(_ptr(c), C.byref(desc), _ptr(cl), _ptr(cu), _ptr(vl), _ptr(vu), C.byref(c0))
        if not self.ptr:
            raise ValueError("create_lp_problem failed")
        if data.primal_start is not None or data.dual_start is not None:
            ps = arr(data.primal_start, n)
            ds = arr(data.dual_start, m)
            lib.set_start_values(self.ptr, _ptr(ps), _ptr(ds))
        self.m, self.n, self.nnz = m, n, int(ci.shape[0])

    def close(self):
        if self.ptr:
            self.lib.lp_problem_free(self.ptr)
            self.ptr = None

    def __del__(self):
        self.close()


def _result_from_c(lib, r: N.CpalResult, m: int, n: int, with_vectors: bool = True) -> LPResult:
    def vec(p, k):
        if not with_vectors or not p:
            return np.zeros(0)
        return np.ctypeslib.as_array(p, shape=(k,)).copy() if k > 0 else np.zeros(0)

    st = N.CpalStats()
    lib.cp_al_gb300_last_stats(C.byref(st))
    stats = {f: getattr(st, f) for f, _ in N.CpalStats._fields_}
    stats["feasibility_iteration"] = r.feasibility_iteration
    for f in ("max_primal_ray_infeasibility", "max_dual_ray_infeasibility", "primal_ray_linear_objective",
              "dual_ray_objective"):
        stats[f] = getattr(r, f)
    stats["feasibility_polishing_time"] = r.feasibility_polishing_time
    return LPResult(
        status=N.TERMINATION_REASONS.get(r.termination_reason, str(r.termination_reason)),
        status_code=r.termination_reason,
        iterations=r.total_count,
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
        setup_sec=r.rescaling_time_sec,
        solve_sec=r.cumulative_time_sec,
        stats=stats,
    )


def solve(data: LPData, params: dict | N.CpalParameters | None = None,
          options: dict | N.CpalOptions | None = None) -> LPResult:
    """One solve through the C entry points (host buffers in, host buffers out)."""
    lib = N.load_lp()
    p = params if isinstance(params, N.CpalParameters) else apply_params(default_parameters(lib), params)
    o = options if isinstance(options, N.CpalOptions) else apply_options(default_options(lib), options)
    prob = _CProblem(lib, data)
    try:
        rp = lib.cp_al_gb300_solve(prob.ptr, C.byref(p), C.byref(o))
        if not rp:
            raise RuntimeError("solve failed: " + N.last_error(lib))
        try:
            return _result_from_c(lib, rp.contents, prob.m, prob.n)
        finally:
            lib.cp_al_result_free(rp)
    finally:
        prob.close()


class LPSession:
    """Problem uploaded once; solve() runs from the device-resident copy
    (equilibration, power iteration and the loop all re-run each time)."""

    def __init__(self, data: LPData, params=None, options=None):
        self.lib = N.load_lp()
        p = params if isinstance(params, N.CpalParameters) else apply_params(default_parameters(self.lib), params)
        o = options if isinstance(options, N.CpalOptions) else apply_options(default_options(self.lib), options)
        self._prob = _CProblem(self.lib, data)
        self.h = self.lib.cp_al_gb300_session_create(self._prob.ptr, C.byref(p), C.byref(o))
        if not self.h:
            raise RuntimeError("session_create failed: " + N.last_error(self.lib))
        self.m, self.n = self._prob.m, self._prob.n

    def solve(self) -> LPResult:
        r = N.CpalResult()
        if self.lib.cp_al_gb300_session_solve(self.h, C.byref(r)) != 0:
            raise RuntimeError("session solve failed: " + N.last_error(self.lib))
        return _result_from_c(self.lib, r, self.m, self.n, with_vectors=False)

    def start(self):
        """Equilibration, power iteration and the initial iterate, no iterations."""
        if self.lib.cp_al_gb300_session_start(self.h) != 0:
            raise RuntimeError("session start failed: " + N.last_error(self.lib))

    def iterate(self, iterations: int) -> LPResult:
        """Continue the started solve for `iterations` more iterations."""
        r = N.CpalResult()
        if self.lib.cp_al_gb300_session_iterate(self.h, int(iterations), C.byref(r)) != 0:
            raise RuntimeError("session iterate failed: " + N.last_error(self.lib))
        return _result_from_c(self.lib, r, self.m, self.n, with_vectors=False)

    def fetch(self):
        x = np.empty(self.n)
        y = np.empty(self.m)
        rc = np.empty(self.n)
        if self.lib.cp_al_gb300_session_fetch(self.h, _ptr(x), _ptr(y) if self.m else None, _ptr(rc)) != 0:
            raise RuntimeError("fetch failed: " + N.last_error(self.lib))
        return x, y, rc

    def scaling(self):
        """(scaled A values, row scales, column scales, cbr, ovr, lambda_est)
        after the device equilibration and power iteration."""
        vals = np.empty(max(self._prob.nnz, 1))
        r = np.empty(max(self.m, 1))
        c = np.empty(self.n)
        bo = np.empty(2)
        lam = C.c_double(0.0)
        if self.lib.cp_al_gb300_session_scaling(self.h, _ptr(vals), _ptr(r), _ptr(c), _ptr(bo), C.byref(lam)) != 0:
            raise RuntimeError("scaling failed: " + N.last_error(self.lib))
        return vals[: self._prob.nnz], r[: self.m], c, bo[0], bo[1], lam.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.cp_al_gb300_session_free(self.h)
            self.h = None
        if getattr(self, "_prob", None):
            self._prob.close()

    def __del__(self):
        self.close()


def solve_batch(items: list[LPData], params: dict | N.CpalParameters | None = None,
                options: dict | N.CpalOptions | None = None,
                sigma0: np.ndarray | None = None) -> tuple[list[LPResult], dict]:
    """All instances in one persistent launch (cp_al_gb300_batch_solve);
    returns the per-instance results (their .stats hold the final controller
    state) and the batch statistics.  sigma0: optional per-instance initial
    sigma for sigma mode."""
    lib = N.load_lp()
    p = params if isinstance(params, N.CpalParameters) else apply_params(default_parameters(lib), params)
    o = options if isinstance(options, N.CpalOptions) else apply_options(default_options(lib), options)
    probs = [_CProblem(lib, d) for d in items]
    try:
        arr = (C.POINTER(N.LpProblem) * len(probs))(*[q.ptr for q in probs])
        res = (C.POINTER(N.CpalResult) * len(probs))()
        info = (N.InstanceInfo * len(probs))()
        st = N.BatchStats()
        s0 = None if sigma0 is None else np.ascontiguousarray(sigma0, dtype=np.float64)
        if lib.cp_al_gb300_batch_solve(len(probs), arr, C.byref(p), C.byref(o), _ptr(s0), res, info,
                                       C.byref(st)) != 0:
            raise RuntimeError("batch solve failed: " + N.last_error(lib))
        out = []
        for q, r, f in zip(probs, res, info):
            try:
                lr = _result_from_c(lib, r.contents, q.m, q.n)
                lr.stats = {k: getattr(f, k) for k, _ in N.InstanceInfo._fields_}
                out.append(lr)
            finally:
                lib.cp_al_result_free(r)
        return out, {f: getattr(st, f) for f, _ in N.BatchStats._fields_}
    finally:
        for q in probs:
            q.close()


def tune_batch(items: list[LPData], params: dict | N.CpalParameters | None = None,
               options: dict | N.CpalOptions | None = None) -> dict:
    """The batch schedule autotuner alone (cp_al_gb300_batch_tune): the
    schedule a later solve_batch of the same batch shape will use, and the
    tuning time."""
    lib = N.load_lp()
    p = params if isinstance(params, N.CpalParameters) else apply_params(default_parameters(lib), params)
    o = options if isinstance(options, N.CpalOptions) else apply_options(default_options(lib), options)
    probs = [_CProblem(lib, d) for d in items]
    try:
        arr = (C.POINTER(N.LpProblem) * len(probs))(*[q.ptr for q in probs])
        st = N.BatchStats()
        if lib.cp_al_gb300_batch_tune(len(probs), arr, C.byref(p), C.byref(o), C.byref(st)) != 0:
            raise RuntimeError("batch tune failed: " + N.last_error(lib))
        return {"block_nnz": st.block_nnz, "blocks_per_sm": st.blocks_per_sm, "tune_sec": st.tune_sec}
    finally:
        for q in probs:
            q.close()
