"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates the reference solver on the CPU in FP64; tests compare the
CUDA library against it.  Nothing in pdal_gb300/ imports this module.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from pdal_gb300 import _native as N  # struct layouts of include/*.h only
from pdal_gb300.lp import LPData, LPResult, apply_options, apply_params

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        L.oracle_cpal_solve.restype = C.POINTER(N.CpalResult)
        L.oracle_cpal_solve.argtypes = [C.POINTER(N.LpProblem), C.POINTER(N.CpalParameters),
                                        C.POINTER(N.CpalOptions), _ip]
        L.oracle_cpal_result_free.argtypes = [C.POINTER(N.CpalResult)]
        L.oracle_cpal_default_options.argtypes = [C.POINTER(N.CpalOptions)]
        L.oracle_cpal_default_parameters.argtypes = [C.POINTER(N.CpalParameters)]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_max_threads.restype = C.c_int
        L.oracle_cpal_rescale.argtypes = [C.POINTER(N.LpProblem), C.POINTER(N.CpalParameters),
                                          C.POINTER(N.CpalOptions), _dp, _dp, _dp, _dp]
        L.oracle_cpal_session_create.restype = C.c_void_p
        L.oracle_cpal_session_create.argtypes = [C.POINTER(N.LpProblem), C.POINTER(N.CpalParameters),
                                                 C.POINTER(N.CpalOptions)]
        L.oracle_cpal_session_iterate.restype = C.c_int
        L.oracle_cpal_session_iterate.argtypes = [C.c_void_p, C.c_int]
        L.oracle_cpal_session_free.argtypes = [C.c_void_p]
        L.oracle_power_iteration.restype = C.c_double
        L.oracle_power_iteration.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, C.c_int, C.c_double, _ip]
        _lib = L
    return _lib


def default_parameters() -> N.CpalParameters:
    p = N.CpalParameters()
    lib().oracle_cpal_default_parameters(C.byref(p))
    return p


def default_options() -> N.CpalOptions:
    o = N.CpalOptions()
    lib().oracle_cpal_default_options(C.byref(o))
    return o


class _Problem:
    """lp_problem_t pointing at numpy arrays kept alive by this object."""

    def __init__(self, data: LPData):
        rp, ci, v, (m, n) = data.csr()
        f = lambda a, k, fill: (np.ascontiguousarray(a, dtype=np.float64) if a is not None else np.full(k, fill))
        self.keep = [rp, ci, v, f(data.c, n, 0.0), f(data.var_lb, n, -np.inf), f(data.var_ub, n, np.inf),
                     f(data.con_lb, m, -np.inf), f(data.con_ub, m, np.inf)]
        p = N.LpProblem()
        p.num_variables, p.num_constraints = n, m
        p.constraint_matrix_row_pointers = rp.ctypes.data_as(_ip)
        p.constraint_matrix_col_indices = ci.ctypes.data_as(_ip)
        p.constraint_matrix_values = v.ctypes.data_as(_dp)
        p.constraint_matrix_num_nonzeros = int(ci.shape[0])
        p.objective_vector = self.keep[3].ctypes.data_as(_dp)
        p.variable_lower_bound = self.keep[4].ctypes.data_as(_dp)
        p.variable_upper_bound = self.keep[5].ctypes.data_as(_dp)
        p.constraint_lower_bound = self.keep[6].ctypes.data_as(_dp)
        p.constraint_upper_bound = self.keep[7].ctypes.data_as(_dp)
        p.objective_constant = float(data.c0)
        if data.primal_start is not None:
            xs = np.ascontiguousarray(data.primal_start, dtype=np.float64)
            self.keep.append(xs)
            p.primal_start = xs.ctypes.data_as(_dp)
        if data.dual_start is not None:
            ys = np.ascontiguousarray(data.dual_start, dtype=np.float64)
            self.keep.append(ys)
            p.dual_start = ys.ctypes.data_as(_dp)
        self.p, self.m, self.n = p, m, n


def _polish_status(L):
    """Statuses of the last oracle solve's primal and dual polishing phases
    (names, or None for a phase that did not run)."""
    a, b = C.c_int(-1), C.c_int(-1)
    L.oracle_cpal_polish_status(C.byref(a), C.byref(b))
    return tuple(N.TERMINATION_REASONS.get(v.value) if v.value >= 0 else None for v in (a, b))


def _restart_targets(L):
    """Restarts of the last oracle solve by target: (current point,
    reflected Halpern iterate, plain Halpern point)."""
    counts = (C.c_int * 3)()
    L.oracle_cpal_restart_targets(counts)
    return tuple(int(v) for v in counts)


def _controllers(L):
    """The benchmark controllers of the last oracle solve: the iteration at
    which the alpha pulse's positive block started (-1: never), its gate (0
    not evaluated, 1 passed, 2 rejected), the iteration at which the sigma
    trigger fired (0: never), the iteration at which the dynamic evaluation
    frequency switched to short blocks (0: never)."""
    out = (C.c_int * 4)()
    L.oracle_cpal_controllers(out)
    return {"pulse_start_iteration": int(out[0]), "pulse_gate": int(out[1]),
            "sigma_trigger_iteration": int(out[2]), "dynamic_eval_iteration": int(out[3])}


def solve_lp(data: LPData, params: dict | None = None, options: dict | None = None, threads: int = 1) -> LPResult:
    L = lib()
    p = apply_params(default_parameters(), params)
    o = apply_options(default_options(), options)
    prob = _Problem(data)
    L.oracle_set_threads(int(threads))
    piters = C.c_int(0)
    rp = L.oracle_cpal_solve(C.byref(prob.p), C.byref(p), C.byref(o), C.byref(piters))
    if not rp:
        raise RuntimeError("oracle solve failed (invalid parameters)")
    try:
        r = rp.contents
        vec = lambda ptr, k: np.ctypeslib.as_array(ptr, shape=(k,)).copy() if k > 0 else np.zeros(0)
        return LPResult(
            status=N.TERMINATION_REASONS[r.termination_reason],
            status_code=r.termination_reason,
            iterations=r.total_count,
            x=vec(r.primal_solution, prob.n),
            y=vec(r.dual_solution, prob.m),
            reduced_cost=vec(r.reduced_cost, prob.n),
            primal_objective=r.primal_objective_value,
            dual_objective=r.dual_objective_value,
            relative_primal_residual=r.relative_primal_residual,
            relative_dual_residual=r.relative_dual_residual,
            relative_gap=r.relative_objective_gap,
            absolute_primal_residual=r.absolute_primal_residual,
            absolute_dual_residual=r.absolute_dual_residual,
            setup_sec=r.rescaling_time_sec,
            solve_sec=r.cumulative_time_sec,
            stats={"max_primal_ray_infeasibility": r.max_primal_ray_infeasibility,
                   "max_dual_ray_infeasibility": r.max_dual_ray_infeasibility,
                   "primal_ray_linear_objective": r.primal_ray_linear_objective,
                   "dual_ray_objective": r.dual_ray_objective,
                   "power_iterations": piters.value, "feasibility_iteration": r.feasibility_iteration,
                   "feasibility_polishing_time": r.feasibility_polishing_time, "polish_status": _polish_status(L),
                   "restart_targets": _restart_targets(L), **_controllers(L)},
        )
    finally:
        L.oracle_cpal_result_free(rp)


def rescale(data: LPData, params: dict | None = None, options: dict | None = None, with_passes: bool = False):
    """(row_scale, col_scale, cbr, ovr, scaled A values) of the reference's
    rescale_problem, from the oracle; with_passes adds the number of
    Curtis-Reid passes run."""
    L = lib()
    p = apply_params(default_parameters(), params)
    o = apply_options(default_options(), options)
    prob = _Problem(data)
    r = np.empty(prob.m)
    d = np.empty(prob.n)
    co = np.empty(2)
    sv = np.empty(int(prob.p.constraint_matrix_num_nonzeros))
    passes = L.oracle_cpal_rescale(C.byref(prob.p), C.byref(p), C.byref(o), r.ctypes.data_as(_dp),
                                   d.ctypes.data_as(_dp), co.ctypes.data_as(_dp), sv.ctypes.data_as(_dp))
    out = (r, d, co[0], co[1], sv)
    return out + (passes,) if with_passes else out


def power_iteration(data: LPData, max_iter: int = 5000, tol: float = 1e-4):
    rp, ci, v, (m, n) = data.csr()
    it = C.c_int(0)
    s = lib().oracle_power_iteration(m, n, rp.ctypes.data_as(_ip), ci.ctypes.data_as(_ip), v.ctypes.data_as(_dp),
                                     max_iter, tol, C.byref(it))
    return s, it.value


class Session:
    """Set up once (equilibration, power iteration), then iterate in blocks;
    used to time the CPU iteration on a bounded sample."""

    def __init__(self, data: LPData, params: dict | None = None, options: dict | None = None, threads: int = 1):
        L = lib()
        self.p = apply_params(default_parameters(), params)
        self.o = apply_options(default_options(), options)
        self.prob = _Problem(data)
        L.oracle_set_threads(int(threads))
        self.h = L.oracle_cpal_session_create(C.byref(self.prob.p), C.byref(self.p), C.byref(self.o))
        if not self.h:
            raise RuntimeError("oracle session failed")

    def iterate(self, iterations: int) -> int:
        return lib().oracle_cpal_session_iterate(self.h, int(iterations))

    def set_threads(self, threads: int):
        """Host threads of the following iterations."""
        lib().oracle_set_threads(int(threads))

    def close(self):
        if self.h:
            lib().oracle_cpal_session_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


def max_threads() -> int:
    return lib().oracle_max_threads()


# ------------------------------------------------------------------ FA_CP (QP)

from pdal_gb300.qp import QPData, QPResult, _csr  # noqa: E402
from pdal_gb300.qp import apply_params as _qp_apply_params  # noqa: E402
from pdal_gb300.qp import result_from_c as _qp_result  # noqa: E402


def _qp_lib():
    L = lib()
    if not getattr(L, "_facp_ready", False):
        L.oracle_facp_solve.restype = C.POINTER(N.FacpResult)
        L.oracle_facp_solve.argtypes = [C.POINTER(N.QpProblem), C.POINTER(N.FacpParameters)]
        L.oracle_facp_result_free.argtypes = [C.POINTER(N.FacpResult)]
        L.oracle_facp_default_parameters.argtypes = [C.POINTER(N.FacpParameters)]
        L.oracle_facp_set_trace.argtypes = [C.c_int]
        L.oracle_facp_polish_status.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L._facp_ready = True
    return L


def qp_default_parameters() -> N.FacpParameters:
    p = N.FacpParameters()
    _qp_lib().oracle_facp_default_parameters(C.byref(p))
    return p


class _QpProblem:
    """qp_problem_t over numpy arrays kept alive by this object (the layout
    create_qp_problem produces: every matrix present, possibly empty)."""

    def __init__(self, data: QPData):
        m, n = data.dims()
        self.keep = []

        def comp(M, rows):
            if M is None:
                rp = np.zeros(rows + 1, dtype=np.int32)
                ci = np.zeros(1, dtype=np.int32)
                v = np.zeros(1)
                nnz = 0
            else:
                rp, ci, v, _ = _csr(M)
                nnz = int(ci.shape[0])
                if nnz == 0:
                    ci, v = np.zeros(1, dtype=np.int32), np.zeros(1)
            c = N.CsrComponent(rp.ctypes.data_as(_ip), ci.ctypes.data_as(_ip), v.ctypes.data_as(_dp))
            self.keep += [rp, ci, v, c]
            return c, nnz

        nr = _csr(data.R)[3][0] if data.R is not None else 0
        cA, nA = comp(data.A, m)
        cQ, nQ = comp(data.Q, n)
        cR, nR = comp(data.R, nr)
        f = lambda a, k, fill: (np.ascontiguousarray(a, dtype=np.float64) if a is not None else np.full(k, fill))
        vecs = [f(data.c, n, 0.0), f(data.var_lb, n, -np.inf), f(data.var_ub, n, np.inf),
                f(data.con_lb, m, -np.inf), f(data.con_ub, m, np.inf)]
        self.keep += vecs
        p = N.QpProblem()
        p.num_variables, p.num_constraints, p.num_rank_lowrank_obj = n, m, nr
        p.objective_vector = vecs[0].ctypes.data_as(_dp)
        p.variable_lower_bound = vecs[1].ctypes.data_as(_dp)
        p.variable_upper_bound = vecs[2].ctypes.data_as(_dp)
        p.constraint_lower_bound = vecs[3].ctypes.data_as(_dp)
        p.constraint_upper_bound = vecs[4].ctypes.data_as(_dp)
        p.objective_constant = float(data.c0)
        p.constraint_matrix = C.pointer(cA)
        p.constraint_matrix_num_nonzeros = nA
        p.objective_sparse_matrix = C.pointer(cQ)
        p.objective_sparse_matrix_num_nonzeros = nQ
        p.objective_lowrank_matrix = C.pointer(cR)
        p.objective_lowrank_matrix_num_nonzeros = nR
        for name, a in (("primal_start", data.primal_start), ("dual_start", data.dual_start)):
            if a is not None:
                s = np.ascontiguousarray(a, dtype=np.float64)
                self.keep.append(s)
                setattr(p, name, s.ctypes.data_as(_dp))
        self.p, self.m, self.n = p, m, n


def qp_scaling(data: QPData, params: dict | None = None):
    """The oracle's equilibration alone: (dcum, rcum, cbr, ovr)."""
    L = _qp_lib()
    if not getattr(L, "_facp_scaling_ready", False):
        L.oracle_facp_scaling.restype = C.c_int
        L.oracle_facp_scaling.argtypes = [C.POINTER(N.QpProblem), C.POINTER(N.FacpParameters), _dp, _dp, _dp]
        L._facp_scaling_ready = True
    p = _qp_apply_params(qp_default_parameters(), params)
    prob = _QpProblem(data)
    d, r, f = np.zeros(max(prob.n, 1)), np.zeros(max(prob.m, 1)), np.zeros(2)
    if L.oracle_facp_scaling(C.byref(prob.p), C.byref(p), d.ctypes.data_as(_dp), r.ctypes.data_as(_dp),
                             f.ctypes.data_as(_dp)) != 0:
        raise RuntimeError("oracle QP scaling failed")
    return d[:prob.n], r[:prob.m], float(f[0]), float(f[1])


def solve_qp(data: QPData, params: dict | None = None, trace: bool = False) -> QPResult:
    """The oracle's FA_CP solve (serial FP64)."""
    L = _qp_lib()
    p = _qp_apply_params(qp_default_parameters(), params)
    prob = _QpProblem(data)
    L.oracle_facp_set_trace(1 if trace else 0)
    rp = L.oracle_facp_solve(C.byref(prob.p), C.byref(p))
    if not rp:
        raise RuntimeError("oracle QP solve failed (invalid parameters)")
    try:
        ps, ds = C.c_int(-1), C.c_int(-1)
        L.oracle_facp_polish_status(C.byref(ps), C.byref(ds))
        return _qp_result(rp.contents, prob.m, prob.n, {"polish_status": (ps.value, ds.value)})
    finally:
        L.oracle_facp_result_free(rp)
