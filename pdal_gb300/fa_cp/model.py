"""The FA_CP modelling class (QP/FA_CP/python/fa_cp/model.py:88-645): the same
constructor, setters, parameter handling, optimize() and solution
properties, solved by libfa_cp_gb300.so through _core.solve_once."""
from __future__ import annotations

import warnings
from typing import Any, Optional, Union

import numpy as np
import scipy.sparse as sp

from . import FA_CP
from ._core import get_default_params, solve_once

ArrayLike = Union[np.ndarray, list, tuple]


def _dense(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _sparse_csr(M) -> sp.csr_matrix:
    csr = M.tocsr().astype(np.float64, copy=False)
    csr.indptr = csr.indptr.astype(np.int32, copy=False)
    csr.indices = csr.indices.astype(np.int32, copy=False)
    csr.sort_indices()
    return csr


def _is_matrix(M) -> bool:
    return isinstance(M, np.ndarray) or sp.issparse(M)


class _ParamsView:
    """Attribute / item access to the model's parameters (aliases allowed)."""

    def __init__(self, model: "Model"):
        object.__setattr__(self, "_m", model)

    def __getattr__(self, name: str):
        key = FA_CP._PARAM_ALIAS.get(name, name)
        if key in self._m._params:
            return self._m._params[key]
        raise AttributeError(f"Unknown parameter '{name}'")

    def __setattr__(self, name: str, value):
        self._m.setParam(name, value)

    def __getitem__(self, name: str):
        return getattr(self, name)

    def __setitem__(self, name: str, value):
        self._m.setParam(name, value)

    def keys(self):
        return self._m._params.keys()


class Model:
    """min 1/2 x'(Q + R'R)x + c'x + c0  s.t.  l <= A x <= u,  lb <= x <= ub."""

    def __init__(self, objective_vector: ArrayLike, constraint_matrix=None, constraint_lower_bound=None,
                 constraint_upper_bound=None, objective_matrix=None, objective_matrix_low_rank=None,
                 variable_lower_bound=None, variable_upper_bound=None, objective_constant: float = 0.0):
        self.num_vars = 0
        self.num_constrs = 0
        for name, M in (("constraint_matrix", constraint_matrix), ("objective_matrix", objective_matrix),
                        ("objective_matrix_low_rank", objective_matrix_low_rank)):
            if M is None:
                continue
            if not hasattr(M, "shape") or len(M.shape) != 2:
                raise ValueError(f"{name} must be a 2D numpy.ndarray or scipy.sparse matrix.")
            if name == "constraint_matrix":
                self.num_constrs, self.num_vars = int(M.shape[0]), int(M.shape[1])
            elif self.num_vars == 0:
                self.num_vars = int(M.shape[1])
            elif M.shape[1] != self.num_vars:
                raise ValueError(f"{name} dimensions mismatch variables ({self.num_vars})")
        if self.num_vars == 0 and constraint_matrix is None and objective_matrix is None \
                and objective_matrix_low_rank is None:
            return
        self.ModelSense = FA_CP.MINIMIZE
        self._params: dict[str, Any] = dict(get_default_params())
        self.Params = _ParamsView(self)
        self.setObjectiveVector(objective_vector)
        self.setObjectiveConstant(objective_constant)
        self.setObjectiveMatrix(objective_matrix)
        self.setObjectiveMatrixLowRank(objective_matrix_low_rank)
        self.setConstraintMatrix(constraint_matrix)
        self.setConstraintLowerBound(constraint_lower_bound)
        self.setConstraintUpperBound(constraint_upper_bound)
        self.setVariableLowerBound(variable_lower_bound)
        self.setVariableUpperBound(variable_upper_bound)
        self._primal_start: Optional[np.ndarray] = None
        self._dual_start: Optional[np.ndarray] = None
        self._clear_solution_cache()

    # ------------------------------------------------------------ setters
    def setObjectiveVector(self, c: ArrayLike) -> None:
        self.c = _dense(c)
        if self.c.ndim != 1:
            raise ValueError(f"setObjectiveVector: c must be 1D, got shape {self.c.shape}")
        if self.c.size != self.num_vars:
            raise ValueError(f"setObjectiveVector: length {self.c.size} != self.num_vars ({self.num_vars})")
        self._clear_solution_cache()

    def setObjectiveConstant(self, c0: float) -> None:
        self.c0 = float(c0)
        self._clear_solution_cache()

    def _matrix(self, M, what: str):
        if not _is_matrix(M):
            raise TypeError(f"{what} must be a numpy.ndarray or scipy.sparse matrix")
        if len(M.shape) != 2:
            raise ValueError(f"{what} must be 2D, got shape {M.shape}")
        if M.shape[1] != self.num_vars:
            raise ValueError(f"{what} shape {M.shape} does not match number of variables ({self.num_vars})")
        return _sparse_csr(M) if sp.issparse(M) else _dense(M)

    def setObjectiveMatrix(self, Q_like) -> None:
        self.Q = None if Q_like is None else self._matrix(Q_like, "setObjectiveMatrix: Q")
        self._clear_solution_cache()

    def setObjectiveMatrixLowRank(self, R_like) -> None:
        self.R = None if R_like is None else self._matrix(R_like, "setObjectiveMatrixLowRank: R")
        self._clear_solution_cache()

    def setConstraintMatrix(self, A_like) -> None:
        if A_like is None:
            self.A = None
            self.num_constrs = 0
            self.constr_lb = None
            self.constr_ub = None
            self._clear_solution_cache()
            return
        self.A = self._matrix(A_like, "setConstraintMatrix: A")
        self.num_constrs = int(self.A.shape[0])
        for name in ("constr_lb", "constr_ub"):
            v = getattr(self, name, None)
            if v is not None and np.asarray(v).size != self.num_constrs:
                raise ValueError(f"setConstraintMatrix: {name} length {np.asarray(v).size} != rows "
                                 f"{self.num_constrs}.")
        self._clear_solution_cache()

    def _bound(self, v, size: int, what: str):
        if v is None:
            return None
        v = _dense(v).ravel()
        if v.size != size:
            raise ValueError(f"{what}: length {v.size} != {size}")
        return v

    def setConstraintLowerBound(self, constr_lb) -> None:
        self.constr_lb = self._bound(constr_lb, self.num_constrs, "setConstraintLowerBound")
        self._clear_solution_cache()

    def setConstraintUpperBound(self, constr_ub) -> None:
        self.constr_ub = self._bound(constr_ub, self.num_constrs, "setConstraintUpperBound")
        self._clear_solution_cache()

    def setVariableLowerBound(self, lb) -> None:
        self.lb = self._bound(lb, self.num_vars, "setVariableLowerBound")
        self._clear_solution_cache()

    def setVariableUpperBound(self, ub) -> None:
        self.ub = self._bound(ub, self.num_vars, "setVariableUpperBound")
        self._clear_solution_cache()

    def setWarmStart(self, primal=None, dual=None) -> None:
        self._primal_start = self._warm(primal, self.num_vars, "primal")
        self._dual_start = self._warm(dual, self.num_constrs, "dual")

    @staticmethod
    def _warm(v, size, what):
        if v is None:
            return None
        v = _dense(v).ravel()
        if v.size != size:
            warnings.warn(f"Warm start {what} size mismatch (expected {size}, got {v.size}).", RuntimeWarning)
            return None
        return v

    def clearWarmStart(self) -> None:
        self.setWarmStart(primal=None, dual=None)

    # ------------------------------------------------------------ parameters
    def setParam(self, name: str, value: Any) -> None:
        self._params[FA_CP._PARAM_ALIAS.get(name, name)] = value

    def getParam(self, name: str) -> Any:
        return self._params.get(FA_CP._PARAM_ALIAS.get(name, name))

    def setParams(self, /, **kwargs) -> None:
        for k, v in kwargs.items():
            self.setParam(k, v)

    # ------------------------------------------------------------ solve
    def optimize(self):
        self._clear_solution_cache()
        if self.ModelSense not in (FA_CP.MINIMIZE, FA_CP.MAXIMIZE):
            raise ValueError("model_sense must be FA_CP.MINIMIZE or FA_CP.MAXIMIZE")
        sign = 1 if self.ModelSense == FA_CP.MINIMIZE else -1
        info = solve_once(self.Q, self.R, self.A, sign * self.c, sign * self.c0, self.lb, self.ub, self.constr_lb,
                          self.constr_ub, zero_tolerance=0.0, params=self._params, primal_start=self._primal_start,
                          dual_start=self._dual_start)
        self._x = np.asarray(info["X"])
        self._y = np.asarray(info["Pi"])
        self._objval = sign * info["PrimalObj"]
        self._dualobj = sign * info["DualObj"]
        self._gap = info["ObjectiveGap"]
        self._rel_gap = info["RelativeObjectiveGap"]
        self._status = str(info["Status"])
        self._status_code = int(info["StatusCode"])
        self._iter = int(info["Iterations"])
        self._runtime = info["RuntimeSec"]
        self._rescale_time = info["RescalingTimeSec"]
        self._rel_p_res = info["RelativePrimalResidual"]
        self._rel_d_res = info["RelativeDualResidual"]
        self._max_p_ray = info["MaxPrimalRayInfeas"]
        self._max_d_ray = info["MaxDualRayInfeas"]
        self._p_ray_lin_obj = sign * info["PrimalRayLinObj"]
        self._d_ray_obj = sign * info["DualRayObj"]

    def _clear_solution_cache(self) -> None:
        self._x = self._y = None
        self._objval = self._dualobj = None
        self._gap = self._rel_gap = None
        self._status = None
        self._status_code = None
        self._iter = None
        self._runtime = self._rescale_time = None
        self._rel_p_res = self._rel_d_res = None
        self._max_p_ray = self._max_d_ray = None
        self._p_ray_lin_obj = self._d_ray_obj = None

    # ------------------------------------------------------------ results
    X = property(lambda self: self._x)
    Pi = property(lambda self: self._y)
    ObjVal = property(lambda self: self._objval)
    DualObj = property(lambda self: self._dualobj)
    Gap = property(lambda self: self._gap)
    RelGap = property(lambda self: self._rel_gap)
    Status = property(lambda self: self._status)
    StatusCode = property(lambda self: self._status_code)
    IterCount = property(lambda self: self._iter)
    Runtime = property(lambda self: self._runtime)
    RescalingTime = property(lambda self: self._rescale_time)
    RelPrimalResidual = property(lambda self: self._rel_p_res)
    RelDualResidual = property(lambda self: self._rel_d_res)
    MaxPrimalRayInfeas = property(lambda self: self._max_p_ray)
    MaxDualRayInfeas = property(lambda self: self._max_d_ray)
    PrimalRayLinObj = property(lambda self: self._p_ray_lin_obj)
    DualRayObj = property(lambda self: self._d_ray_obj)
    PrimalInfeas = property(lambda self: self._rel_p_res)
    DualInfeas = property(lambda self: self._rel_d_res)
