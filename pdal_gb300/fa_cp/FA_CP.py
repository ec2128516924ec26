"""Constants and parameter aliases of the FA_CP Python interface
(QP/FA_CP/python/fa_cp/FA_CP.py)."""

MINIMIZE = 1
MAXIMIZE = -1

OPTIMAL = 0
PRIMAL_INFEASIBLE = 1
DUAL_INFEASIBLE = 2
TIME_LIMIT = 3
ITERATION_LIMIT = 4
UNSPECIFIED = -1

# user-facing name -> parameter key of get_default_params()
_PARAM_ALIAS = {
    "TimeLimit": "time_sec_limit",
    "IterationLimit": "iteration_limit",
    "LogLevel": "verbose",
    "Verbosity": "verbose",
    "OutputFlag": "verbose",
    "LogToConsole": "verbose",
    "TermCheckFreq": "termination_evaluation_frequency",
    "OptimalityTol": "eps_optimal_relative",
    "FeasibilityTol": "eps_feasible_relative",
    "RuizIters": "l_inf_ruiz_iterations",
    "UsePCAlpha": "has_pock_chambolle_alpha",
    "PCAlpha": "pock_chambolle_alpha",
    "BoundObjRescaling": "bound_objective_rescaling",
    "RestartArtificialThresh": "artificial_restart_threshold",
    "RestartSufficientReduction": "sufficient_reduction_for_restart",
    "RestartNecessaryReduction": "necessary_reduction_for_restart",
    "RestartKp": "k_p",
    "ReflectionCoeff": "reflection_coefficient",
    "FeasibilityPolishing": "feasibility_polishing",
    "FeasibilityPolishingTol": "eps_feas_polish_relative",
    "OptimalityNorm": "optimality_norm",
    "SVMaxIter": "sv_max_iter",
    "SVTol": "sv_tol",
}

from ._core import get_default_params, solve_once  # noqa: E402,F401
