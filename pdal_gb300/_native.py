"""ctypes mirror of the C interfaces in include/ (cp_al_types.h, cp_al.h,
cp_al_gb300.h for the LP library; fa_cp_types.h, fa_cp.h, fa_cp_gb300.h for
the QP library), plus the loader of the in-tree libraries.

The loader never falls back to anything: if the CUDA library is missing it
raises, so a product path cannot silently run elsewhere.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIBDIR = Path(__file__).resolve().parent / "lib"

TERMINATION_REASONS = {
    0: "UNSPECIFIED",
    1: "OPTIMAL",
    2: "PRIMAL_INFEASIBLE",
    3: "DUAL_INFEASIBLE",
    4: "INFEASIBLE_OR_UNBOUNDED",
    5: "TIME_LIMIT",
    6: "ITERATION_LIMIT",
    7: "FEAS_POLISH_SUCCESS",
}

NORM_L2, NORM_LINF = 0, 1
MATRIX_DENSE, MATRIX_CSR, MATRIX_CSC, MATRIX_COO = 0, 1, 2, 3
PRECISION_FP64, PRECISION_FP32_REFINE = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class LpProblem(C.Structure):
    _fields_ = [
        ("num_variables", C.c_int),
        ("num_constraints", C.c_int),
        ("variable_lower_bound", _dp),
        ("variable_upper_bound", _dp),
        ("objective_vector", _dp),
        ("objective_constant", C.c_double),
        ("constraint_matrix_row_pointers", _ip),
        ("constraint_matrix_col_indices", _ip),
        ("constraint_matrix_values", _dp),
        ("constraint_matrix_num_nonzeros", C.c_int),
        ("constraint_lower_bound", _dp),
        ("constraint_upper_bound", _dp),
        ("primal_start", _dp),
        ("dual_start", _dp),
    ]


class RestartParams(C.Structure):
    _fields_ = [
        ("artificial_restart_threshold", C.c_double),
        ("sufficient_reduction_for_restart", C.c_double),
        ("necessary_reduction_for_restart", C.c_double),
        ("k_p", C.c_double),
        ("k_i", C.c_double),
        ("k_d", C.c_double),
        ("i_smooth", C.c_double),
    ]


class TerminationCriteria(C.Structure):
    _fields_ = [
        ("eps_optimal_relative", C.c_double),
        ("eps_feasible_relative", C.c_double),
        ("eps_feas_polish_relative", C.c_double),
        ("time_sec_limit", C.c_double),
        ("iteration_limit", C.c_int),
    ]


class CpalParameters(C.Structure):
    _fields_ = [
        ("l_inf_ruiz_iterations", C.c_int),
        ("has_pock_chambolle_alpha", C.c_bool),
        ("pock_chambolle_alpha", C.c_double),
        ("bound_objective_rescaling", C.c_bool),
        ("verbose", C.c_bool),
        ("termination_evaluation_frequency", C.c_int),
        ("sv_max_iter", C.c_int),
        ("sv_tol", C.c_double),
        ("termination_criteria", TerminationCriteria),
        ("restart_params", RestartParams),
        ("reflection_coefficient", C.c_double),
        ("feasibility_polishing", C.c_bool),
        ("optimality_norm", C.c_int),
        ("presolve", C.c_bool),
        ("matrix_zero_tol", C.c_double),
    ]


class CpalResult(C.Structure):
    _fields_ = [
        ("num_variables", C.c_int),
        ("num_constraints", C.c_int),
        ("num_nonzeros", C.c_int),
        ("num_reduced_variables", C.c_int),
        ("num_reduced_constraints", C.c_int),
        ("num_reduced_nonzeros", C.c_int),
        ("primal_solution", _dp),
        ("dual_solution", _dp),
        ("reduced_cost", _dp),
        ("total_count", C.c_int),
        ("rescaling_time_sec", C.c_double),
        ("cumulative_time_sec", C.c_double),
        ("presolve_time", C.c_double),
        ("presolve_status", C.c_int),
        ("absolute_primal_residual", C.c_double),
        ("relative_primal_residual", C.c_double),
        ("absolute_dual_residual", C.c_double),
        ("relative_dual_residual", C.c_double),
        ("primal_objective_value", C.c_double),
        ("dual_objective_value", C.c_double),
        ("objective_gap", C.c_double),
        ("relative_objective_gap", C.c_double),
        ("max_primal_ray_infeasibility", C.c_double),
        ("max_dual_ray_infeasibility", C.c_double),
        ("primal_ray_linear_objective", C.c_double),
        ("dual_ray_objective", C.c_double),
        ("termination_reason", C.c_int),
        ("feasibility_polishing_time", C.c_double),
        ("feasibility_iteration", C.c_int),
    ]


class _Dense(C.Structure):
    _fields_ = [("A", _dp)]


class _Csr(C.Structure):
    _fields_ = [("nnz", C.c_int), ("row_ptr", _ip), ("col_ind", _ip), ("vals", _dp)]


class _Csc(C.Structure):
    _fields_ = [("nnz", C.c_int), ("col_ptr", _ip), ("row_ind", _ip), ("vals", _dp)]


class _Coo(C.Structure):
    _fields_ = [("nnz", C.c_int), ("row_ind", _ip), ("col_ind", _ip), ("vals", _dp)]


class _MatrixData(C.Union):
    _fields_ = [("dense", _Dense), ("csr", _Csr), ("csc", _Csc), ("coo", _Coo)]


class MatrixDesc(C.Structure):
    """LP/CP_AL/include/cp_al_types.h:145-189 (the CP_AL layout, without
    FA_CP's zero_tolerance member)."""

    _fields_ = [("m", C.c_int), ("n", C.c_int), ("fmt", C.c_int), ("data", _MatrixData)]


class CpalOptions(C.Structure):
    _fields_ = [
        ("al_lambda", C.c_double),
        ("sigma_mode", C.c_int),
        ("sigma_set", C.c_int),
        ("sigma", C.c_double),
        ("sigma_adaptive", C.c_int),
        ("sigma_init_factor", C.c_double),
        ("sigma_min_factor", C.c_double),
        ("sigma_max_factor", C.c_double),
        ("lambda_factor", C.c_double),
        ("lambda_param_set", C.c_int),
        ("lambda_param", C.c_double),
        ("sigma_balance_gain", C.c_double),
        ("sigma_i_smooth", C.c_double),
        ("sigma_kp", C.c_double),
        ("sigma_ki", C.c_double),
        ("sigma_kd", C.c_double),
        ("sigma_update_min", C.c_double),
        ("sigma_update_max", C.c_double),
        ("step_margin", C.c_double),
        ("restart_sufficient", C.c_double),
        ("restart_necessary", C.c_double),
        ("restart_artificial", C.c_double),
        ("restart_select", C.c_int),
        ("restart_select_margin", C.c_double),
        ("restart_select_min_iters", C.c_int),
        ("restart_select_threepoint", C.c_int),
        ("restart_select_min_time", C.c_double),
        ("cr_iterations", C.c_int),
        ("cr_early_stop", C.c_int),
        ("cr_early_stop_threshold", C.c_double),
        ("precision", C.c_int),
        ("fp32_switch_tol", C.c_double),
        ("fp32_max_iterations", C.c_int),
        ("spmv_nnz_per_block", C.c_int),
        ("device", C.c_int),
        ("graph_blocks", C.c_int),
        ("timing", C.c_int),
        ("fp32_stall_evals", C.c_int),
        ("batch_blocks_per_sm", C.c_int),
        ("dual_panels", C.c_int),
        ("panel_width", C.c_int),
        ("primal_hot_rows", C.c_int),
        ("power_method", C.c_int),
        ("primal_staged", C.c_int),
        ("infeasibility_detection", C.c_int),
        ("eps_infeasible", C.c_double),
        ("persistent_loop", C.c_int),
        ("dual_fused_finish", C.c_int),
        ("device_transpose", C.c_int),
        ("alpha_direct_pulse", C.c_int),
        ("pulse_force", C.c_int),
        ("pulse_trace", C.c_int),
        ("pulse_test_limit", C.c_int),
        ("sigma_trigger", C.c_int),
        ("sigma_trigger_min_iters", C.c_int),
        ("sigma_trigger_primal", C.c_double),
        ("sigma_trigger_dual", C.c_double),
        ("sigma_trigger_ratio", C.c_double),
        ("dynamic_eval", C.c_int),
        ("dynamic_eval_fast", C.c_int),
        ("dynamic_eval_after_sec", C.c_double),
        ("dynamic_eval_after_iters", C.c_int),
        ("dynamic_eval_min_iters", C.c_int),
        ("dynamic_eval_small_res", C.c_double),
        ("dynamic_eval_large_res", C.c_double),
        ("dynamic_eval_ratio", C.c_double),
        ("dynamic_eval_bootstrap_iters", C.c_int),
        ("dual_concurrent", C.c_int),
    ]


class CpalStats(C.Structure):
    _fields_ = [
        ("setup_sec", C.c_double),
        ("loop_sec", C.c_double),
        ("total_sec", C.c_double),
        ("lambda_est", C.c_double),
        ("power_iterations", C.c_int),
        ("restarts", C.c_int),
        ("fp32_iterations", C.c_int),
        ("kernel_launches", C.c_int64),
        ("h2d_bytes", C.c_int64),
        ("d2h_bytes", C.c_int64),
        ("primal_weight", C.c_double),
        ("step_size", C.c_double),
        ("al_penalty", C.c_double),
        ("avg_primal_ms", C.c_double),
        ("avg_dual_ms", C.c_double),
        ("avg_block_ms", C.c_double),
        ("timed_blocks", C.c_int),
        ("avg_primal32_ms", C.c_double),
        ("avg_dual32_ms", C.c_double),
        ("avg_block32_ms", C.c_double),
        ("timed_blocks32", C.c_int),
        ("prepare_sec", C.c_double),
        ("upload_sec", C.c_double),
        ("equilibration_sec", C.c_double),
        ("power_sec", C.c_double),
        ("polish_primal_status", C.c_int),
        ("polish_dual_status", C.c_int),
        ("cr_passes", C.c_int),
        ("panel_rows", C.c_int),
        ("panels", C.c_int),
        ("avg_dual_rows_ms", C.c_double),
        ("avg_dual_panels_ms", C.c_double),
        ("avg_dual_rows32_ms", C.c_double),
        ("avg_dual_panels32_ms", C.c_double),
        ("pulse_start_iteration", C.c_int),
        ("pulse_gate", C.c_int),
        ("sigma_trigger_iteration", C.c_int),
        ("dynamic_eval_iteration", C.c_int),
        ("upload_plan_sec", C.c_double),
        ("upload_alloc_sec", C.c_double),
    ]


class BatchStats(C.Structure):
    _fields_ = [
        ("instances", C.c_int),
        ("optimal", C.c_int),
        ("grid_blocks", C.c_int),
        ("host_prep_sec", C.c_double),
        ("upload_sec", C.c_double),
        ("kernel_sec", C.c_double),
        ("download_sec", C.c_double),
        ("total_sec", C.c_double),
        ("solves_per_sec", C.c_double),
        ("iterations_p50", C.c_int),
        ("iterations_p99", C.c_int),
        ("iterations_max", C.c_int),
        ("total_iterations", C.c_longlong),
        ("device_bytes", C.c_longlong),
        ("block_nnz", C.c_int),
        ("blocks_per_sm", C.c_int),
        ("tune_sec", C.c_double),
    ]


class InstanceInfo(C.Structure):
    _fields_ = [
        ("sigma", C.c_double),
        ("sigma_best", C.c_double),
        ("primal_weight", C.c_double),
        ("step_size", C.c_double),
        ("lambda_est", C.c_double),
        ("restarts", C.c_int),
        ("power_iterations", C.c_int),
        ("fp32_iterations", C.c_int),
    ]


class FeatureStats(C.Structure):
    """cp_al_feature_stats_t (include/cp_al_policy.h)."""
    _fields_ = [(f, C.c_double) for f in (
        "coeff_log_range", "row_logmax_std", "col_logmax_std", "row_logspan_mean", "col_logspan_mean",
        "row_span2_fraction", "col_span2_fraction", "row_nnz_cv", "col_nnz_cv", "equality_fraction",
        "two_sided_variable_fraction", "objective_density")]


SOLVE_FN = C.CFUNCTYPE(C.c_void_p, C.POINTER(LpProblem), C.POINTER(CpalParameters))

# name -> (restype, argtypes); every symbol include/cp_al.h,
# include/cp_al_gb300.h and include/cp_al_policy.h declare
LP_SYMBOLS = {
    "create_lp_problem": (C.POINTER(LpProblem), [_dp, C.POINTER(MatrixDesc), _dp, _dp, _dp, _dp, _dp]),
    "set_start_values": (None, [C.POINTER(LpProblem), _dp, _dp]),
    "solve_lp_problem": (C.POINTER(CpalResult), [C.POINTER(LpProblem), C.POINTER(CpalParameters)]),
    "set_default_parameters": (None, [C.POINTER(CpalParameters)]),
    "cp_al_result_free": (None, [C.POINTER(CpalResult)]),
    "lp_problem_free": (None, [C.POINTER(LpProblem)]),
    "cp_al_gb300_default_options": (None, [C.POINTER(CpalOptions)]),
    "cp_al_gb300_options_from_env": (None, [C.POINTER(CpalOptions)]),
    "cp_al_gb300_solve": (
        C.POINTER(CpalResult),
        [C.POINTER(LpProblem), C.POINTER(CpalParameters), C.POINTER(CpalOptions)],
    ),
    "cp_al_gb300_last_stats": (None, [C.POINTER(CpalStats)]),
    "cp_al_gb300_last_error": (C.c_char_p, []),
    "cp_al_gb300_unbuilt_switch": (C.c_char_p, []),
    "cp_al_gb300_session_create": (
        C.c_void_p,
        [C.POINTER(LpProblem), C.POINTER(CpalParameters), C.POINTER(CpalOptions)],
    ),
    "cp_al_gb300_session_solve": (C.c_int, [C.c_void_p, C.POINTER(CpalResult)]),
    "cp_al_gb300_session_fetch": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "cp_al_gb300_session_free": (None, [C.c_void_p]),
    "cp_al_gb300_session_scaling": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp]),
    "cp_al_gb300_session_start": (C.c_int, [C.c_void_p]),
    "cp_al_gb300_session_iterate": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(CpalResult)]),
    "cp_al_gb300_batch_solve": (
        C.c_int,
        [C.c_int, C.POINTER(C.POINTER(LpProblem)), C.POINTER(CpalParameters), C.POINTER(CpalOptions), _dp,
         C.POINTER(C.POINTER(CpalResult)), C.POINTER(InstanceInfo), C.POINTER(BatchStats)],
    ),
    "read_mps_file": (C.POINTER(LpProblem), [C.c_char_p]),
    "cp_al_gb300_batch_tune": (
        C.c_int,
        [C.c_int, C.POINTER(C.POINTER(LpProblem)), C.POINTER(CpalParameters), C.POINTER(CpalOptions),
         C.POINTER(BatchStats)],
    ),
    "cp_al_feature_stats": (C.c_int, [C.POINTER(LpProblem), C.POINTER(FeatureStats)]),
    "cp_al_unified_policy": (C.c_char_p, [C.POINTER(FeatureStats)]),
    "cp_al_feature_policy": (C.c_int, [C.POINTER(LpProblem), C.POINTER(CpalParameters), C.POINTER(FeatureStats)]),
    "cp_al_structural_tail": (
        C.POINTER(CpalResult), [C.POINTER(LpProblem), C.POINTER(CpalParameters), C.POINTER(FeatureStats), C.c_int]),
    "cp_al_policy_set_solver": (None, [SOLVE_FN]),
    "cp_al_gb300_primal_kkt_noalloc": (
        C.c_int,
        [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
         C.c_void_p, C.c_void_p],
    ),
}

_LIBS: dict[str, C.CDLL] = {}


# ---------------------------------------------------------------- FA_CP (QP)

SIGMA_RULES = {
    "fixed": 0, "residual_balance": 1, "kkt_balance": 2, "displacement": 3,
    "progress": 4, "greedy_score": 5, "guarded": 6, "balanced_guarded": 7,
}
Q_TYPES = {0: "SPARSE_Q", 1: "DIAG_Q", 2: "LOW_RANK_PLUS_SPARSE_Q", 3: "LOW_RANK_Q", 4: "NON_Q"}


class CsrComponent(C.Structure):
    _fields_ = [("row_ptr", _ip), ("col_ind", _ip), ("val", _dp)]


class QpProblem(C.Structure):
    """QP/FA_CP/include/fa_cp_types.h:56-83"""

    _fields_ = [
        ("num_variables", C.c_int),
        ("num_constraints", C.c_int),
        ("num_rank_lowrank_obj", C.c_int),
        ("variable_lower_bound", _dp),
        ("variable_upper_bound", _dp),
        ("objective_vector", _dp),
        ("objective_constant", C.c_double),
        ("constraint_matrix", C.POINTER(CsrComponent)),
        ("constraint_matrix_num_nonzeros", C.c_int),
        ("objective_sparse_matrix", C.POINTER(CsrComponent)),
        ("objective_sparse_matrix_num_nonzeros", C.c_int),
        ("objective_lowrank_matrix", C.POINTER(CsrComponent)),
        ("objective_lowrank_matrix_num_nonzeros", C.c_int),
        ("constraint_lower_bound", _dp),
        ("constraint_upper_bound", _dp),
        ("primal_start", _dp),
        ("dual_start", _dp),
    ]


class FacpTerminationCriteria(C.Structure):
    _fields_ = [
        ("eps_optimal_relative", C.c_double),
        ("eps_feasible_relative", C.c_double),
        ("eps_feas_polish_relative", C.c_double),
        ("eps_infeasible", C.c_double),
        ("time_sec_limit", C.c_double),
        ("iteration_limit", C.c_int),
    ]


class FacpParameters(C.Structure):
    """QP/FA_CP/include/fa_cp_types.h:111-139"""

    _fields_ = [
        ("l_inf_ruiz_iterations", C.c_int),
        ("has_pock_chambolle_alpha", C.c_bool),
        ("pock_chambolle_alpha", C.c_double),
        ("bound_objective_rescaling", C.c_bool),
        ("trajectory_csv", C.c_char_p),
        ("use_al_qp", C.c_bool),
        ("al_sigma", C.c_double),
        ("sigma_update_rule", C.c_int),
        ("sigma_update_gain", C.c_double),
        ("sigma_clip_low", C.c_double),
        ("sigma_clip_high", C.c_double),
        ("sigma_min", C.c_double),
        ("sigma_max", C.c_double),
        ("sigma_rollback_tol", C.c_double),
        ("sigma_zero_threshold", C.c_double),
        ("sigma_activation_threshold", C.c_double),
        ("sigma_normal_motion_threshold", C.c_double),
        ("sigma_activation_value", C.c_double),
        ("verbose", C.c_int),
        ("termination_evaluation_frequency", C.c_int),
        ("sv_max_iter", C.c_int),
        ("sv_tol", C.c_double),
        ("termination_criteria", FacpTerminationCriteria),
        ("restart_params", RestartParams),
        ("reflection_coefficient", C.c_double),
        ("feasibility_polishing", C.c_bool),
        ("optimality_norm", C.c_int),
    ]


class FacpResult(C.Structure):
    """QP/FA_CP/include/fa_cp_types.h:141-176"""

    _fields_ = [
        ("num_variables", C.c_int),
        ("num_constraints", C.c_int),
        ("num_nonzeros", C.c_int),
        ("num_reduced_variables", C.c_int),
        ("num_reduced_constraints", C.c_int),
        ("num_reduced_nonzeros", C.c_int),
        ("primal_solution", _dp),
        ("dual_solution", _dp),
        ("reduced_cost", _dp),
        ("total_count", C.c_int),
        ("total_inner_count", C.c_int),
        ("rescaling_time_sec", C.c_double),
        ("cumulative_time_sec", C.c_double),
        ("absolute_primal_residual", C.c_double),
        ("relative_primal_residual", C.c_double),
        ("absolute_dual_residual", C.c_double),
        ("relative_dual_residual", C.c_double),
        ("primal_objective_value", C.c_double),
        ("dual_objective_value", C.c_double),
        ("objective_gap", C.c_double),
        ("relative_objective_gap", C.c_double),
        ("max_primal_ray_infeasibility", C.c_double),
        ("max_dual_ray_infeasibility", C.c_double),
        ("primal_ray_linear_objective", C.c_double),
        ("dual_ray_objective", C.c_double),
        ("final_al_sigma", C.c_double),
        ("sigma_update_count", C.c_int),
        ("sigma_update_rule", C.c_int),
        ("termination_reason", C.c_int),
        ("feasibility_polishing_time", C.c_double),
        ("feasibility_iteration", C.c_int),
    ]


class QpMatrixDesc(C.Structure):
    """QP/FA_CP/include/fa_cp_types.h:178-222 (CP_AL's layout plus zero_tolerance)."""

    _fields_ = [("m", C.c_int), ("n", C.c_int), ("fmt", C.c_int), ("zero_tolerance", C.c_double),
                ("data", _MatrixData)]


class FacpOptions(C.Structure):
    _fields_ = [
        ("device", C.c_int),
        ("blocks_per_sm", C.c_int),
        ("restart_select", C.c_int),
        ("restart_select_margin", C.c_double),
        ("restart_select_min_iters", C.c_int),
        ("restart_select_min_time", C.c_double),
        ("precision", C.c_int),
        ("fp32_switch_tol", C.c_double),
        ("fp32_stall_evals", C.c_int),
        ("barrier_spin_limit", C.c_longlong),
        ("barrier_extra_arrivals", C.c_int),
    ]


class FacpStats(C.Structure):
    _fields_ = [
        ("setup_sec", C.c_double),
        ("loop_sec", C.c_double),
        ("total_sec", C.c_double),
        ("max_singular_value", C.c_double),
        ("q_norm", C.c_double),
        ("q_nonconvexity", C.c_double),
        ("q_type", C.c_int),
        ("grid_blocks", C.c_int),
        ("restarts", C.c_int),
        ("evaluations", C.c_int),
        ("kernel_launches", C.c_int64),
        ("inner_iterations", C.c_int64),
        ("primal_weight", C.c_double),
        ("step_size", C.c_double),
        ("device_loop_ms", C.c_double),
        ("equilibration_sec", C.c_double),
        ("upload_sec", C.c_double),
        ("power_sec", C.c_double),
        ("power_iterations_a", C.c_int),
        ("power_iterations_q", C.c_int),
        ("fp32_iterations", C.c_int),
        ("polish_primal_status", C.c_int),
        ("polish_dual_status", C.c_int),
    ]


QP_SYMBOLS = {
    "create_qp_problem": (
        C.POINTER(QpProblem),
        [_dp, C.POINTER(QpMatrixDesc), C.POINTER(QpMatrixDesc), C.POINTER(QpMatrixDesc), _dp, _dp, _dp, _dp, _dp],
    ),
    "set_start_values": (None, [C.POINTER(QpProblem), _dp, _dp]),
    "solve_qp_problem": (C.POINTER(FacpResult), [C.POINTER(QpProblem), C.POINTER(FacpParameters)]),
    "set_default_parameters": (None, [C.POINTER(FacpParameters)]),
    "fa_cp_result_free": (None, [C.POINTER(FacpResult)]),
    "qp_problem_free": (None, [C.POINTER(QpProblem)]),
    "fa_cp_gb300_default_options": (None, [C.POINTER(FacpOptions)]),
    "fa_cp_gb300_options_from_env": (None, [C.POINTER(FacpOptions)]),
    "fa_cp_gb300_solve": (
        C.POINTER(FacpResult),
        [C.POINTER(QpProblem), C.POINTER(FacpParameters), C.POINTER(FacpOptions)],
    ),
    "fa_cp_gb300_last_stats": (None, [C.POINTER(FacpStats)]),
    "fa_cp_gb300_last_error": (C.c_char_p, []),
    "fa_cp_gb300_rand_sequence": (None, [C.c_uint, C.c_int, _ip]),
    "read_mps_file": (C.POINTER(QpProblem), [C.c_char_p]),
    "fa_cp_gb300_scaling": (
        C.c_int, [C.POINTER(QpProblem), C.POINTER(FacpParameters), C.POINTER(FacpOptions), _dp, _dp, _dp],
    ),
}


# ---------------------------------------------------------------- learned warm start

_fp = C.POINTER(C.c_float)
LEARN_SYMBOLS = {
    "pdal_mlp_create": (C.c_void_p, [C.c_int, C.c_int, C.c_int, C.c_uint, C.c_int]),
    "pdal_mlp_free": (None, [C.c_void_p]),
    "pdal_mlp_num_params": (C.c_longlong, [C.c_void_p]),
    "pdal_mlp_get_params": (C.c_int, [C.c_void_p, _fp]),
    "pdal_mlp_set_params": (C.c_int, [C.c_void_p, _fp]),
    "pdal_mlp_set_data": (C.c_int, [C.c_void_p, C.c_int, _fp, _fp]),
    "pdal_mlp_train": (C.c_double, [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_uint]),
    "pdal_mlp_loss_grad": (C.c_double, [C.c_void_p, C.c_int, _fp, _fp, _fp]),
    "pdal_mlp_predict": (C.c_int, [C.c_void_p, C.c_int, _fp, _fp, C.c_int]),
    "pdal_mlp_last_error": (C.c_char_p, []),
    "pdal_transport_warm_start": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int] + [_dp] * 7 + [C.c_int]
                                  + [_dp] * 5),
}


def load_learn() -> C.CDLL:
    return load("libpdal_learn_gb300.so", LEARN_SYMBOLS)


def lib_path(name: str) -> Path:
    return LIBDIR / name


def load(name: str, symbols: dict) -> C.CDLL:
    if name in _LIBS:
        return _LIBS[name]
    path = lib_path(name)
    if not path.exists():
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first (python -m pdal_gb300.build); "
            "there is no CPU fallback"
        )
    lib = C.CDLL(str(path))
    for sym, (res, args) in symbols.items():
        fn = getattr(lib, sym)
        fn.restype = res
        fn.argtypes = args
    _LIBS[name] = lib
    return lib


def load_lp() -> C.CDLL:
    return load("libcp_al_gb300.so", LP_SYMBOLS)


def load_qp() -> C.CDLL:
    return load("libfa_cp_gb300.so", QP_SYMBOLS)


def last_error(lib: C.CDLL) -> str:
    fn = getattr(lib, "fa_cp_gb300_last_error", None) or lib.cp_al_gb300_last_error
    msg = fn()
    return msg.decode() if msg else ""
