"""Struct layouts and enumerator values of the drop-in headers: the probe
program that prints them (sizeof, offsetof of every member, every
enumerator), run against either header set.  tests/golden/make_ref_layouts.py
records the reference's (LP/CP_AL/include/cp_al_types.h,
QP/FA_CP/include/fa_cp_types.h) in tests/golden/ref_layouts.json;
tests/test_reference_headers.py holds this repository's headers to it."""
from __future__ import annotations

import subprocess
from pathlib import Path

LP_STRUCTS = {
    "lp_problem_t": ["num_variables", "num_constraints", "variable_lower_bound", "variable_upper_bound",
                     "objective_vector", "objective_constant", "constraint_matrix_row_pointers",
                     "constraint_matrix_col_indices", "constraint_matrix_values", "constraint_matrix_num_nonzeros",
                     "constraint_lower_bound", "constraint_upper_bound", "primal_start", "dual_start"],
    "restart_parameters_t": ["artificial_restart_threshold", "sufficient_reduction_for_restart",
                             "necessary_reduction_for_restart", "k_p", "k_i", "k_d", "i_smooth"],
    "termination_criteria_t": ["eps_optimal_relative", "eps_feasible_relative", "eps_feas_polish_relative",
                               "time_sec_limit", "iteration_limit"],
    "cp_al_parameters_t": ["l_inf_ruiz_iterations", "has_pock_chambolle_alpha", "pock_chambolle_alpha",
                           "bound_objective_rescaling", "verbose", "termination_evaluation_frequency",
                           "sv_max_iter", "sv_tol", "termination_criteria", "restart_params",
                           "reflection_coefficient", "feasibility_polishing", "optimality_norm", "presolve",
                           "matrix_zero_tol"],
    "cp_al_result_t": ["num_variables", "num_constraints", "num_nonzeros", "num_reduced_variables",
                       "num_reduced_constraints", "num_reduced_nonzeros", "primal_solution", "dual_solution",
                       "reduced_cost", "total_count", "rescaling_time_sec", "cumulative_time_sec", "presolve_time",
                       "presolve_status", "absolute_primal_residual", "relative_primal_residual",
                       "absolute_dual_residual", "relative_dual_residual", "primal_objective_value",
                       "dual_objective_value", "objective_gap", "relative_objective_gap",
                       "max_primal_ray_infeasibility", "max_dual_ray_infeasibility", "primal_ray_linear_objective",
                       "dual_ray_objective", "termination_reason", "feasibility_polishing_time",
                       "feasibility_iteration"],
    "matrix_desc_t": ["m", "n", "fmt", "data", "data.dense.A", "data.csr.nnz", "data.csr.row_ptr",
                      "data.csr.col_ind", "data.csr.vals", "data.csc.nnz", "data.csc.col_ptr", "data.csc.row_ind",
                      "data.csc.vals", "data.coo.nnz", "data.coo.row_ind", "data.coo.col_ind", "data.coo.vals"],
}
QP_STRUCTS = {
    "CsrComponent": ["row_ptr", "col_ind", "val"],
    "qp_problem_t": ["num_variables", "num_constraints", "num_rank_lowrank_obj", "variable_lower_bound",
                     "variable_upper_bound", "objective_vector", "objective_constant", "constraint_matrix",
                     "constraint_matrix_num_nonzeros", "objective_sparse_matrix",
                     "objective_sparse_matrix_num_nonzeros", "objective_lowrank_matrix",
                     "objective_lowrank_matrix_num_nonzeros", "constraint_lower_bound", "constraint_upper_bound",
                     "primal_start", "dual_start"],
    "restart_parameters_t": LP_STRUCTS["restart_parameters_t"],
    "termination_criteria_t": ["eps_optimal_relative", "eps_feasible_relative", "eps_feas_polish_relative",
                               "eps_infeasible", "time_sec_limit", "iteration_limit"],
    "fa_cp_parameters_t": ["l_inf_ruiz_iterations", "has_pock_chambolle_alpha", "pock_chambolle_alpha",
                           "bound_objective_rescaling", "trajectory_csv", "use_al_qp", "al_sigma",
                           "sigma_update_rule", "sigma_update_gain", "sigma_clip_low", "sigma_clip_high",
                           "sigma_min", "sigma_max", "sigma_rollback_tol", "sigma_zero_threshold",
                           "sigma_activation_threshold", "sigma_normal_motion_threshold", "sigma_activation_value",
                           "verbose", "termination_evaluation_frequency", "sv_max_iter", "sv_tol",
                           "termination_criteria", "restart_params", "reflection_coefficient",
                           "feasibility_polishing", "optimality_norm"],
    "fa_cp_result_t": ["num_variables", "num_constraints", "num_nonzeros", "num_reduced_variables",
                       "num_reduced_constraints", "num_reduced_nonzeros", "primal_solution", "dual_solution",
                       "reduced_cost", "total_count", "total_inner_count", "rescaling_time_sec",
                       "cumulative_time_sec", "absolute_primal_residual", "relative_primal_residual",
                       "absolute_dual_residual", "relative_dual_residual", "primal_objective_value",
                       "dual_objective_value", "objective_gap", "relative_objective_gap",
                       "max_primal_ray_infeasibility", "max_dual_ray_infeasibility", "primal_ray_linear_objective",
                       "dual_ray_objective", "final_al_sigma", "sigma_update_count", "sigma_update_rule",
                       "termination_reason", "feasibility_polishing_time", "feasibility_iteration"],
    "matrix_desc_t": ["m", "n", "fmt", "zero_tolerance", "data", "data.dense.A", "data.csr.nnz", "data.csr.row_ptr",
                      "data.csr.col_ind", "data.csr.vals", "data.csc.nnz", "data.csc.col_ptr", "data.csc.row_ind",
                      "data.csc.vals", "data.coo.nnz", "data.coo.row_ind", "data.coo.col_ind", "data.coo.vals"],
}
COMMON_ENUMS = ["TERMINATION_REASON_UNSPECIFIED", "TERMINATION_REASON_OPTIMAL", "TERMINATION_REASON_PRIMAL_INFEASIBLE",
                "TERMINATION_REASON_DUAL_INFEASIBLE", "TERMINATION_REASON_INFEASIBLE_OR_UNBOUNDED",
                "TERMINATION_REASON_TIME_LIMIT", "TERMINATION_REASON_ITERATION_LIMIT",
                "TERMINATION_REASON_FEAS_POLISH_SUCCESS", "NORM_TYPE_L2", "NORM_TYPE_L_INF", "matrix_dense",
                "matrix_csr", "matrix_csc", "matrix_coo"]
QP_ENUMS = COMMON_ENUMS + ["FA_CP_SPARSE_Q", "FA_CP_DIAG_Q", "FA_CP_LOW_RANK_PLUS_SPARSE_Q", "FA_CP_LOW_RANK_Q",
                           "FA_CP_NON_Q", "FA_CP_SIGMA_UPDATE_FIXED", "FA_CP_SIGMA_UPDATE_RESIDUAL_BALANCE",
                           "FA_CP_SIGMA_UPDATE_KKT_BALANCE", "FA_CP_SIGMA_UPDATE_DISPLACEMENT",
                           "FA_CP_SIGMA_UPDATE_PROGRESS", "FA_CP_SIGMA_UPDATE_GREEDY_SCORE",
                           "FA_CP_SIGMA_UPDATE_GUARDED", "FA_CP_SIGMA_UPDATE_BALANCED_GUARDED"]


def probe_source(kind: str) -> str:
    header, structs, enums = (("cp_al_types.h", LP_STRUCTS, COMMON_ENUMS) if kind == "lp"
                              else ("fa_cp_types.h", QP_STRUCTS, QP_ENUMS))
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{header}"', "int main(void) {"]
    for s, fields in structs.items():
        lines.append(f'  printf("{s} %zu\\n", sizeof({s}));')
        for f in fields:
            lines.append(f'  printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    for e in enums:
        lines.append(f'  printf("{e} %d\\n", (int){e});')
    lines += ["  return 0;", "}"]
    return "\n".join(lines) + "\n"


def run_probe(kind: str, include_dirs: list[Path], work: Path) -> dict[str, int]:
    """{name: value} printed by the probe compiled against include_dirs."""
    work.mkdir(parents=True, exist_ok=True)
    src = work / f"probe_{kind}.c"
    exe = work / f"probe_{kind}"
    src.write_text(probe_source(kind))
    cmd = ["gcc", "-std=gnu99"]
    for d in include_dirs:
        cmd += ["-I", str(d)]
    subprocess.run(cmd + [str(src), "-o", str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.check_output([str(exe)], text=True)
    return {k: int(v) for k, v in (line.rsplit(" ", 1) for line in out.splitlines())}
