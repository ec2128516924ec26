/*
 * fa_cp_types.h -- data types of the FA_CP (convex QP) C interface.
 *
 * Member order, types and enumerator values are those of the FA_CP reference
 * interface (QP/FA_CP/include/fa_cp_types.h:28-222) so that callers compiled
 * against it link against libfa_cp_gb300.so unchanged.  This header and
 * cp_al_types.h define the same enum names with the reference's values and
 * are not meant to be included in the same translation unit (the two
 * reference libraries are separate too).
 */
#pragma once

#include <stdbool.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TERMINATION_REASON_UNSPECIFIED,
    TERMINATION_REASON_OPTIMAL,
    TERMINATION_REASON_PRIMAL_INFEASIBLE,
    TERMINATION_REASON_DUAL_INFEASIBLE,
    TERMINATION_REASON_INFEASIBLE_OR_UNBOUNDED,
    TERMINATION_REASON_TIME_LIMIT,
    TERMINATION_REASON_ITERATION_LIMIT,
    TERMINATION_REASON_FEAS_POLISH_SUCCESS
} termination_reason_t;

typedef enum { NORM_TYPE_L2 = 0, NORM_TYPE_L_INF = 1 } norm_type_t;

typedef struct {
    int *row_ptr;
    int *col_ind;
    double *val;
} CsrComponent;

typedef enum {
    FA_CP_SPARSE_Q,
    FA_CP_DIAG_Q,
    FA_CP_LOW_RANK_PLUS_SPARSE_Q,
    FA_CP_LOW_RANK_Q,
    FA_CP_NON_Q
} quad_obj_type_t;

/* QP/FA_CP/include/fa_cp_types.h:56-83: min 1/2 x'Qx + c'x (Q = sparse part +
 * R'R), con_lb <= A x <= con_ub, var_lb <= x <= var_ub. */
typedef struct {
    int num_variables;
    int num_constraints;
    int num_rank_lowrank_obj;
    double *variable_lower_bound;
    double *variable_upper_bound;
    double *objective_vector;
    double objective_constant;

    CsrComponent *constraint_matrix;
    int constraint_matrix_num_nonzeros;

    CsrComponent *objective_sparse_matrix;
    int objective_sparse_matrix_num_nonzeros;

    CsrComponent *objective_lowrank_matrix;
    int objective_lowrank_matrix_num_nonzeros;

    double *constraint_lower_bound;
    double *constraint_upper_bound;

    double *primal_start;
    double *dual_start;
} qp_problem_t;

typedef struct {
    double artificial_restart_threshold;
    double sufficient_reduction_for_restart;
    double necessary_reduction_for_restart;
    double k_p;
    double k_i;
    double k_d;
    double i_smooth;
} restart_parameters_t;

typedef struct {
    double eps_optimal_relative;
    double eps_feasible_relative;
    double eps_feas_polish_relative;
    double eps_infeasible;
    double time_sec_limit;
    int iteration_limit;
} termination_criteria_t;

typedef enum {
    FA_CP_SIGMA_UPDATE_FIXED = 0,
    FA_CP_SIGMA_UPDATE_RESIDUAL_BALANCE = 1,
    FA_CP_SIGMA_UPDATE_KKT_BALANCE = 2,
    FA_CP_SIGMA_UPDATE_DISPLACEMENT = 3,
    FA_CP_SIGMA_UPDATE_PROGRESS = 4,
    FA_CP_SIGMA_UPDATE_GREEDY_SCORE = 5,
    FA_CP_SIGMA_UPDATE_GUARDED = 6,
    FA_CP_SIGMA_UPDATE_BALANCED_GUARDED = 7
} sigma_update_rule_t;

/* QP/FA_CP/include/fa_cp_types.h:111-139 */
typedef struct {
    int l_inf_ruiz_iterations;
    bool has_pock_chambolle_alpha;
    double pock_chambolle_alpha;
    bool bound_objective_rescaling;
    const char *trajectory_csv;
    bool use_al_qp;
    double al_sigma;
    sigma_update_rule_t sigma_update_rule;
    double sigma_update_gain;
    double sigma_clip_low;
    double sigma_clip_high;
    double sigma_min;
    double sigma_max;
    double sigma_rollback_tol;
    double sigma_zero_threshold;
    double sigma_activation_threshold;
    double sigma_normal_motion_threshold;
    double sigma_activation_value;
    int verbose;
    int termination_evaluation_frequency;
    int sv_max_iter;
    double sv_tol;
    termination_criteria_t termination_criteria;
    restart_parameters_t restart_params;
    double reflection_coefficient;
    bool feasibility_polishing;
    norm_type_t optimality_norm;
} fa_cp_parameters_t;

/* QP/FA_CP/include/fa_cp_types.h:141-176 */
typedef struct {
    int num_variables;
    int num_constraints;
    int num_nonzeros;

    int num_reduced_variables;
    int num_reduced_constraints;
    int num_reduced_nonzeros;

    double *primal_solution;
    double *dual_solution;
    double *reduced_cost;

    int total_count;
    int total_inner_count;
    double rescaling_time_sec;
    double cumulative_time_sec;

    double absolute_primal_residual;
    double relative_primal_residual;
    double absolute_dual_residual;
    double relative_dual_residual;
    double primal_objective_value;
    double dual_objective_value;
    double objective_gap;
    double relative_objective_gap;
    double max_primal_ray_infeasibility;
    double max_dual_ray_infeasibility;
    double primal_ray_linear_objective;
    double dual_ray_objective;
    double final_al_sigma;
    int sigma_update_count;
    sigma_update_rule_t sigma_update_rule;
    termination_reason_t termination_reason;
    double feasibility_polishing_time;
    int feasibility_iteration;
} fa_cp_result_t;

typedef enum { matrix_dense = 0, matrix_csr = 1, matrix_csc = 2, matrix_coo = 3 } matrix_format_t;

/* QP/FA_CP/include/fa_cp_types.h:178-222 (adds zero_tolerance to CP_AL's). */
typedef struct {
    int m;
    int n;
    matrix_format_t fmt;
    double zero_tolerance; /* |x| <= zero_tolerance is dropped */

    union MatrixData {
        struct MatrixDense {
            const double *A;
        } dense;
        struct MatrixCSR {
            int nnz;
            const int *row_ptr;
            const int *col_ind;
            const double *vals;
        } csr;
        struct MatrixCSC {
            int nnz;
            const int *col_ptr;
            const int *row_ind;
            const double *vals;
        } csc;
        struct MatrixCOO {
            int nnz;
            const int *row_ind;
            const int *col_ind;
            const double *vals;
        } coo;
    } data;
} matrix_desc_t;

#ifdef __cplusplus
} /* extern "C" */
#endif
