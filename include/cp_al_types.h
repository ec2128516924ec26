/*
 * cp_al_types.h -- data types of the CP_AL (LP) C interface.
 *
 * These structs and enums must keep the exact member order, types and
 * enumerator values of the CP_AL reference interface
 * (LP/CP_AL/include/cp_al_types.h:29-189) so that a caller compiled against
 * the reference header can link against libcp_al_gb300.so unchanged.  The only
 * difference is that the reference's `#include "PSLP_stats.h"` (presolve
 * statistics, cp_al_types.h:20) is dropped: no member of these structs uses it.
 */
#pragma once

#include <stdbool.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

/* LP/CP_AL/include/cp_al_types.h:29-39 */
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

/* LP/CP_AL/include/cp_al_types.h:41-45 */
typedef enum { NORM_TYPE_L2 = 0, NORM_TYPE_L_INF = 1 } norm_type_t;

/* LP/CP_AL/include/cp_al_types.h:47-66: the problem in CSR form, owned by the
 * caller of create_lp_problem and released by lp_problem_free. */
typedef struct {
    int num_variables;
    int num_constraints;
    double *variable_lower_bound;
    double *variable_upper_bound;
    double *objective_vector;
    double objective_constant;

    int *constraint_matrix_row_pointers;
    int *constraint_matrix_col_indices;
    double *constraint_matrix_values;
    int constraint_matrix_num_nonzeros;

    double *constraint_lower_bound;
    double *constraint_upper_bound;

    double *primal_start;
    double *dual_start;
} lp_problem_t;

/* LP/CP_AL/include/cp_al_types.h:68-77 */
typedef struct {
    double artificial_restart_threshold;
    double sufficient_reduction_for_restart;
    double necessary_reduction_for_restart;
    double k_p;
    double k_i;
    double k_d;
    double i_smooth;
} restart_parameters_t;

/* LP/CP_AL/include/cp_al_types.h:79-86 */
typedef struct {
    double eps_optimal_relative;
    double eps_feasible_relative;
    double eps_feas_polish_relative;
    double time_sec_limit;
    int iteration_limit;
} termination_criteria_t;

/* LP/CP_AL/include/cp_al_types.h:88-105 */
typedef struct {
    int l_inf_ruiz_iterations;
    bool has_pock_chambolle_alpha;
    double pock_chambolle_alpha;
    bool bound_objective_rescaling;
    bool verbose;
    int termination_evaluation_frequency;
    int sv_max_iter;
    double sv_tol;
    termination_criteria_t termination_criteria;
    restart_parameters_t restart_params;
    double reflection_coefficient;
    bool feasibility_polishing;
    norm_type_t optimality_norm;
    bool presolve;
    double matrix_zero_tol;
} cp_al_parameters_t;

/* LP/CP_AL/include/cp_al_types.h:107-143 */
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
    double rescaling_time_sec;
    double cumulative_time_sec;
    double presolve_time;
    int presolve_status;

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
    termination_reason_t termination_reason;
    double feasibility_polishing_time;
    int feasibility_iteration;
} cp_al_result_t;

/* LP/CP_AL/include/cp_al_types.h:145-189 */
typedef enum { matrix_dense = 0, matrix_csr = 1, matrix_csc = 2, matrix_coo = 3 } matrix_format_t;

typedef struct {
    int m;
    int n;
    matrix_format_t fmt;

    union MatrixData {
        struct MatrixDense {
            const double *A; /* row-major m*n */
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
