/*
 * fa_cp.h -- the FA_CP (convex QP) C entry points, exported by
 * libfa_cp_gb300.so.  Each replaces the reference function of the same name
 * (QP/FA_CP/include/fa_cp.h:28-50, implemented in QP/FA_CP/src/fa_cp.c).
 * Errors return NULL with one line on stderr (the reference exits).
 */
#pragma once

#include "fa_cp_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* QP/FA_CP/src/fa_cp.c:28-289: A, Q (sparse part) and R (low-rank factor,
 * Q += R'R) are each optional; n comes from A, then Q, then R. */
qp_problem_t *create_qp_problem(const double *objective_c, const matrix_desc_t *Q_desc,
                                const matrix_desc_t *R_desc, const matrix_desc_t *A_desc,
                                const double *con_lb, const double *con_ub, const double *var_lb,
                                const double *var_ub, const double *objective_constant);

/* QP/FA_CP/src/fa_cp.c:324-350 */
void set_start_values(qp_problem_t *prob, const double *primal, const double *dual);

/* QP/FA_CP/src/fa_cp.c:352-376; params == NULL selects the defaults. */
fa_cp_result_t *solve_qp_problem(const qp_problem_t *prob, const fa_cp_parameters_t *params);

/* QP/FA_CP/src/utils.cu:494-537 */
void set_default_parameters(fa_cp_parameters_t *params);

/* QP/FA_CP/src/fa_cp.c:290-298 (also frees reduced_cost) */
void fa_cp_result_free(fa_cp_result_t *results);

/* QP/FA_CP/src/fa_cp.c:300-322 */
void qp_problem_free(qp_problem_t *prob);

#ifdef __cplusplus
} /* extern "C" */
#endif
