/*
 * cp_al.h -- the CP_AL (LP) C entry points, exported by libcp_al_gb300.so.
 *
 * Each declaration replaces the reference function of the same name
 * (LP/CP_AL/include/cp_al.h:28-47, implemented in LP/CP_AL/src/cp_al.c).
 * Behavioural differences at this boundary:
 *   - errors never exit(): a bad argument, an invalid evaluation frequency or a
 *     CUDA failure returns NULL (create/solve) and prints one line to stderr;
 *   - cp_al_result_free also frees reduced_cost (the reference leaks it);
 *   - solve_lp_problem runs on the current CUDA device; there is no CPU path.
 */
#pragma once

#include "cp_al_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* LP/CP_AL/include/cp_al.h:29-35, LP/CP_AL/src/cp_al.c:26-116.
 * Deep-copies A (dense, CSR, CSC or COO; converted to CSR) and the vectors.
 * NULL vectors take the reference defaults: c = 0, var bounds = -inf/+inf,
 * constraint bounds = -inf/+inf, objective constant = 0. */
lp_problem_t *create_lp_problem(const double *objective_c, const matrix_desc_t *A_desc, const double *con_lb,
                                const double *con_ub, const double *var_lb, const double *var_ub,
                                const double *objective_constant);

/* LP/CP_AL/include/cp_al.h:38, LP/CP_AL/src/cp_al.c:148-178. Copies the warm
 * start (either pointer may be NULL, which clears that half). */
void set_start_values(lp_problem_t *prob, const double *primal, const double *dual);

/* LP/CP_AL/include/cp_al.h:41, LP/CP_AL/src/cp_al.c:180-209. params == NULL
 * selects set_default_parameters(). Returns a malloc'd result or NULL. */
cp_al_result_t *solve_lp_problem(lp_problem_t *prob, const cp_al_parameters_t *params);

/* LP/CP_AL/include/cp_al.h:44, defaults of LP/CP_AL/src/utils.cu:361-394. */
void set_default_parameters(cp_al_parameters_t *params);

/* LP/CP_AL/include/cp_al.h:46, LP/CP_AL/src/cp_al.c:118-128. */
void cp_al_result_free(cp_al_result_t *results);

/* LP/CP_AL/include/cp_al.h:48, LP/CP_AL/src/cp_al.c:130-146. */
void lp_problem_free(lp_problem_t *prob);

#ifdef __cplusplus
} /* extern "C" */
#endif
