/*
 * The few helpers the reference MPS readers (LP/CP_AL/src/mps_parser.c,
 * QP/FA_CP/src/mps_parser.c) call from the rest of their libraries, so that
 * each reader builds alone as a shared object for the parity tests:
 * safe_malloc / safe_calloc / safe_realloc (abort on failure, as the
 * reference's do) and the problem free function of its library.  Compiled
 * once with -DREF_LP and once with -DREF_QP by oracle/build.py (build_ref).
 * Test infrastructure only.
 */
#include <stdio.h>
#include <stdlib.h>

void *safe_malloc(size_t size) {
    void *p = malloc(size ? size : 1);
    if (!p) abort();
    return p;
}

void *safe_calloc(size_t num, size_t size) {
    void *p = calloc(num ? num : 1, size ? size : 1);
    if (!p) abort();
    return p;
}

void *safe_realloc(void *ptr, size_t size) {
    void *p = realloc(ptr, size ? size : 1);
    if (!p) abort();
    return p;
}

#ifdef REF_LP
#include "cp_al_types.h"
void lp_problem_free(lp_problem_t *p) {
    if (!p) return;
    free(p->constraint_matrix_row_pointers);
    free(p->constraint_matrix_col_indices);
    free(p->constraint_matrix_values);
    free(p->variable_lower_bound);
    free(p->variable_upper_bound);
    free(p->objective_vector);
    free(p->constraint_lower_bound);
    free(p->constraint_upper_bound);
    free(p->primal_start);
    free(p->dual_start);
    free(p);
}
#endif

#ifdef REF_QP
#include "fa_cp_types.h"
static void free_component(CsrComponent *c) {
    if (!c) return;
    free(c->row_ptr);
    free(c->col_ind);
    free(c->val);
    free(c);
}
void qp_problem_free(qp_problem_t *p) {
    if (!p) return;
    free_component(p->constraint_matrix);
    free_component(p->objective_sparse_matrix);
    free_component(p->objective_lowrank_matrix);
    free(p->variable_lower_bound);
    free(p->variable_upper_bound);
    free(p->objective_vector);
    free(p->constraint_lower_bound);
    free(p->constraint_upper_bound);
    free(p->primal_start);
    free(p->dual_start);
    free(p);
}
#endif
