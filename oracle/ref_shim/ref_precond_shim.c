/*
 * Helpers for the reference's FA_CP equilibration (QP/FA_CP/src/preconditioner.c)
 * built alone for the parity tests: the CSR deep copy its problem copy calls,
 * and ref_facp_rescale, which runs rescale_problem and hands back the scale
 * vectors and the bound/objective factors.  Compiled by oracle/build.py
 * (build_ref) with ref_mps_shim.c for the allocation helpers.  Test
 * infrastructure only.
 */
#include <stdlib.h>
#include <string.h>

#include "internal_types.h"

void *safe_malloc(size_t size);
rescale_info_t *rescale_problem(const fa_cp_parameters_t *params, const qp_problem_t *working_problem);

CsrComponent *deepcopy_csr_component(const CsrComponent *src, size_t num_rows, size_t nnz) {
    CsrComponent *c = (CsrComponent *)safe_malloc(sizeof(CsrComponent));
    c->row_ptr = (int *)safe_malloc((num_rows + 1) * sizeof(int));
    c->col_ind = (int *)safe_malloc((nnz ? nnz : 1) * sizeof(int));
    c->val = (double *)safe_malloc((nnz ? nnz : 1) * sizeof(double));
    if (src && src->row_ptr) memcpy(c->row_ptr, src->row_ptr, (num_rows + 1) * sizeof(int));
    else memset(c->row_ptr, 0, (num_rows + 1) * sizeof(int));
    if (nnz) {
        memcpy(c->col_ind, src->col_ind, nnz * sizeof(int));
        memcpy(c->val, src->val, nnz * sizeof(double));
    }
    return c;
}

static void free_component(CsrComponent *c) {
    if (!c) return;
    free(c->row_ptr);
    free(c->col_ind);
    free(c->val);
    free(c);
}

int ref_facp_rescale(const qp_problem_t *prob, const fa_cp_parameters_t *params, double *var_rescale,
                     double *con_rescale, double *bound_obj) {
    rescale_info_t *ri = rescale_problem(params, prob);
    if (!ri) return -1;
    memcpy(var_rescale, ri->var_rescale, (size_t)prob->num_variables * sizeof(double));
    memcpy(con_rescale, ri->con_rescale, (size_t)prob->num_constraints * sizeof(double));
    bound_obj[0] = ri->con_bound_rescale;
    bound_obj[1] = ri->obj_vec_rescale;
    qp_problem_t *s = ri->scaled_problem;
    free_component(s->constraint_matrix);
    free_component(s->objective_sparse_matrix);
    free_component(s->objective_lowrank_matrix);
    free(s->variable_lower_bound);
    free(s->variable_upper_bound);
    free(s->objective_vector);
    free(s->constraint_lower_bound);
    free(s->constraint_upper_bound);
    free(s->primal_start);
    free(s->dual_start);
    free(s);
    free(ri->con_rescale);
    free(ri->var_rescale);
    free(ri);
    return 0;
}
