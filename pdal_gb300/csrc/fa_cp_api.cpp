/*
 * fa_cp_api.cpp -- host-only part of the FA_CP C interface: problem
 * construction from dense/CSR/CSC/COO descriptions of A, Q and R, warm
 * starts, defaults and the free functions.
 *
 * Interface: QP/FA_CP/include/fa_cp.h:28-50; behaviour of
 * QP/FA_CP/src/fa_cp.c:28-376 and the converters of
 * QP/FA_CP/src/utils.cu:1145-1332: dense input drops |a| <= tol with tol =
 * zero_tolerance if positive, else 1e-12; CSC and COO drop |a| <= tol only for
 * a positive zero_tolerance, and COO rows keep their input order; CSR is
 * copied as given.  Every matrix of the problem is present afterwards (an
 * absent one is empty with all-zero row pointers), which also gives the
 * solver well-defined row pointers where the reference keeps a one-element
 * array.
 */
#include "../../include/fa_cp.h"
#include "../../include/fa_cp_gb300.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace {

double *fill_or_copy(int n, const double *src, double fill) {
    double *d = (double *)malloc(sizeof(double) * (n > 0 ? (size_t)n : 1));
    if (!d) return nullptr;
    if (src)
        memcpy(d, src, sizeof(double) * (size_t)n);
    else
        for (int i = 0; i < n; ++i) d[i] = fill;
    return d;
}

CsrComponent *empty_component(int rows) {
    CsrComponent *c = (CsrComponent *)calloc(1, sizeof(CsrComponent));
    if (!c) return nullptr;
    c->row_ptr = (int *)calloc((size_t)rows + 1, sizeof(int));
    c->col_ind = (int *)malloc(sizeof(int));
    c->val = (double *)malloc(sizeof(double));
    return c;
}

void free_component(CsrComponent *c) {
    if (!c) return;
    free(c->row_ptr);
    free(c->col_ind);
    free(c->val);
    free(c);
}

/* Converts one matrix description; returns the component and its nonzero
 * count, or nullptr with a message. */
CsrComponent *convert(const matrix_desc_t *d, const char *what, int *nnz_out) {
    const int m = d->m, n = d->n;
    if (m < 0 || n < 0) {
        fprintf(stderr, "[interface] %s matrix: negative dimensions.\n", what);
        return nullptr;
    }
    CsrComponent *c = (CsrComponent *)calloc(1, sizeof(CsrComponent));
    if (!c) return nullptr;
    c->row_ptr = (int *)calloc((size_t)m + 1, sizeof(int));
    int nnz = 0;
    bool ok = c->row_ptr != nullptr;
    switch (d->fmt) {
    case matrix_dense: {
        const double tol = d->zero_tolerance > 0 ? d->zero_tolerance : 1e-12;
        const double *A = d->data.dense.A;
        long long cnt = 0;
        for (long long i = 0; ok && i < (long long)m * n; ++i)
            if (std::fabs(A[i]) > tol) ++cnt;
        if (cnt > 2147483647LL) ok = false;
        if (!ok) break;
        c->col_ind = (int *)malloc(sizeof(int) * (cnt > 0 ? cnt : 1));
        c->val = (double *)malloc(sizeof(double) * (cnt > 0 ? cnt : 1));
        if (!c->col_ind || !c->val) {
            ok = false;
            break;
        }
        for (int i = 0; i < m; ++i) {
            c->row_ptr[i] = nnz;
            for (int j = 0; j < n; ++j) {
                const double v = A[(size_t)i * n + j];
                if (std::fabs(v) > tol) {
                    c->col_ind[nnz] = j;
                    c->val[nnz] = v;
                    ++nnz;
                }
            }
        }
        c->row_ptr[m] = nnz;
        break;
    }
    case matrix_csr: {
        nnz = d->data.csr.nnz;
        if (nnz < 0 || (m > 0 && !d->data.csr.row_ptr) || (nnz > 0 && (!d->data.csr.col_ind || !d->data.csr.vals))) {
            ok = false;
            break;
        }
        c->col_ind = (int *)malloc(sizeof(int) * (nnz > 0 ? (size_t)nnz : 1));
        c->val = (double *)malloc(sizeof(double) * (nnz > 0 ? (size_t)nnz : 1));
        if (!c->col_ind || !c->val) {
            ok = false;
            break;
        }
        if (d->data.csr.row_ptr) memcpy(c->row_ptr, d->data.csr.row_ptr, sizeof(int) * ((size_t)m + 1));
        if (nnz > 0) {
            memcpy(c->col_ind, d->data.csr.col_ind, sizeof(int) * (size_t)nnz);
            memcpy(c->val, d->data.csr.vals, sizeof(double) * (size_t)nnz);
        }
        break;
    }
    case matrix_csc:
    case matrix_coo: {
        const bool csc = d->fmt == matrix_csc;
        const double tol = d->zero_tolerance > 0 ? d->zero_tolerance : 0.0;
        const int nin = csc ? d->data.csc.nnz : d->data.coo.nnz;
        const double *v = csc ? d->data.csc.vals : d->data.coo.vals;
        if (nin < 0 || (nin > 0 && !v)) {
            ok = false;
            break;
        }
        /* (row, col) of input entry k */
        const int *cp = d->data.csc.col_ptr, *ri = d->data.csc.row_ind;
        const int *r = d->data.coo.row_ind, *cc = d->data.coo.col_ind;
        int *rows = (int *)malloc(sizeof(int) * (nin > 0 ? (size_t)nin : 1));
        int *cols = (int *)malloc(sizeof(int) * (nin > 0 ? (size_t)nin : 1));
        if (!rows || !cols) {
            free(rows);
            free(cols);
            ok = false;
            break;
        }
        if (csc) {
            for (int j = 0; j < n && ok; ++j)
                for (int k = cp[j]; k < cp[j + 1]; ++k) {
                    if (k < 0 || k >= nin) {
                        ok = false;
                        break;
                    }
                    rows[k] = ri[k];
                    cols[k] = j;
                }
        } else {
            for (int k = 0; k < nin; ++k) {
                rows[k] = r[k];
                cols[k] = cc[k];
            }
        }
        for (int k = 0; ok && k < nin; ++k) {
            if (tol > 0 && std::fabs(v[k]) <= tol) continue;
            if (rows[k] < 0 || rows[k] >= m || cols[k] < 0 || cols[k] >= n) {
                fprintf(stderr, "[interface] %s matrix: index out of range\n", what);
                ok = false;
                break;
            }
            c->row_ptr[rows[k] + 1]++;
            ++nnz;
        }
        if (ok) {
            for (int i = 0; i < m; ++i) c->row_ptr[i + 1] += c->row_ptr[i];
            c->col_ind = (int *)malloc(sizeof(int) * (nnz > 0 ? (size_t)nnz : 1));
            c->val = (double *)malloc(sizeof(double) * (nnz > 0 ? (size_t)nnz : 1));
            int *next = (int *)malloc(sizeof(int) * (m > 0 ? (size_t)m : 1));
            if (!c->col_ind || !c->val || !next) {
                ok = false;
            } else {
                for (int i = 0; i < m; ++i) next[i] = c->row_ptr[i];
                /* CSC visits columns in order, so its rows come out sorted;
                 * COO keeps the input order inside each row */
                for (int k = 0; k < nin; ++k) {
                    if (tol > 0 && std::fabs(v[k]) <= tol) continue;
                    const int pos = next[rows[k]]++;
                    c->col_ind[pos] = cols[k];
                    c->val[pos] = v[k];
                }
            }
            free(next);
        }
        free(rows);
        free(cols);
        break;
    }
    default:
        fprintf(stderr, "[interface] %s matrix: unsupported format %d.\n", what, (int)d->fmt);
        ok = false;
    }
    if (!ok) {
        free_component(c);
        return nullptr;
    }
    if (!c->col_ind) c->col_ind = (int *)malloc(sizeof(int));
    if (!c->val) c->val = (double *)malloc(sizeof(double));
    *nnz_out = nnz;
    return c;
}

} // namespace

extern "C" {

qp_problem_t *create_qp_problem(const double *objective_c, const matrix_desc_t *Q_desc,
                                const matrix_desc_t *R_desc, const matrix_desc_t *A_desc,
                                const double *con_lb, const double *con_ub, const double *var_lb,
                                const double *var_ub, const double *objective_constant) {
    int n = 0, m = 0;
    if (A_desc) {
        n = A_desc->n;
        m = A_desc->m;
    } else if (Q_desc) {
        n = Q_desc->n;
    } else if (R_desc) {
        n = R_desc->n;
    } else {
        fprintf(stderr, "[interface] Error: At least one matrix (A, Q, or R) must be provided.\n");
        return nullptr;
    }
    if (n < 0 || m < 0) {
        fprintf(stderr, "[interface] create_qp_problem: negative dimensions.\n");
        return nullptr;
    }
    if ((Q_desc && (Q_desc->m != n || Q_desc->n != n)) || (R_desc && R_desc->n != n)) {
        fprintf(stderr, "[interface] create_qp_problem: Q must be n x n and R must have n columns.\n");
        return nullptr;
    }
    qp_problem_t *p = (qp_problem_t *)calloc(1, sizeof(qp_problem_t));
    if (!p) return nullptr;
    p->num_variables = n;
    p->num_constraints = m;
    p->num_rank_lowrank_obj = R_desc ? R_desc->m : 0;
    int nnz = 0;
    p->constraint_matrix = A_desc ? convert(A_desc, "A", &nnz) : empty_component(m);
    p->constraint_matrix_num_nonzeros = A_desc ? nnz : 0;
    nnz = 0;
    p->objective_sparse_matrix = Q_desc ? convert(Q_desc, "Q", &nnz) : empty_component(n);
    p->objective_sparse_matrix_num_nonzeros = Q_desc ? nnz : 0;
    nnz = 0;
    p->objective_lowrank_matrix = R_desc ? convert(R_desc, "R", &nnz) : empty_component(0);
    p->objective_lowrank_matrix_num_nonzeros = R_desc ? nnz : 0;
    p->objective_constant = objective_constant ? *objective_constant : 0.0;
    p->objective_vector = fill_or_copy(n, objective_c, 0.0);
    p->variable_lower_bound = fill_or_copy(n, var_lb, -INFINITY);
    p->variable_upper_bound = fill_or_copy(n, var_ub, INFINITY);
    p->constraint_lower_bound = fill_or_copy(m, con_lb, -INFINITY);
    p->constraint_upper_bound = fill_or_copy(m, con_ub, INFINITY);
    if (!p->constraint_matrix || !p->objective_sparse_matrix || !p->objective_lowrank_matrix || !p->objective_vector ||
        !p->variable_lower_bound || !p->variable_upper_bound || !p->constraint_lower_bound ||
        !p->constraint_upper_bound) {
        qp_problem_free(p);
        return nullptr;
    }
    return p;
}

void set_start_values(qp_problem_t *prob, const double *primal, const double *dual) {
    if (!prob) return;
    free(prob->primal_start);
    free(prob->dual_start);
    prob->primal_start = nullptr;
    prob->dual_start = nullptr;
    if (primal) {
        prob->primal_start = (double *)malloc(sizeof(double) * (prob->num_variables > 0 ? prob->num_variables : 1));
        if (prob->primal_start) memcpy(prob->primal_start, primal, sizeof(double) * (size_t)prob->num_variables);
    }
    if (dual) {
        prob->dual_start = (double *)malloc(sizeof(double) * (prob->num_constraints > 0 ? prob->num_constraints : 1));
        if (prob->dual_start) memcpy(prob->dual_start, dual, sizeof(double) * (size_t)prob->num_constraints);
    }
}

void set_default_parameters(fa_cp_parameters_t *p) { /* QP/FA_CP/src/utils.cu:494-537 */
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->l_inf_ruiz_iterations = 10;
    p->has_pock_chambolle_alpha = true;
    p->pock_chambolle_alpha = 1.0;
    p->bound_objective_rescaling = true;
    p->trajectory_csv = nullptr;
    p->use_al_qp = true;
    p->al_sigma = 0.0;
    p->sigma_update_rule = FA_CP_SIGMA_UPDATE_GUARDED;
    p->sigma_update_gain = 0.5;
    p->sigma_clip_low = 0.6;
    p->sigma_clip_high = 1.7;
    p->sigma_min = 1e-8;
    p->sigma_max = 10.0;
    p->sigma_rollback_tol = 1.25;
    p->sigma_zero_threshold = 1e-8;
    p->sigma_activation_threshold = 2.0;
    p->sigma_normal_motion_threshold = 1e-10;
    p->sigma_activation_value = 0.1;
    p->verbose = 1;
    p->termination_evaluation_frequency = 200;
    p->feasibility_polishing = false;
    p->reflection_coefficient = 1.0;
    p->sv_max_iter = 5000;
    p->sv_tol = 1e-4;
    p->termination_criteria.eps_optimal_relative = 1e-4;
    p->termination_criteria.eps_feasible_relative = 1e-4;
    p->termination_criteria.eps_infeasible = 1e-10;
    p->termination_criteria.time_sec_limit = 3600.0;
    p->termination_criteria.iteration_limit = 2147483647;
    p->termination_criteria.eps_feas_polish_relative = 1e-6;
    p->restart_params.artificial_restart_threshold = 0.36;
    p->restart_params.sufficient_reduction_for_restart = 0.2;
    p->restart_params.necessary_reduction_for_restart = 0.8;
    p->restart_params.k_p = 0.99;
    p->restart_params.k_i = 0.01;
    p->restart_params.k_d = 0.0;
    p->restart_params.i_smooth = 0.3;
    p->optimality_norm = NORM_TYPE_L_INF;
}

void fa_cp_result_free(fa_cp_result_t *r) {
    if (!r) return;
    free(r->primal_solution);
    free(r->dual_solution);
    free(r->reduced_cost);
    free(r);
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

void fa_cp_gb300_default_options(fa_cp_gb300_options_t *o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->device = -1;
    o->blocks_per_sm = 0;
    o->restart_select = 0;
    o->restart_select_margin = 1.0;
    o->restart_select_min_iters = 0;
    o->restart_select_min_time = 0.0;
    o->precision = 0;
    o->fp32_switch_tol = 1e-5;
    o->fp32_stall_evals = 25;
}

static const char *env_value(const char *primary, const char *fallback) {
    const char *v = getenv(primary);
    if ((!v || !v[0]) && fallback) v = getenv(fallback);
    return v;
}

void fa_cp_gb300_options_from_env(fa_cp_gb300_options_t *o) { /* fa_cp_core_op.cu:35-66, 908-916, 1130-1169 */
    fa_cp_gb300_default_options(o);
    if (!o) return;
    const char *v = env_value("FA_CP_RESTART_SELECT", "FA_CP_RESTART_SELECT_LEGACY");
    if (v && v[0]) o->restart_select = atoi(v);
    v = env_value("FA_CP_RESTART_SELECT_MIN_ITERS", nullptr);
    if (v && v[0]) o->restart_select_min_iters = atoi(v);
    for (int k = 0; k < 2; ++k) {
        const char *name = k == 0 ? "FA_CP_RESTART_SELECT_MIN_TIME" : "FA_CP_RESTART_SELECT_MARGIN";
        v = env_value(name, nullptr);
        if (!v || !v[0]) continue;
        char *end = nullptr;
        const double d = strtod(v, &end);
        if (end == v || !std::isfinite(d)) continue;
        if (k == 0)
            o->restart_select_min_time = d;
        else
            o->restart_select_margin = d;
    }
    v = env_value("FA_CP_GB300_PRECISION", nullptr);
    if (v && strcmp(v, "fp32_refine") == 0) o->precision = 1;
}

} // extern "C"

/* ---------------------------------------------------------------------- */
/* read_mps_file: QP/FA_CP/include/mps_parser.h:23                         */
/* ---------------------------------------------------------------------- */
#include "../../include/fa_cp_mps_parser.h"
#include "mps_reader.h"

#include <string>
#include <vector>

namespace pdal {
void facp_set_last_error(const std::string &msg);
} // namespace pdal

namespace {

template <class T>
bool copy_out(const std::vector<T> &v, T **dst) {
    *dst = nullptr;
    if (v.empty()) return true;
    *dst = (T *)malloc(v.size() * sizeof(T));
    if (!*dst) return false;
    memcpy(*dst, v.data(), v.size() * sizeof(T));
    return true;
}

/* A component with the reader's rows + 1 row pointers; empty column and
 * value arrays get one element so that no pointer of the problem is NULL. */
CsrComponent *component(const pdal::mps::Csr &A) {
    CsrComponent *c = (CsrComponent *)calloc(1, sizeof(CsrComponent));
    if (!c) return nullptr;
    const bool ok = copy_out(A.row_ptr, &c->row_ptr) && copy_out(A.col_ind, &c->col_ind) &&
                    copy_out(A.val, &c->val);
    if (ok && !c->col_ind) c->col_ind = (int *)calloc(1, sizeof(int));
    if (ok && !c->val) c->val = (double *)calloc(1, sizeof(double));
    if (!ok || !c->row_ptr || !c->col_ind || !c->val) {
        free_component(c);
        return nullptr;
    }
    return c;
}

} // namespace

extern "C" qp_problem_t *read_mps_file(const char *filename) {
    pdal::facp_set_last_error("");
    pdal::mps::Model M;
    std::string err;
    if (!pdal::mps::read_file(filename, true, M, err)) {
        fprintf(stderr, "[fa_cp_gb300] read_mps_file: %s\n", err.c_str());
        pdal::facp_set_last_error("read_mps_file: " + err);
        return nullptr;
    }
    qp_problem_t *p = (qp_problem_t *)calloc(1, sizeof(qp_problem_t));
    if (!p) {
        pdal::facp_set_last_error("read_mps_file: out of host memory");
        return nullptr;
    }
    p->num_variables = M.num_cols;
    p->num_constraints = M.num_rows;
    p->num_rank_lowrank_obj = 0;
    p->objective_constant = M.objective_constant;
    p->constraint_matrix_num_nonzeros = (int)M.A.val.size();
    p->objective_sparse_matrix_num_nonzeros = (int)M.Q.val.size();
    p->objective_lowrank_matrix_num_nonzeros = 0;
    pdal::mps::Csr lowrank;
    lowrank.row_ptr.assign(1, 0);
    p->constraint_matrix = component(M.A);
    p->objective_sparse_matrix = component(M.Q);
    p->objective_lowrank_matrix = component(lowrank);
    const bool ok = p->constraint_matrix && p->objective_sparse_matrix && p->objective_lowrank_matrix &&
                    copy_out(M.c, &p->objective_vector) && copy_out(M.var_lb, &p->variable_lower_bound) &&
                    copy_out(M.var_ub, &p->variable_upper_bound) &&
                    copy_out(M.con_lb, &p->constraint_lower_bound) &&
                    copy_out(M.con_ub, &p->constraint_upper_bound);
    if (!ok) {
        qp_problem_free(p);
        pdal::facp_set_last_error("read_mps_file: out of host memory");
        return nullptr;
    }
    return p;
}
