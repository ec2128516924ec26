/*
 * cp_al_api.cpp -- host-only part of the CP_AL C interface: problem
 * construction from dense/CSR/CSC/COO, warm starts, defaults, the
 * environment plane and the free functions.
 *
 * Interface: LP/CP_AL/include/cp_al.h:28-47; behaviour of
 * LP/CP_AL/src/cp_al.c:26-209 and the converters of
 * LP/CP_AL/src/utils.cu:1042-1192 (dense drops exact zeros; CSC and COO keep
 * the given entries, rows filled in input order).
 */
#include "../../include/cp_al.h"
#include "../../include/cp_al_gb300.h"
#include "common.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace {

/* memcpy of a large array by the host threads (the destination's pages are
 * first touched in parallel too): the deep copies of a 20M-nonzero problem
 * are ~300 MB */
void copy_bytes(void *dst, const void *src, size_t bytes) {
    const int nt = bytes >= (8u << 20) ? pdal::host_threads((long long)(bytes >> 4)) : 1;
    if (nt <= 1) {
        memcpy(dst, src, bytes);
        return;
    }
    pdal::parallel_for(nt, [&](int t) {
        const size_t b0 = bytes * t / nt & ~size_t(63), b1 = t + 1 == nt ? bytes : bytes * (t + 1) / nt & ~size_t(63);
        memcpy(static_cast<char *>(dst) + b0, static_cast<const char *>(src) + b0, b1 - b0);
    });
}

double *fill_or_copy(int n, const double *src, double fill) {
    double *d = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    if (!d) return nullptr;
    if (src)
        copy_bytes(d, src, sizeof(double) * (size_t)n);
    else
        for (int i = 0; i < n; ++i) d[i] = fill;
    return d;
}

/* rows of the result are filled in input order, like counting sort */
int to_csr_from_pairs(int m, int n, int nnz, const int *r, const int *c, const double *v, lp_problem_t *p,
                      const char *what) {
    int *rp = (int *)calloc((size_t)m + 1, sizeof(int));
    int *ci = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    double *vv = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    int *next = (int *)malloc(sizeof(int) * (m > 0 ? m : 1));
    if (!rp || !ci || !vv || !next) {
        free(rp);
        free(ci);
        free(vv);
        free(next);
        return -1;
    }
    for (int k = 0; k < nnz; ++k) {
        if (r[k] < 0 || r[k] >= m || c[k] < 0 || c[k] >= n) {
            fprintf(stderr, "[interface] %s: index out of range\n", what);
            free(rp);
            free(ci);
            free(vv);
            free(next);
            return -1;
        }
        rp[r[k] + 1]++;
    }
    for (int i = 0; i < m; ++i) rp[i + 1] += rp[i];
    for (int i = 0; i < m; ++i) next[i] = rp[i];
    for (int k = 0; k < nnz; ++k) {
        const int pos = next[r[k]]++;
        ci[pos] = c[k];
        vv[pos] = v[k];
    }
    free(next);
    p->constraint_matrix_row_pointers = rp;
    p->constraint_matrix_col_indices = ci;
    p->constraint_matrix_values = vv;
    p->constraint_matrix_num_nonzeros = nnz;
    return 0;
}

double env_double(const char *name, double def) {
    const char *raw = getenv(name);
    if (!raw || !raw[0]) return def;
    char *end = nullptr;
    const double v = strtod(raw, &end);
    if (end == raw || !std::isfinite(v)) return def;
    return v;
}

int env_int(const char *name, int def) {
    const char *raw = getenv(name);
    if (!raw || !raw[0]) return def;
    char *end = nullptr;
    const long v = strtol(raw, &end, 10);
    if (end == raw) return def;
    return (int)v;
}

bool env_set(const char *name) {
    const char *raw = getenv(name);
    return raw && raw[0] != '\0';
}

bool env_parses(const char *name) {
    const char *raw = getenv(name);
    if (!raw || !raw[0]) return false;
    char *end = nullptr;
    const double v = strtod(raw, &end);
    return end != raw && std::isfinite(v);
}

} // namespace

extern "C" {

lp_problem_t *create_lp_problem(const double *objective_c, const matrix_desc_t *A_desc, const double *con_lb,
                                const double *con_ub, const double *var_lb, const double *var_ub,
                                const double *objective_constant) {
    if (!A_desc || A_desc->m < 0 || A_desc->n < 0) {
        fprintf(stderr, "[interface] create_lp_problem: invalid matrix descriptor.\n");
        return nullptr;
    }
    lp_problem_t *p = (lp_problem_t *)calloc(1, sizeof(lp_problem_t));
    if (!p) return nullptr;
    const int m = A_desc->m, n = A_desc->n;
    p->num_variables = n;
    p->num_constraints = m;
    int rc = 0;
    switch (A_desc->fmt) {
    case matrix_dense: {
        const double *A = A_desc->data.dense.A;
        long long nnz = 0;
        for (long long i = 0; i < (long long)m * n; ++i)
            if (std::fabs(A[i]) > 0.0) ++nnz;
        if (nnz > 2147483647LL) {
            rc = -1;
            break;
        }
        int *rp = (int *)malloc(sizeof(int) * ((size_t)m + 1));
        int *ci = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
        double *vv = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
        if (!rp || !ci || !vv) {
            free(rp);
            free(ci);
            free(vv);
            rc = -1;
            break;
        }
        int nz = 0;
        for (int i = 0; i < m; ++i) {
            rp[i] = nz;
            for (int j = 0; j < n; ++j) {
                const double v = A[(size_t)i * n + j];
                if (std::fabs(v) > 0.0) {
                    ci[nz] = j;
                    vv[nz] = v;
                    ++nz;
                }
            }
        }
        rp[m] = nz;
        p->constraint_matrix_row_pointers = rp;
        p->constraint_matrix_col_indices = ci;
        p->constraint_matrix_values = vv;
        p->constraint_matrix_num_nonzeros = nz;
        break;
    }
    case matrix_csr: {
        const int nnz = A_desc->data.csr.nnz;
        if (nnz < 0 || (m > 0 && !A_desc->data.csr.row_ptr)) {
            rc = -1;
            break;
        }
        int *rp = (int *)malloc(sizeof(int) * ((size_t)m + 1));
        int *ci = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
        double *vv = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
        if (!rp || !ci || !vv) {
            free(rp);
            free(ci);
            free(vv);
            rc = -1;
            break;
        }
        if (A_desc->data.csr.row_ptr)
            copy_bytes(rp, A_desc->data.csr.row_ptr, sizeof(int) * ((size_t)m + 1));
        else
            rp[0] = 0;
        if (nnz) {
            copy_bytes(ci, A_desc->data.csr.col_ind, sizeof(int) * (size_t)nnz);
            copy_bytes(vv, A_desc->data.csr.vals, sizeof(double) * (size_t)nnz);
        }
        p->constraint_matrix_row_pointers = rp;
        p->constraint_matrix_col_indices = ci;
        p->constraint_matrix_values = vv;
        p->constraint_matrix_num_nonzeros = nnz;
        break;
    }
    case matrix_csc: {
        const int nnz = A_desc->data.csc.nnz;
        const int *cp = A_desc->data.csc.col_ptr;
        if (nnz < 0 || (n > 0 && !cp)) {
            rc = -1;
            break;
        }
        /* expand column pointers to column indices, then place by row */
        int *cols = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
        if (!cols) {
            rc = -1;
            break;
        }
        for (int j = 0; j < n; ++j)
            for (int k = cp[j]; k < cp[j + 1]; ++k)
                if (k >= 0 && k < nnz) cols[k] = j;
        rc = to_csr_from_pairs(m, n, nnz, A_desc->data.csc.row_ind, cols, A_desc->data.csc.vals, p, "CSC");
        free(cols);
        if (rc) fprintf(stderr, "[interface] CSC->CSR failed.\n");
        break;
    }
    case matrix_coo: {
        const int nnz = A_desc->data.coo.nnz;
        rc = to_csr_from_pairs(m, n, nnz, A_desc->data.coo.row_ind, A_desc->data.coo.col_ind, A_desc->data.coo.vals,
                               p, "COO");
        if (rc) fprintf(stderr, "[interface] COO->CSR failed.\n");
        break;
    }
    default:
        fprintf(stderr, "[interface] make_problem_from_matrix: unsupported matrix format %d.\n", (int)A_desc->fmt);
        rc = -1;
    }
    if (rc) {
        free(p);
        return nullptr;
    }
    p->objective_constant = objective_constant ? *objective_constant : 0.0;
    p->objective_vector = fill_or_copy(n, objective_c, 0.0);
    p->variable_lower_bound = fill_or_copy(n, var_lb, -INFINITY);
    p->variable_upper_bound = fill_or_copy(n, var_ub, INFINITY);
    p->constraint_lower_bound = fill_or_copy(m, con_lb, -INFINITY);
    p->constraint_upper_bound = fill_or_copy(m, con_ub, INFINITY);
    if (!p->objective_vector || !p->variable_lower_bound || !p->variable_upper_bound || !p->constraint_lower_bound ||
        !p->constraint_upper_bound) {
        lp_problem_free(p);
        return nullptr;
    }
    return p;
}

void set_start_values(lp_problem_t *prob, const double *primal, const double *dual) {
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

/* LP/CP_AL/src/utils.cu:361-394 */
void set_default_parameters(cp_al_parameters_t *params) {
    if (!params) return;
    memset(params, 0, sizeof(*params));
    params->l_inf_ruiz_iterations = 10;
    params->has_pock_chambolle_alpha = true;
    params->pock_chambolle_alpha = 1.0;
    params->bound_objective_rescaling = true;
    params->verbose = false;
    params->termination_evaluation_frequency = 200;
    params->feasibility_polishing = false;
    params->reflection_coefficient = env_double("CP_AL_REFLECTION_COEFFICIENT", 1.0);
    params->reflection_coefficient = std::fmax(0.0, std::fmin(params->reflection_coefficient, 2.0));
    params->sv_max_iter = 5000;
    params->sv_tol = 1e-4;
    params->termination_criteria.eps_optimal_relative = 1e-4;
    params->termination_criteria.eps_feasible_relative = 1e-4;
    params->termination_criteria.time_sec_limit = 3600.0;
    params->termination_criteria.iteration_limit = 2147483647;
    params->termination_criteria.eps_feas_polish_relative = 1e-6;
    params->restart_params.artificial_restart_threshold = 0.36;
    params->restart_params.sufficient_reduction_for_restart = 0.2;
    params->restart_params.necessary_reduction_for_restart = 0.5;
    params->restart_params.k_p = 0.99;
    params->restart_params.k_i = 0.01;
    params->restart_params.k_d = 0.0;
    params->restart_params.i_smooth = 0.3;
    params->optimality_norm = NORM_TYPE_L2;
    params->presolve = true;
    params->matrix_zero_tol = 1e-9;
}

void cp_al_result_free(cp_al_result_t *results) {
    if (!results) return;
    free(results->primal_solution);
    free(results->dual_solution);
    free(results->reduced_cost);
    free(results);
}

void lp_problem_free(lp_problem_t *prob) {
    if (!prob) return;
    free(prob->constraint_matrix_row_pointers);
    free(prob->constraint_matrix_col_indices);
    free(prob->constraint_matrix_values);
    free(prob->variable_lower_bound);
    free(prob->variable_upper_bound);
    free(prob->objective_vector);
    free(prob->constraint_lower_bound);
    free(prob->constraint_upper_bound);
    free(prob->primal_start);
    free(prob->dual_start);
    memset(prob, 0, sizeof(*prob));
    free(prob);
}

void cp_al_gb300_default_options(cp_al_gb300_options_t *o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->al_lambda = 0.05;
    o->sigma_mode = 0;
    o->sigma_set = 0;
    o->sigma = 0.0;
    o->sigma_adaptive = 1;
    o->sigma_init_factor = 6.0;
    o->sigma_min_factor = 1e-4;
    o->sigma_max_factor = 100.0;
    o->lambda_factor = 2.01;
    o->lambda_param_set = 0;
    o->lambda_param = 0.0;
    o->sigma_balance_gain = 0.15;
    o->sigma_i_smooth = NAN;
    o->sigma_kp = NAN;
    o->sigma_ki = NAN;
    o->sigma_kd = NAN;
    o->sigma_update_min = 0.60;
    o->sigma_update_max = 1.70;
    o->step_margin = 0.998 * 0.998;
    o->restart_sufficient = NAN;
    o->restart_necessary = NAN;
    o->restart_artificial = NAN;
    o->restart_select = 0;
    o->restart_select_margin = 1.0;
    o->restart_select_min_iters = 0;
    o->restart_select_threepoint = 0;
    o->restart_select_min_time = 0.0;
    o->cr_iterations = 0;
    o->cr_early_stop = 0;
    o->cr_early_stop_threshold = 0.1;
    o->precision = CP_AL_GB300_FP64;
    o->fp32_switch_tol = 1e-5;
    o->fp32_max_iterations = -1;
    o->spmv_nnz_per_block = 0;
    o->device = -1;
    o->graph_blocks = 1;
    o->timing = 0;
    o->fp32_stall_evals = 25;
    o->dual_panels = -1;
    o->panel_width = 0;
    o->primal_hot_rows = -1;
    o->power_method = -1;
    o->primal_staged = -1;
    o->infeasibility_detection = 0;
    o->eps_infeasible = 1e-8;
    o->persistent_loop = -1;
    o->dual_fused_finish = -1;
    o->device_transpose = -1;
    o->alpha_direct_pulse = 0;
    o->pulse_force = 0;
    o->pulse_trace = 0;
    o->pulse_test_limit = 0;
    o->sigma_trigger = 0;
    o->sigma_trigger_min_iters = 200;
    o->sigma_trigger_primal = 1e-2;
    o->sigma_trigger_dual = 1e-6;
    o->sigma_trigger_ratio = 1e6;
    o->dynamic_eval = 0;
    o->dynamic_eval_fast = 50;
    o->dynamic_eval_after_sec = -1.0;
    o->dynamic_eval_after_iters = -1;
    o->dynamic_eval_min_iters = 0;
    o->dynamic_eval_small_res = 1e-6;
    o->dynamic_eval_large_res = 1e-4;
    o->dynamic_eval_ratio = 1e4;
    o->dynamic_eval_bootstrap_iters = 0;
    o->dual_concurrent = -1;
}

/* Each variable is read the way the reference reads it
 * (LP/CP_AL/src/solver.cu:377-413: empty = unset, strtod/strtol, non-finite
 * ignored). */
/* The enabling reads of the controllers not built: LP/CP_AL/src/solver.cu:592
 * (rollback trial), 3168-3180 (adaptive lambda and its profiles). */
const char *cp_al_gb300_unbuilt_switch(void) {
    static const char *const kSwitches[] = {"CP_AL_ADAPTIVE_LAMBDA", "CP_AL_ALPHA_ROLLBACK_TRIAL"};
    for (const char *name : kSwitches)
        if (env_int(name, 0) != 0) return name;
    if (const char *prof = getenv("CP_AL_LAMBDA_PROFILE")) {
        static const char *const kProfiles[] = {"grid4_race", "race4", "mp_race", "safe_race", "mp_auto", "safe_auto"};
        for (const char *p : kProfiles)
            if (strcmp(prof, p) == 0) return "CP_AL_LAMBDA_PROFILE";
    }
    return nullptr;
}

void cp_al_gb300_options_from_env(cp_al_gb300_options_t *o) {
    if (!o) return;
    cp_al_gb300_default_options(o);
    o->al_lambda = env_double("CP_AL_LAMBDA", o->al_lambda);
    const bool sigma_env = env_set("CP_AL_SIGMA");
    o->sigma_mode = (sigma_env || env_int("CP_AL_SIGMA_MODE", 0) != 0) ? 1 : 0;
    o->sigma_set = env_parses("CP_AL_SIGMA") ? 1 : 0;
    o->sigma = env_double("CP_AL_SIGMA", 0.0);
    o->sigma_adaptive = env_int("CP_AL_SIGMA_ADAPTIVE", sigma_env ? 0 : 1) != 0;
    o->sigma_init_factor = env_double("CP_AL_SIGMA_INIT_FACTOR", o->sigma_init_factor);
    o->sigma_min_factor = env_double("CP_AL_SIGMA_MIN_FACTOR", o->sigma_min_factor);
    o->sigma_max_factor = env_double("CP_AL_SIGMA_MAX_FACTOR", o->sigma_max_factor);
    o->lambda_factor = env_double("CP_AL_LAMBDA_FACTOR", o->lambda_factor);
    o->lambda_param_set = env_parses("CP_AL_LAMBDA_PARAM") ? 1 : 0;
    o->lambda_param = env_double("CP_AL_LAMBDA_PARAM", 0.0);
    o->sigma_balance_gain = env_double("CP_AL_SIGMA_BALANCE_GAIN", o->sigma_balance_gain);
    o->sigma_i_smooth = env_double("CP_AL_SIGMA_I_SMOOTH", NAN);
    o->sigma_kp = env_double("CP_AL_SIGMA_KP", NAN);
    o->sigma_ki = env_double("CP_AL_SIGMA_KI", NAN);
    o->sigma_kd = env_double("CP_AL_SIGMA_KD", NAN);
    o->sigma_update_min = env_double("CP_AL_SIGMA_UPDATE_MIN", o->sigma_update_min);
    o->sigma_update_max = env_double("CP_AL_SIGMA_UPDATE_MAX", o->sigma_update_max);
    o->step_margin = env_double("CP_AL_STEP_MARGIN", o->step_margin);
    o->restart_sufficient = env_double("CP_AL_RESTART_SUFFICIENT", NAN);
    o->restart_necessary = env_double("CP_AL_RESTART_NECESSARY", NAN);
    o->restart_artificial = env_double("CP_AL_RESTART_ARTIFICIAL", NAN);
    o->restart_select = env_int("CP_AL_RESTART_SELECT", 0);
    o->restart_select_margin = env_double("CP_AL_RESTART_SELECT_MARGIN", 1.0);
    o->restart_select_min_iters = env_int("CP_AL_RESTART_SELECT_MIN_ITERS", 0);
    o->restart_select_threepoint = env_int("CP_AL_RESTART_SELECT_THREEPOINT", 0);
    o->restart_select_min_time = env_double("CP_AL_RESTART_SELECT_MIN_TIME", 0.0);
    /* LP/CP_AL/src/preconditioner.cu:174-178, 403-411 (atoi / atof, as read there) */
    const char *cr = getenv("CP_AL_CR_SCALING");
    int cr_iters = (cr && cr[0] != '\0' && atoi(cr) != 0) ? 20 : 0;
    const char *cr_it = getenv("CP_AL_CR_ITERS");
    if (cr_iters > 0 && cr_it && cr_it[0] != '\0') cr_iters = atoi(cr_it);
    o->cr_iterations = cr_iters < 0 ? 0 : cr_iters;
    const char *cr_es = getenv("CP_AL_CR_EARLY_STOP");
    o->cr_early_stop = (cr_es && atoi(cr_es) != 0) ? 1 : 0;
    const char *cr_th = getenv("CP_AL_CR_EARLY_STOP_THRESHOLD");
    o->cr_early_stop_threshold = cr_th ? atof(cr_th) : 0.1;
    /* LP/CP_AL/src/solver.cu:889-892, 1214-1216, 1497-1509 */
    o->alpha_direct_pulse = env_int("CP_AL_ALPHA_DIRECT_PULSE", 0) != 0;
    o->pulse_force = env_int("CP_AL_DETERMINISTIC_PULSE_FORCE", 0) != 0;
    o->pulse_trace = env_int("CP_AL_ALPHA_DIRECT_PULSE_TRACE", 0) != 0;
    o->pulse_test_limit = env_int("CP_AL_ALPHA_DIRECT_PULSE_TEST_TRAJECTORY_LIMIT", 0);
    o->sigma_trigger = env_int("CP_AL_SIGMA_TRIGGER", 0) != 0;
    o->sigma_trigger_min_iters = env_int("CP_AL_SIGMA_TRIGGER_MIN_ITERS", 200);
    o->sigma_trigger_primal = env_double("CP_AL_SIGMA_TRIGGER_PRIMAL", 1e-2);
    o->sigma_trigger_dual = env_double("CP_AL_SIGMA_TRIGGER_DUAL", 1e-6);
    o->sigma_trigger_ratio = env_double("CP_AL_SIGMA_TRIGGER_RATIO", 1e6);
    /* LP/CP_AL/src/solver.cu:1231-1255 */
    o->dynamic_eval = env_int("CP_AL_DYNAMIC_EVAL", 0) != 0;
    o->dynamic_eval_fast = env_int("CP_AL_DYNAMIC_EVAL_FAST", 50);
    o->dynamic_eval_after_sec = env_double("CP_AL_DYNAMIC_EVAL_AFTER_SEC", -1.0);
    o->dynamic_eval_after_iters = env_int("CP_AL_DYNAMIC_EVAL_AFTER_ITERS", -1);
    o->dynamic_eval_min_iters = env_int("CP_AL_DYNAMIC_EVAL_MIN_ITERS", 0);
    o->dynamic_eval_small_res = env_double("CP_AL_DYNAMIC_EVAL_SMALL_RES", 1e-6);
    o->dynamic_eval_large_res = env_double("CP_AL_DYNAMIC_EVAL_LARGE_RES", 1e-4);
    o->dynamic_eval_ratio = env_double("CP_AL_DYNAMIC_EVAL_RATIO", 1e4);
    o->dynamic_eval_bootstrap_iters = env_int("CP_AL_DYNAMIC_EVAL_BOOTSTRAP_ITERS", 0);
}

} // extern "C"

/* ---------------------------------------------------------------------- */
/* read_mps_file: LP/CP_AL/include/mps_parser.h:22                         */
/* ---------------------------------------------------------------------- */
#include "../../include/cp_al_mps_parser.h"
#include "mps_reader.h"

#include <string>
#include <vector>

namespace pdal {
void set_last_error(const std::string &msg);
void clear_last_error();
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

} // namespace

extern "C" lp_problem_t *read_mps_file(const char *filename) {
    pdal::clear_last_error();
    pdal::mps::Model M;
    std::string err;
    if (!pdal::mps::read_file(filename, false, M, err)) {
        pdal::set_last_error("read_mps_file: " + err);
        return nullptr;
    }
    lp_problem_t *p = (lp_problem_t *)calloc(1, sizeof(lp_problem_t));
    if (!p) {
        pdal::set_last_error("read_mps_file: out of host memory");
        return nullptr;
    }
    p->num_variables = M.num_cols;
    p->num_constraints = M.num_rows;
    p->constraint_matrix_num_nonzeros = (int)M.A.val.size();
    p->objective_constant = M.objective_constant;
    const bool ok = copy_out(M.c, &p->objective_vector) && copy_out(M.var_lb, &p->variable_lower_bound) &&
                    copy_out(M.var_ub, &p->variable_upper_bound) &&
                    copy_out(M.con_lb, &p->constraint_lower_bound) &&
                    copy_out(M.con_ub, &p->constraint_upper_bound) &&
                    copy_out(M.A.row_ptr, &p->constraint_matrix_row_pointers) &&
                    copy_out(M.A.col_ind, &p->constraint_matrix_col_indices) &&
                    copy_out(M.A.val, &p->constraint_matrix_values);
    if (!ok) {
        lp_problem_free(p);
        pdal::set_last_error("read_mps_file: out of host memory");
        return nullptr;
    }
    return p;
}
