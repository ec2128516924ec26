/*
 * A harness around the reference command's policy layer: LP/CP_AL/src/cli.c
 * is included unmodified, where it lies, and its static feature, policy and
 * structural-tail functions are exported for the parity tests
 * (tests/test_policy.py).  The solver the structural tail calls is a
 * callback the test scripts; the other library functions cli.c calls are
 * small stand-ins (warm-start copy, result free, status names), none of
 * which the policies' decisions depend on.  Built by oracle/build.py
 * (build_ref) with ref_mps_shim.c into oracle/_ref/libref_cli_policy.so.
 * Test infrastructure only.
 */
#define main ref_cli_command_main
#include "cli.c"
#undef main

typedef cp_al_result_t *(*ref_solve_fn)(lp_problem_t *, const cp_al_parameters_t *);
static ref_solve_fn g_solve;

void ref_cli_set_solver(ref_solve_fn fn) { g_solve = fn; }

cp_al_result_t *solve_lp_problem(lp_problem_t *prob, const cp_al_parameters_t *params) {
    return g_solve ? g_solve(prob, params) : NULL;
}

void set_start_values(lp_problem_t *prob, const double *primal, const double *dual) {
    free(prob->primal_start);
    free(prob->dual_start);
    prob->primal_start = NULL;
    prob->dual_start = NULL;
    if (primal) {
        prob->primal_start = safe_malloc(sizeof(double) * (size_t)(prob->num_variables > 0 ? prob->num_variables : 1));
        memcpy(prob->primal_start, primal, sizeof(double) * (size_t)prob->num_variables);
    }
    if (dual) {
        prob->dual_start = safe_malloc(sizeof(double) * (size_t)(prob->num_constraints > 0 ? prob->num_constraints : 1));
        memcpy(prob->dual_start, dual, sizeof(double) * (size_t)prob->num_constraints);
    }
}

void cp_al_result_free(cp_al_result_t *r) {
    if (!r) return;
    free(r->primal_solution);
    free(r->dual_solution);
    free(r->reduced_cost);
    free(r);
}

const char *termination_reason_to_string(termination_reason_t reason) {
    static const char *const names[] = {"OPTIMAL", "PRIMAL_INFEASIBLE", "DUAL_INFEASIBLE", "INFEASIBLE_OR_UNBOUNDED",
                                        "TIME_LIMIT", "ITERATION_LIMIT", "UNSPECIFIED", "FEAS_POLISH_SUCCESS"};
    switch (reason) {
    case TERMINATION_REASON_OPTIMAL: return names[0];
    case TERMINATION_REASON_PRIMAL_INFEASIBLE: return names[1];
    case TERMINATION_REASON_DUAL_INFEASIBLE: return names[2];
    case TERMINATION_REASON_INFEASIBLE_OR_UNBOUNDED: return names[3];
    case TERMINATION_REASON_TIME_LIMIT: return names[4];
    case TERMINATION_REASON_ITERATION_LIMIT: return names[5];
    case TERMINATION_REASON_UNSPECIFIED: return names[6];
    case TERMINATION_REASON_FEAS_POLISH_SUCCESS: return names[7];
    default: return "UNKNOWN";
    }
}

const char *get_presolve_status_str(enum PresolveStatus_ status) {
    (void)status;
    return "UNSPECIFIED";
}

void set_default_parameters(cp_al_parameters_t *params) { memset(params, 0, sizeof(*params)); }

lp_problem_t *read_mps_file(const char *filename) {
    (void)filename;
    return NULL;
}

/* the reference's features as twelve doubles in the struct's order */
void ref_cli_feature_stats(const lp_problem_t *prob, double *out) {
    feature_matrix_stats_t s = compute_feature_matrix_stats(prob);
    memcpy(out, &s, sizeof(s));
}

static feature_matrix_stats_t from_array(const double *in) {
    feature_matrix_stats_t s;
    memcpy(&s, in, sizeof(s));
    return s;
}

void ref_cli_unified_policy(const double *stats) {
    feature_matrix_stats_t s = from_array(stats);
    apply_unified_policy(&s);
}

void ref_cli_feature_policy(const lp_problem_t *prob, cp_al_parameters_t *params, const double *stats) {
    feature_matrix_stats_t s = from_array(stats);
    apply_feature_auto_policy(prob, params, &s);
}

cp_al_result_t *ref_cli_structural_tail(lp_problem_t *prob, const cp_al_parameters_t *params, const double *stats,
                                        int tail_pulse) {
    feature_matrix_stats_t s = from_array(stats);
    return run_structural_tail_cut(prob, params, &s, tail_pulse != 0);
}
