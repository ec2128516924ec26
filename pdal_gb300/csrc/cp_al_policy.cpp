/*
 * cp_al_policy.cpp -- the CP_AL command's benchmark policy layer
 * (LP/CP_AL/src/cli.c:52-470, 588-833) as library functions.
 *
 * Nothing here touches the GPU: the features are one pass over the host CSR
 * matrix, the policies set CP_AL_* environment variables (and the evaluation
 * frequency and reflection coefficient of the parameters), and the structural
 * tail calls solve_lp_problem once or twice.  The decision rules, their
 * thresholds and the variables they set are the reference's, since the
 * benchmark protocol is defined by them; the stderr lines keep the
 * reference's tags and fields for the log collectors that read them.
 */
#include "../../include/cp_al.h"
#include "../../include/cp_al_policy.h"

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

namespace {

cp_al_solve_fn g_solve = nullptr;

bool flag(const char *name) {
    const char *v = getenv(name);
    return v && v[0] != '\0' && atoi(v) != 0;
}

const char *env_or(const char *name, const char *fallback) {
    const char *v = getenv(name);
    return (v && v[0] != '\0') ? v : fallback;
}

void put(const char *name, const char *value) { setenv(name, value, 1); }
void drop(const char *name) { unsetenv(name); }

const char *reason_name(termination_reason_t r) {
    switch (r) {
    case TERMINATION_REASON_OPTIMAL: return "OPTIMAL";
    case TERMINATION_REASON_PRIMAL_INFEASIBLE: return "PRIMAL_INFEASIBLE";
    case TERMINATION_REASON_DUAL_INFEASIBLE: return "DUAL_INFEASIBLE";
    case TERMINATION_REASON_INFEASIBLE_OR_UNBOUNDED: return "INFEASIBLE_OR_UNBOUNDED";
    case TERMINATION_REASON_TIME_LIMIT: return "TIME_LIMIT";
    case TERMINATION_REASON_ITERATION_LIMIT: return "ITERATION_LIMIT";
    case TERMINATION_REASON_UNSPECIFIED: return "UNSPECIFIED";
    case TERMINATION_REASON_FEAS_POLISH_SUCCESS: return "FEAS_POLISH_SUCCESS";
    default: return "UNKNOWN";
    }
}

cp_al_result_t *run_solve(lp_problem_t *prob, const cp_al_parameters_t *params) {
    return g_solve ? g_solve(prob, params) : solve_lp_problem(prob, params);
}

/* Running sums of a sample: mean, standard deviation and coefficient of
 * variation as cli.c:69-88 forms them (population moments from the sum and
 * the sum of squares, a negative variance clamped to zero). */
struct Moments {
    double sum = 0.0, sq = 0.0;
    void add(double v) {
        sum += v;
        sq += v * v;
    }
    double mean(int n) const { return n > 0 ? sum / (double)n : 0.0; }
    double stddev(int n) const {
        if (n <= 0) return 0.0;
        const double mu = sum / (double)n;
        return std::sqrt(std::fmax(sq / (double)n - mu * mu, 0.0));
    }
    double cv(int n) const {
        if (n <= 0 || sum <= 0.0) return 0.0;
        const double mu = sum / (double)n;
        return std::sqrt(std::fmax(sq / (double)n - mu * mu, 0.0)) / mu;
    }
};

/* the decades spanned by the magnitudes of one row or column */
struct Span {
    double lo = DBL_MAX, hi = 0.0;
    void add(double v) {
        lo = std::fmin(lo, v);
        hi = std::fmax(hi, v);
    }
    bool seen() const { return hi > 0.0 && lo < DBL_MAX; }
};

/* A row's or column's span statistics: log10 of its largest magnitude, its
 * span in decades, and the count with a span of two decades or more. */
struct SpanStats {
    Moments logmax;
    double logspan_sum = 0.0;
    int seen = 0, wide = 0;
    void add(const Span &s) {
        if (!s.seen()) return;
        const double top = std::log10(s.hi);
        const double decades = std::log10(s.hi / s.lo);
        logmax.add(top);
        logspan_sum += decades;
        wide += decades >= 2.0 ? 1 : 0;
        seen += 1;
    }
};

} // namespace

extern "C" {

void cp_al_policy_set_solver(cp_al_solve_fn fn) { g_solve = fn; }

int cp_al_feature_stats(const lp_problem_t *prob, cp_al_feature_stats_t *out) {
    if (!prob || !out) return -1;
    memset(out, 0, sizeof(*out));
    const int m = prob->num_constraints, n = prob->num_variables, nnz = prob->constraint_matrix_num_nonzeros;
    if (m <= 0 || n <= 0 || nnz <= 0) return 0;
    const int *rp = prob->constraint_matrix_row_pointers, *ci = prob->constraint_matrix_col_indices;
    const double *av = prob->constraint_matrix_values;

    std::vector<Span> col(n);
    std::vector<int> col_count(n, 0);
    Span all;
    SpanStats rows, cols;
    Moments row_len, col_len;
    for (int i = 0; i < m; ++i) {
        const int b = rp[i], e = rp[i + 1];
        row_len.add((double)(e - b)); /* stored entries, as cli.c:120-122 counts them */
        Span r;
        for (int k = b; k < e; ++k) {
            const double v = std::fabs(av[k]);
            const int j = ci[k];
            if (!std::isfinite(v) || v <= 0.0 || j < 0 || j >= n) continue;
            all.add(v);
            r.add(v);
            col[j].add(v);
            col_count[j] += 1;
        }
        rows.add(r);
    }
    for (int j = 0; j < n; ++j) {
        col_len.add((double)col_count[j]); /* usable entries only (cli.c:139-141) */
        cols.add(col[j]);
    }
    out->coeff_log_range = all.seen() ? std::log10(all.hi / all.lo) : 0.0;
    out->row_logmax_std = rows.logmax.stddev(rows.seen);
    out->col_logmax_std = cols.logmax.stddev(cols.seen);
    out->row_logspan_mean = rows.seen > 0 ? rows.logspan_sum / (double)rows.seen : 0.0;
    out->col_logspan_mean = cols.seen > 0 ? cols.logspan_sum / (double)cols.seen : 0.0;
    out->row_span2_fraction = rows.seen > 0 ? (double)rows.wide / (double)rows.seen : 0.0;
    out->col_span2_fraction = cols.seen > 0 ? (double)cols.wide / (double)cols.seen : 0.0;
    out->row_nnz_cv = row_len.cv(m);
    out->col_nnz_cv = col_len.cv(n);

    int eq = 0, boxed = 0, priced = 0;
    for (int i = 0; i < m; ++i) {
        const double lo = prob->constraint_lower_bound[i], up = prob->constraint_upper_bound[i];
        eq += (std::isfinite(lo) && std::isfinite(up) && lo == up) ? 1 : 0;
    }
    for (int j = 0; j < n; ++j) {
        boxed += (std::isfinite(prob->variable_lower_bound[j]) && std::isfinite(prob->variable_upper_bound[j])) ? 1 : 0;
        priced += std::fabs(prob->objective_vector[j]) > 0.0 ? 1 : 0;
    }
    out->equality_fraction = (double)eq / (double)m;
    out->two_sided_variable_fraction = (double)boxed / (double)n;
    out->objective_density = (double)priced / (double)n;
    return 0;
}

int cp_al_feature_policy(const lp_problem_t *prob, cp_al_parameters_t *params, const cp_al_feature_stats_t *stats) {
    if (!flag("CP_AL_FEATURE_AUTO_POLICY")) return 0;
    if (!stats) {
        fprintf(stderr, "[feature-auto-policy-error] reason=missing-precomputed-stats\n");
        return 0;
    }
    const std::string variant = env_or("CP_AL_FEATURE_POLICY_VARIANT", "safe0");
    const bool probe = variant == "probe";
    const bool always = variant == "always_select" || variant == "always_noselect";
    const bool trigger = variant == "trigger" || variant == "trigger_select" || probe;
    const bool select = variant == "always_select" || variant == "trigger_select";

    int eval_freq = 200;
    if (const char *v = getenv("CP_AL_UNIFIED_EVAL_FREQ"); v && v[0] != '\0' && atoi(v) > 0) eval_freq = atoi(v);
    if (params) {
        params->termination_evaluation_frequency = eval_freq;
        params->reflection_coefficient = 1.0;
    }
    put("CP_AL_LAMBDA", "0");
    put("CP_AL_LAMBDA_FACTOR", "2.01");
    put("CP_AL_ADAPTIVE_LAMBDA", "0");
    drop("CP_AL_LAMBDA_PROFILE");
    drop("CP_AL_LAMBDA_GRID");

    /* Curtis-Reid effort from the column-count spread and the coefficient
     * range (cli.c:269-298) unless CP_AL_FEATURE_CR_ITERS fixes it */
    const cp_al_feature_stats_t &f = *stats;
    int cr_override = -1, cr = 0;
    if (const char *v = getenv("CP_AL_FEATURE_CR_ITERS"); v && v[0] != '\0') {
        cr_override = atoi(v) < 0 ? 0 : atoi(v);
        cr = cr_override;
    } else if (f.col_nnz_cv <= 0.19012745) {
        cr = 5;
    } else if (f.col_nnz_cv <= 0.39521255) {
        cr = 50;
    } else {
        cr = f.coeff_log_range <= 3.222854 ? 5 : 20;
    }
    char buf[32];
    snprintf(buf, sizeof(buf), "%d", cr);
    put("CP_AL_CR_ITERS", buf);
    put("CP_AL_CR_SCALING", cr > 0 ? "1" : "0");

    const char *init_factor = env_or("CP_AL_FEATURE_SIGMA_INIT_FACTOR", "6.0");
    const char *trig_iters = env_or("CP_AL_FEATURE_SIGMA_TRIGGER_MIN_ITERS", "200");
    const char *trig_p = env_or("CP_AL_FEATURE_SIGMA_TRIGGER_PRIMAL", "1e-2");
    const char *trig_d = env_or("CP_AL_FEATURE_SIGMA_TRIGGER_DUAL", "1e-6");
    const char *trig_r = env_or("CP_AL_FEATURE_SIGMA_TRIGGER_RATIO", "1e6");
    put("CP_AL_SIGMA_MODE", always ? "1" : "0");
    put("CP_AL_SIGMA_ADAPTIVE", "1");
    put("CP_AL_SIGMA_INIT_FACTOR", init_factor);
    put("CP_AL_SIGMA_TRIGGER", trigger ? "1" : "0");
    put("CP_AL_SIGMA_TRIGGER_MIN_ITERS", trig_iters);
    put("CP_AL_SIGMA_TRIGGER_PRIMAL", trig_p);
    put("CP_AL_SIGMA_TRIGGER_DUAL", trig_d);
    put("CP_AL_SIGMA_TRIGGER_RATIO", trig_r);

    put("CP_AL_DYNAMIC_EVAL", trigger && !probe ? "1" : "0");
    put("CP_AL_DYNAMIC_EVAL_FAST", env_or("CP_AL_FEATURE_DYNAMIC_EVAL_FAST", "50"));
    put("CP_AL_DYNAMIC_EVAL_MIN_ITERS", "200");
    put("CP_AL_DYNAMIC_EVAL_SMALL_RES", "1e-6");
    put("CP_AL_DYNAMIC_EVAL_LARGE_RES", "1e-4");
    put("CP_AL_DYNAMIC_EVAL_RATIO", "1e4");

    put("CP_AL_RESTART_SELECT", select ? "3" : "0");
    drop("CP_AL_RESTART_SELECT_PROFILE");
    put("CP_AL_RESTART_SELECT_MARGIN", "0.9");
    put("CP_AL_RESTART_SUFFICIENT", "0.2");
    put("CP_AL_RESTART_NECESSARY", "0.8");
    put("CP_AL_RESTART_ARTIFICIAL", "0.36");
    drop("CP_AL_STEP_MARGIN");

    const int m = prob ? prob->num_constraints : 0, n = prob ? prob->num_variables : 0;
    const int nnz = prob ? prob->constraint_matrix_num_nonzeros : 0;
    const double dm = m > 0 ? m : 1, dn = n > 0 ? n : 1, dnz = nnz > 0 ? nnz : 1;
    fprintf(stderr,
            "[feature-auto-policy] version=2 variant=%s eval_base=200 refl=1 rows=%d cols=%d nnz=%d "
            "n_over_m=%.6e nnz_per_col=%.6e sigma_pid=1 sigma_always=%d sigma_trigger=%d "
            "sigma_probe=%d sigma_init_factor=%s sigma_trigger_min_iters=%s "
            "restart_select=%d cr_override=%d cr_selected=%d coeff_log_range=%.6e row_logmax_std=%.6e "
            "col_logmax_std=%.6e row_logspan_mean=%.6e col_logspan_mean=%.6e row_span2_frac=%.6e "
            "col_span2_frac=%.6e row_nnz_cv=%.6e col_nnz_cv=%.6e equality_frac=%.6e two_sided_var_frac=%.6e "
            "objective_density=%.6e\n",
            variant.c_str(), m, n, nnz, dn / dm, dnz / dn, always ? 1 : 0, trigger ? 1 : 0, probe ? 1 : 0,
            init_factor, trig_iters, select ? 3 : 0, cr_override, cr, f.coeff_log_range, f.row_logmax_std,
            f.col_logmax_std, f.row_logspan_mean, f.col_logspan_mean, f.row_span2_fraction, f.col_span2_fraction,
            f.row_nnz_cv, f.col_nnz_cv, f.equality_fraction, f.two_sided_variable_fraction, f.objective_density);
    return 1;
}

const char *cp_al_unified_policy(const cp_al_feature_stats_t *stats) {
    if (!flag("CP_AL_UNIFIED_POLICY")) return nullptr;
    if (!stats) {
        fprintf(stderr, "[unified-policy-error] reason=missing-precomputed-stats\n");
        return nullptr;
    }
    const cp_al_feature_stats_t &f = *stats;
    put("CP_AL_FEATURE_AUTO_POLICY", "1");
    put("CP_AL_FEATURE_POLICY_VARIANT", "safe0");
    const char *route;
    if (f.objective_density <= 0.01 && f.col_nnz_cv >= 5.0) {
        route = "lowobj_highcv_eval100_cr5";
        put("CP_AL_FEATURE_CR_ITERS", "5");
        put("CP_AL_UNIFIED_EVAL_FREQ", "100");
        drop("CP_AL_STRUCTURAL_TAIL_CUT");
        drop("CP_AL_TAIL_ONLY_PULSE");
    } else if (f.equality_fraction == 0.0) {
        route = "zero_equality_cr0";
        put("CP_AL_FEATURE_CR_ITERS", "0");
        drop("CP_AL_STRUCTURAL_TAIL_CUT");
        drop("CP_AL_TAIL_ONLY_PULSE");
    } else {
        route = "high_equality_tail_or_base";
        drop("CP_AL_FEATURE_CR_ITERS");
        put("CP_AL_STRUCTURAL_TAIL_CUT", "1");
        put("CP_AL_TAIL_ONLY_PULSE", "1");
    }
    fprintf(stderr,
            "[unified-policy] version=2 route=%s equality_frac=%.6e row_nnz_cv=%.6e col_nnz_cv=%.6e "
            "objective_density=%.6e row_logmax_std=%.6e\n",
            route, f.equality_fraction, f.row_nnz_cv, f.col_nnz_cv, f.objective_density, f.row_logmax_std);
    return route;
}

cp_al_result_t *cp_al_structural_tail(lp_problem_t *prob, const cp_al_parameters_t *params,
                                      const cp_al_feature_stats_t *stats, int tail_pulse) {
    if (!stats) {
        fprintf(stderr, "[structural-tail-error] reason=missing-precomputed-stats\n");
        return run_solve(prob, params);
    }
    const cp_al_feature_stats_t &f = *stats;
    /* the predicate (cli.c:617-628): a dense objective over rows of one
     * scale, with all or none of the rows equalities */
    const bool uniform = f.objective_density >= 0.99 && f.row_logmax_std <= 0.05;
    const bool low_eq = uniform && f.equality_fraction <= 0.001;
    const bool high_eq = uniform && f.equality_fraction >= 0.99;
    const bool cut = low_eq || high_eq;
    const bool pulse = tail_pulse && cut;
    const double base_fraction = high_eq ? 0.05 : 0.75;
    const double limit = params->termination_criteria.time_sec_limit;
    if (!std::isfinite(limit) || limit <= 0.0) {
        fprintf(stderr, "[structural-tail-error] reason=invalid-time-limit value=%.12e\n", limit);
        return run_solve(prob, params);
    }
    auto config_line = [&](double base_limit) {
        if (cut)
            fprintf(stderr,
                    "[structural-tail-config] enabled=1 structural_early_cut=1 structural_low_equality=%d "
                    "structural_high_equality=%d base_fraction=%.2f rescue_fraction=%.2f rescue_profile=cr0 "
                    "base_alpha=0 tail_pulse_requested=%d tail_pulse_enabled=%d "
                    "tail_pulse_alpha=2.000000000000e-03 equality_fraction=%.12e objective_density=%.12e "
                    "row_logmax_std=%.12e original_limit=%.12e base_limit=%.12e\n",
                    low_eq ? 1 : 0, high_eq ? 1 : 0, base_fraction, 1.0 - base_fraction, tail_pulse ? 1 : 0,
                    pulse ? 1 : 0, f.equality_fraction, f.objective_density, f.row_logmax_std, limit, base_limit);
        else
            fprintf(stderr,
                    "[structural-tail-config] enabled=1 structural_early_cut=0 structural_low_equality=0 "
                    "structural_high_equality=0 base_fraction=1.00 rescue_fraction=0.00 rescue_profile=none "
                    "base_alpha=0 tail_pulse_requested=%d tail_pulse_enabled=0 "
                    "tail_pulse_alpha=2.000000000000e-03 equality_fraction=%.12e objective_density=%.12e "
                    "row_logmax_std=%.12e original_limit=%.12e base_limit=%.12e\n",
                    tail_pulse ? 1 : 0, f.equality_fraction, f.objective_density, f.row_logmax_std, limit, limit);
    };
    auto base_line = [](const cp_al_result_t *r) {
        fprintf(stderr, "[structural-tail-base] status=%s solve_sec=%.12e precondition_sec=%.12e iterations=%d\n",
                reason_name(r->termination_reason), r->cumulative_time_sec, r->rescaling_time_sec, r->total_count);
    };

    if (!cut) {
        put("CP_AL_ALPHA_DIRECT_PULSE", "0");
        put("CP_AL_DETERMINISTIC_PULSE_FORCE", "0");
        config_line(limit);
        cp_al_result_t *r = run_solve(prob, params);
        if (!r) {
            fprintf(stderr, "[structural-tail-error] reason=null-single-phase-result\n");
            return nullptr;
        }
        base_line(r);
        fprintf(stderr,
                "[structural-tail-final] phases=1 tail_started=0 status=%s structural_early_cut=0 base_fraction=1.00 "
                "rescue_profile=none base_solve_sec=%.12e rescue_solve_sec=0 aggregate_solve_sec=%.12e "
                "budget_excess=%.12e total_iterations=%d\n",
                reason_name(r->termination_reason), r->cumulative_time_sec, r->cumulative_time_sec,
                std::fmax(r->cumulative_time_sec - limit, 0.0), r->total_count);
        return r;
    }

    /* phase 1: the base solve on its share of the time */
    cp_al_parameters_t base_params = *params;
    base_params.termination_criteria.time_sec_limit = base_fraction * limit;
    config_line(base_params.termination_criteria.time_sec_limit);
    put("CP_AL_ALPHA_DIRECT_PULSE", "0");
    put("CP_AL_DETERMINISTIC_PULSE_FORCE", "0");
    cp_al_result_t *base = run_solve(prob, &base_params);
    if (!base) {
        fprintf(stderr, "[structural-tail-error] reason=null-base-result\n");
        return nullptr;
    }
    const double base_sec = base->cumulative_time_sec;
    base_line(base);
    auto one_phase = [&](const char *tail) {
        fprintf(stderr,
                "[structural-tail-final] phases=1 tail_started=0 status=%s structural_early_cut=1 base_fraction=%.2f "
                "rescue_profile=cr0 base_solve_sec=%.12e rescue_solve_sec=0 aggregate_solve_sec=%.12e "
                "budget_excess=%.12e total_iterations=%d%s\n",
                reason_name(base->termination_reason), base_fraction, base_sec, base_sec,
                std::fmax(base_sec - limit, 0.0), base->total_count, tail);
        return base;
    };
    if (base->termination_reason == TERMINATION_REASON_OPTIMAL) return one_phase("");
    const double remaining = std::fmax(limit - base_sec, 0.0);
    if (remaining <= 0.0) return one_phase(" reason=no-remaining-budget");

    /* phase 2: the rescue, warm-started at the base solve's point */
    set_start_values(prob, base->primal_solution, base->dual_solution);
    double moved = 0.0; /* distance of the stored start from the base point (cli.c:588-605) */
    for (int j = 0; j < prob->num_variables; ++j) {
        const double d = prob->primal_start[j] - base->primal_solution[j];
        moved += d * d;
    }
    for (int i = 0; i < prob->num_constraints; ++i) {
        const double d = prob->dual_start[i] - base->dual_solution[i];
        moved += d * d;
    }
    moved = std::sqrt(moved);
    cp_al_parameters_t rescue_params = *params;
    put("CP_AL_FEATURE_CR_ITERS", "0");
    const clock_t c0 = clock();
    cp_al_feature_policy(prob, &rescue_params, stats);
    const double policy_sec = (double)(clock() - c0) / CLOCKS_PER_SEC;
    rescue_params.termination_evaluation_frequency = 200;
    rescue_params.termination_criteria.time_sec_limit = remaining;
    put("CP_AL_ALPHA_DIRECT_PULSE", pulse ? "1" : "0");
    put("CP_AL_DETERMINISTIC_PULSE_FORCE", pulse ? "1" : "0");
    fprintf(stderr,
            "[structural-tail-start] profile=cr0 remaining_limit=%.12e anchor_copy_l2=%.12e policy_sec=%.12e "
            "tail_pulse_requested=%d tail_pulse_enabled=%d\n",
            remaining, moved, policy_sec, tail_pulse ? 1 : 0, pulse ? 1 : 0);
    cp_al_result_t *rescue = run_solve(prob, &rescue_params);
    if (!rescue) {
        fprintf(stderr, "[structural-tail-error] reason=null-rescue-result\n");
        return base;
    }
    const double rescue_sec = rescue->cumulative_time_sec;
    fprintf(stderr, "[structural-tail-rescue] status=%s solve_sec=%.12e precondition_sec=%.12e iterations=%d\n",
            reason_name(rescue->termination_reason), rescue_sec, rescue->rescaling_time_sec, rescue->total_count);
    /* the result accounts for both phases (cli.c:800-804) */
    rescue->cumulative_time_sec += base_sec;
    rescue->rescaling_time_sec += base->rescaling_time_sec;
    rescue->presolve_time += base->presolve_time;
    rescue->feasibility_polishing_time += base->feasibility_polishing_time;
    rescue->total_count += base->total_count;
    fprintf(stderr,
            "[structural-tail-final] phases=2 tail_started=1 status=%s structural_early_cut=1 base_fraction=%.2f "
            "rescue_profile=cr0 base_solve_sec=%.12e rescue_solve_sec=%.12e aggregate_solve_sec=%.12e "
            "budget_excess=%.12e total_iterations=%d anchor_copy_l2=%.12e\n",
            reason_name(rescue->termination_reason), base_fraction, base_sec, rescue_sec, rescue->cumulative_time_sec,
            std::fmax(rescue->cumulative_time_sec - limit, 0.0), rescue->total_count, moved);
    cp_al_result_free(base);
    return rescue;
}

} // extern "C"
