/*
 * cli_fa_cp.cpp -- the `fa_cp` command: drop-in for the FA_CP binary
 * (QP/FA_CP/src/cli.c:261-455) on top of libfa_cp_gb300.so.
 *
 *     fa_cp [OPTIONS] <mps_or_qps_file> <output_dir>
 *
 * Same options, defaults and exit codes; writes <name>_summary.txt,
 * <name>_primal_solution.txt and <name>_dual_solution.txt into output_dir in
 * the reference's formats (cli.c:112-170), <name> being the file name up to
 * its first dot, and the per-evaluation CSV of --trajectory_csv.  -f runs
 * the feasibility polishing phases for problems without Q; for a QP the
 * library warns and solves without them.
 */
#include "../../include/fa_cp.h"
#include "../../include/fa_cp_mps_parser.h"

#include <getopt.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

namespace {

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

/* QP/FA_CP/src/utils.cu:390-411 */
const char *rule_name(sigma_update_rule_t r) {
    switch (r) {
    case FA_CP_SIGMA_UPDATE_FIXED: return "fixed";
    case FA_CP_SIGMA_UPDATE_RESIDUAL_BALANCE: return "residual";
    case FA_CP_SIGMA_UPDATE_KKT_BALANCE: return "kkt";
    case FA_CP_SIGMA_UPDATE_DISPLACEMENT: return "displacement";
    case FA_CP_SIGMA_UPDATE_PROGRESS: return "progress";
    case FA_CP_SIGMA_UPDATE_GREEDY_SCORE: return "greedy";
    case FA_CP_SIGMA_UPDATE_GUARDED: return "guarded";
    case FA_CP_SIGMA_UPDATE_BALANCED_GUARDED: return "balanced_guarded";
    default: return "unknown";
    }
}

/* cli.c:40-79: the accepted spellings of each rule */
bool parse_rule(const char *v, sigma_update_rule_t *r) {
    struct Name {
        const char *s;
        sigma_update_rule_t r;
    };
    static const Name names[] = {
        {"fixed", FA_CP_SIGMA_UPDATE_FIXED},
        {"none", FA_CP_SIGMA_UPDATE_FIXED},
        {"residual", FA_CP_SIGMA_UPDATE_RESIDUAL_BALANCE},
        {"kkt", FA_CP_SIGMA_UPDATE_KKT_BALANCE},
        {"displacement", FA_CP_SIGMA_UPDATE_DISPLACEMENT},
        {"progress", FA_CP_SIGMA_UPDATE_PROGRESS},
        {"greedy", FA_CP_SIGMA_UPDATE_GREEDY_SCORE},
        {"guarded", FA_CP_SIGMA_UPDATE_GUARDED},
        {"zero-aware", FA_CP_SIGMA_UPDATE_GUARDED},
        {"zero_aware", FA_CP_SIGMA_UPDATE_GUARDED},
        {"balanced_guarded", FA_CP_SIGMA_UPDATE_BALANCED_GUARDED},
        {"balanced-guarded", FA_CP_SIGMA_UPDATE_BALANCED_GUARDED},
        {"guarded_balanced", FA_CP_SIGMA_UPDATE_BALANCED_GUARDED},
        {"scaled_guarded", FA_CP_SIGMA_UPDATE_BALANCED_GUARDED},
    };
    for (const Name &n : names)
        if (strcmp(v, n.s) == 0) {
            *r = n.r;
            return true;
        }
    return false;
}

std::string instance_name(const char *path) {
    std::string s(path);
    while (s.size() > 1 && s.back() == '/') s.pop_back();
    const size_t slash = s.find_last_of('/');
    if (slash != std::string::npos && s.size() > 1) s = s.substr(slash + 1);
    const size_t dot = s.find('.');
    return dot == std::string::npos ? s : s.substr(0, dot);
}

std::string out_path(const char *dir, const std::string &name, const char *suffix) {
    return std::string(dir) + "/" + name + suffix;
}

void save_vector(const double *v, int n, const char *dir, const std::string &name, const char *suffix) {
    if (!v) return;
    const std::string p = out_path(dir, name, suffix);
    FILE *f = fopen(p.c_str(), "w");
    if (!f) {
        perror("Error opening solution file");
        return;
    }
    for (int i = 0; i < n; ++i) fprintf(f, "%.10g\n", v[i]);
    fclose(f);
}

void save_summary(const fa_cp_result_t *r, const char *dir, const std::string &name) {
    const std::string p = out_path(dir, name, "_summary.txt");
    FILE *f = fopen(p.c_str(), "w");
    if (!f) {
        perror("Error opening summary file");
        return;
    }
    fprintf(f, "Termination Reason: %s\n", reason_name(r->termination_reason));
    fprintf(f, "Runtime (sec): %e\n", r->cumulative_time_sec);
    fprintf(f, "Iterations Count: %d\n", r->total_count);
    if (r->total_inner_count > 0) fprintf(f, "Inner Iterations Count: %d\n", r->total_inner_count);
    fprintf(f, "Primal Objective Value: %e\n", r->primal_objective_value);
    fprintf(f, "Dual Objective Value: %e\n", r->dual_objective_value);
    fprintf(f, "Relative Primal Residual: %e\n", r->relative_primal_residual);
    fprintf(f, "Relative Dual Residual: %e\n", r->relative_dual_residual);
    fprintf(f, "Absolute Objective Gap: %e\n", r->objective_gap);
    fprintf(f, "Relative Objective Gap: %e\n", r->relative_objective_gap);
    fprintf(f, "Final AL Sigma: %e\n", r->final_al_sigma);
    fprintf(f, "Sigma Update Rule: %s\n", rule_name(r->sigma_update_rule));
    fprintf(f, "Sigma Update Count: %d\n", r->sigma_update_count);
    fprintf(f, "Rows: %d\n", r->num_constraints);
    fprintf(f, "Columns: %d\n", r->num_variables);
    fprintf(f, "Nonzeros: %d\n", r->num_nonzeros);
    if (r->feasibility_polishing_time > 0.0) {
        fprintf(f, "Feasibility Polishing Time (sec): %e\n", r->feasibility_polishing_time);
        fprintf(f, "Feasibility Polishing Iteration Count: %d\n", r->feasibility_iteration);
    }
    fclose(f);
}

/* One command-line option: long name, short letter (0 if none), value name
 * in the help (nullptr for a switch), help line, and what it sets.  Names,
 * meanings and defaults are the reference command's (QP/FA_CP/src/cli.c:
 * 265-400), which scripts call by name; the table and the help wording are
 * this command's own. */
struct Option {
    const char *name;
    char letter;
    const char *value;
    const char *help;
    bool (*apply)(fa_cp_parameters_t &, const char *); /* false: bad value, message printed */
};

using P = fa_cp_parameters_t;

bool set_norm(P &p, const char *v) {
    if (strcmp(v, "l2") == 0) {
        p.optimality_norm = NORM_TYPE_L2;
    } else if (strcmp(v, "linf") == 0) {
        p.optimality_norm = NORM_TYPE_L_INF;
    } else {
        fprintf(stderr, "Error: opt_norm must be 'l2' or 'linf'\n");
        return false;
    }
    return true;
}

bool set_rule(P &p, const char *v) {
    if (parse_rule(v, &p.sigma_update_rule)) return true;
    fprintf(stderr, "Error: sigma_update must be fixed, residual, kkt, displacement, progress, greedy, "
                    "guarded, or balanced_guarded\n");
    return false;
}

#define PDAL_DBL(field) [](P &p, const char *v) { return p.field = atof(v), true; }
#define PDAL_INT(field) [](P &p, const char *v) { return p.field = atoi(v), true; }

const Option kOptions[] = {
    {"eps_opt", 0, "TOL", "stop when the relative duality gap is below TOL (1e-4)",
     PDAL_DBL(termination_criteria.eps_optimal_relative)},
    {"eps_feas", 0, "TOL", "and both relative residuals are below TOL (1e-4)",
     PDAL_DBL(termination_criteria.eps_feasible_relative)},
    {"opt_norm", 0, "l2|linf", "norm of the residuals in that test (linf)", set_norm},
    {"eps_infeas_detect", 0, "TOL", "tolerance of the infeasibility certificates (1e-10)",
     PDAL_DBL(termination_criteria.eps_infeasible)},
    {"iter_limit", 0, "N", "give up after N iterations (no limit)", PDAL_INT(termination_criteria.iteration_limit)},
    {"time_limit", 0, "SEC", "give up after SEC seconds of wall time (3600)",
     PDAL_DBL(termination_criteria.time_sec_limit)},
    {"eval_freq", 0, "N", "iterations between two evaluations of the stopping test (200)",
     PDAL_INT(termination_evaluation_frequency)},
    {"l_inf_ruiz_iter", 0, "N", "passes of Ruiz max-norm equilibration (10)", PDAL_INT(l_inf_ruiz_iterations)},
    {"pock_chambolle_alpha", 0, "A", "exponent of the Pock-Chambolle scaling pass (1.0)",
     PDAL_DBL(pock_chambolle_alpha)},
    {"no_pock_chambolle", 0, nullptr, "skip the Pock-Chambolle scaling pass",
     [](P &p, const char *) { return p.has_pock_chambolle_alpha = false, true; }},
    {"no_bound_obj_rescaling", 0, nullptr, "skip the scaling of bounds and objective",
     [](P &p, const char *) { return p.bound_objective_rescaling = false, true; }},
    {"sv_max_iter", 0, "N", "cap on power-iteration steps for the largest singular value (5000)",
     PDAL_INT(sv_max_iter)},
    {"sv_tol", 0, "TOL", "power-iteration stopping tolerance (1e-4)", PDAL_DBL(sv_tol)},
    {"no_al_qp", 0, nullptr, "use the plain (non-augmented) primal-dual update",
     [](P &p, const char *) { return p.use_al_qp = false, true; }},
    {"al_sigma", 0, "S", "initial augmentation weight sigma of the primal subproblem (0)", PDAL_DBL(al_sigma)},
    {"sigma_update", 0, "RULE",
     "how sigma changes at restarts: fixed, residual, kkt, displacement, progress, greedy, guarded or "
     "balanced_guarded (guarded)",
     set_rule},
    {"sigma_update_gain", 0, "G", "damping of each sigma change, in the log domain (0.5)",
     PDAL_DBL(sigma_update_gain)},
    {"sigma_clip_low", 0, "F", "smallest factor one restart may apply to sigma (0.6)", PDAL_DBL(sigma_clip_low)},
    {"sigma_clip_high", 0, "F", "largest factor one restart may apply to sigma (1.7)", PDAL_DBL(sigma_clip_high)},
    {"sigma_min", 0, "S", "floor of a positive adaptive sigma (1e-8)", PDAL_DBL(sigma_min)},
    {"sigma_max", 0, "S", "ceiling of an adaptive sigma (10)", PDAL_DBL(sigma_max)},
    {"sigma_rollback_tol", 0, "F",
     "return to the best sigma seen when the restart score grows by more than F (1.25; <= 0: never)",
     PDAL_DBL(sigma_rollback_tol)},
    {"sigma_zero_threshold", 0, "S", "a guarded sigma below S becomes exactly 0 (1e-8)",
     PDAL_DBL(sigma_zero_threshold)},
    {"sigma_activation_threshold", 0, "R",
     "primal residual over the larger of dual residual and gap that switches guarded sigma on (2)",
     PDAL_DBL(sigma_activation_threshold)},
    {"sigma_normal_motion_threshold", 0, "R", "smallest |A dx| / |dx| that lets guarded sigma switch on (1e-10)",
     PDAL_DBL(sigma_normal_motion_threshold)},
    {"sigma_activation_value", 0, "S",
     "sigma a guarded rule starts from when it switches on; theta of sigma = theta * dual step for "
     "balanced_guarded (0.1)",
     PDAL_DBL(sigma_activation_value)},
    {"feasibility_polishing", 'f', nullptr, "polishing phases after the solve (problems without Q)",
     [](P &p, const char *) { return p.feasibility_polishing = true, true; }},
    {"eps_feas_polish", 0, "TOL", "residual target of the polishing phases (1e-6)",
     PDAL_DBL(termination_criteria.eps_feas_polish_relative)},
    {"trajectory_csv", 0, "PATH", "append one CSV line per evaluation to PATH",
     [](P &p, const char *v) { return p.trajectory_csv = v, true; }},
    {"verbose", 'v', "LEVEL", "0 silent, 1 summary, 2 every evaluation (1)", PDAL_INT(verbose)},
};
#undef PDAL_DBL
#undef PDAL_INT
constexpr int kNumOptions = sizeof(kOptions) / sizeof(kOptions[0]);
constexpr int kHelpCode = 'h';
constexpr int kFirstCode = 0x200; /* getopt return value of option i: kFirstCode + i */

void usage(const char *prog) {
    fprintf(stderr, "Usage: %s [OPTIONS] <mps_file> <output_dir>\n\n", prog);
    fprintf(stderr, "Solves the convex quadratic program in <mps_file> (MPS or QPS text, optionally\n");
    fprintf(stderr, "gzip-compressed) on the GPU and writes into <output_dir>, for an input NAME.qps:\n");
    fprintf(stderr, "  NAME_summary.txt          status, iterations, objectives, residuals, sigma, times\n");
    fprintf(stderr, "  NAME_primal_solution.txt  one value of x per line\n");
    fprintf(stderr, "  NAME_dual_solution.txt    one value of y per line\n\n");
    fprintf(stderr, "Options (defaults in parentheses):\n");
    fprintf(stderr, "  -h, --help  show this text\n");
    for (const Option &o : kOptions) {
        char head[64];
        snprintf(head, sizeof head, "--%s%s%s", o.name, o.value ? " " : "", o.value ? o.value : "");
        if (o.letter)
            fprintf(stderr, "  -%c, %-38s %s\n", o.letter, head, o.help);
        else
            fprintf(stderr, "      %-38s %s\n", head, o.help);
    }
}

} // namespace

int main(int argc, char *argv[]) {
    fa_cp_parameters_t params;
    set_default_parameters(&params);

    struct option long_options[kNumOptions + 2];
    std::string shorts = "h";
    long_options[0] = {"help", no_argument, nullptr, kHelpCode};
    for (int i = 0; i < kNumOptions; ++i) {
        const Option &o = kOptions[i];
        long_options[i + 1] = {o.name, o.value ? required_argument : no_argument, nullptr, kFirstCode + i};
        if (o.letter) {
            shorts += o.letter;
            if (o.value) shorts += ':';
        }
    }
    long_options[kNumOptions + 1] = {nullptr, 0, nullptr, 0};
    shorts += "p"; /* accepted and ignored, as by the reference command */
    int opt;
    while ((opt = getopt_long(argc, argv, shorts.c_str(), long_options, nullptr)) != -1) {
        if (opt == kHelpCode) {
            usage(argv[0]);
            return 0;
        }
        if (opt == '?') return 1;
        int idx = -1;
        if (opt >= kFirstCode && opt < kFirstCode + kNumOptions) {
            idx = opt - kFirstCode;
        } else {
            for (int i = 0; i < kNumOptions; ++i)
                if (kOptions[i].letter && kOptions[i].letter == opt) idx = i;
        }
        if (idx >= 0 && !kOptions[idx].apply(params, optarg)) return 1;
    }
    if (argc - optind != 2) {
        fprintf(stderr, "Error: You must specify an input file and an output directory.\n\n");
        usage(argv[0]);
        return 1;
    }
    const char *filename = argv[optind];
    const char *output_dir = argv[optind + 1];
    const std::string name = instance_name(filename);
    qp_problem_t *problem = read_mps_file(filename);
    if (!problem) {
        fprintf(stderr, "Failed to read or parse the file.\n");
        return 1;
    }
    fa_cp_result_t *result = solve_qp_problem(problem, &params);
    if (!result) {
        fprintf(stderr, "Solver failed.\n");
    } else {
        save_summary(result, output_dir, name);
        save_vector(result->primal_solution, problem->num_variables, output_dir, name, "_primal_solution.txt");
        save_vector(result->dual_solution, problem->num_constraints, output_dir, name, "_dual_solution.txt");
        fa_cp_result_free(result);
    }
    qp_problem_free(problem);
    return 0;
}
