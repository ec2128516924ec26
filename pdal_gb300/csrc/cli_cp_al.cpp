/*
 * cli_cp_al.cpp -- the `cp_al` command: drop-in for the CP_AL binary
 * (LP/CP_AL/src/cli.c:836-1092) on top of libcp_al_gb300.so.
 *
 *     cp_al [OPTIONS] <mps_file> <output_dir>
 *
 * Same options, defaults and exit codes; writes <name>_summary.txt,
 * <name>_primal_solution.txt and <name>_dual_solution.txt into output_dir in
 * the reference's formats (cli.c:472-586), <name> being the file name up to
 * its first dot.  The solver reads the CP_AL_* environment variables the way
 * solve_lp_problem does.  The benchmark policy layer runs as in the reference
 * (cli.c:1031-1071, functions of include/cp_al_policy.h): with
 * CP_AL_UNIFIED_POLICY, CP_AL_FEATURE_AUTO_POLICY or
 * CP_AL_STRUCTURAL_TAIL_CUT set, the LP's features are computed, the
 * unified decision list and then the feature policy set their variables,
 * CP_AL_FEATURE_AUDIT_ONLY stops there, and the structural tail (when set)
 * runs the solve.  Not built: presolve (PSLP is not part of this build).
 */
#include "../../include/cp_al.h"
#include "../../include/cp_al_mps_parser.h"
#include "../../include/cp_al_policy.h"

#include <getopt.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>

namespace {

bool env_flag(const char *name) {
    const char *v = getenv(name);
    return v && v[0] && atoi(v) != 0;
}

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

/* cli.c:481-498: basename up to the first '.' */
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

void save_summary(const cp_al_result_t *r, const char *dir, const std::string &name) {
    const std::string p = out_path(dir, name, "_summary.txt");
    FILE *f = fopen(p.c_str(), "w");
    if (!f) {
        perror("Error opening summary file");
        return;
    }
    fprintf(f, "Termination Reason: %s\n", reason_name(r->termination_reason));
    /* no presolve lines: presolve_time is always 0 in this build (cli.c:545-552) */
    fprintf(f, "Precondition time (sec): %e\n", r->rescaling_time_sec);
    fprintf(f, "Runtime (sec): %e\n", r->cumulative_time_sec);
    fprintf(f, "Iterations Count: %d\n", r->total_count);
    fprintf(f, "Primal Objective Value: %e\n", r->primal_objective_value);
    fprintf(f, "Dual Objective Value: %e\n", r->dual_objective_value);
    fprintf(f, "Relative Primal Residual: %e\n", r->relative_primal_residual);
    fprintf(f, "Relative Dual Residual: %e\n", r->relative_dual_residual);
    fprintf(f, "Absolute Objective Gap: %e\n", r->objective_gap);
    fprintf(f, "Relative Objective Gap: %e\n", r->relative_objective_gap);
    fprintf(f, "Rows: %d\n", r->num_constraints);
    fprintf(f, "Columns: %d\n", r->num_variables);
    fprintf(f, "Nonzeros: %d\n", r->num_nonzeros);
    if (r->feasibility_polishing_time > 0.0) {
        fprintf(f, "Feasibility Polishing Time (sec): %e\n", r->feasibility_polishing_time);
        fprintf(f, "Feasibility Polishing Iteration Count: %d\n", r->feasibility_iteration);
    }
    fclose(f);
}

/* One command-line option: its long name, its short letter (0 if none),
 * whether it takes a value, what it sets, and its help line.  The names,
 * meanings and defaults are the reference command's (LP/CP_AL/src/cli.c:
 * 908-1005), which scripts call by name; the table, its order and the help
 * wording are this command's own. */
struct Option {
    const char *name;
    char letter;
    const char *value; /* name of the value in the help, nullptr for a switch */
    const char *help;
    /* returns false on a bad value (message already printed) */
    bool (*apply)(cp_al_parameters_t &, const char *);
};

bool set_norm(cp_al_parameters_t &p, const char *v) {
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

const Option kOptions[] = {
    {"eps_opt", 0, "TOL", "stop when the relative duality gap is below TOL (1e-4)",
     [](cp_al_parameters_t &p, const char *v) { return p.termination_criteria.eps_optimal_relative = atof(v), true; }},
    {"eps_feas", 0, "TOL", "and both relative residuals are below TOL (1e-4)",
     [](cp_al_parameters_t &p, const char *v) { return p.termination_criteria.eps_feasible_relative = atof(v), true; }},
    {"opt_norm", 0, "l2|linf", "norm of the residuals in that test (l2)", set_norm},
    {"iter_limit", 0, "N", "give up after N iterations (no limit)",
     [](cp_al_parameters_t &p, const char *v) { return p.termination_criteria.iteration_limit = atoi(v), true; }},
    {"time_limit", 0, "SEC", "give up after SEC seconds of wall time (3600)",
     [](cp_al_parameters_t &p, const char *v) { return p.termination_criteria.time_sec_limit = atof(v), true; }},
    {"eval_freq", 0, "N", "iterations between two evaluations of the stopping test (200, at least 3)",
     [](cp_al_parameters_t &p, const char *v) { return p.termination_evaluation_frequency = atoi(v), true; }},
    {"l_inf_ruiz_iter", 0, "N", "passes of Ruiz max-norm equilibration (10)",
     [](cp_al_parameters_t &p, const char *v) { return p.l_inf_ruiz_iterations = atoi(v), true; }},
    {"pock_chambolle_alpha", 0, "A", "exponent of the Pock-Chambolle scaling pass (1.0)",
     [](cp_al_parameters_t &p, const char *v) { return p.pock_chambolle_alpha = atof(v), true; }},
    {"no_pock_chambolle", 0, nullptr, "skip the Pock-Chambolle scaling pass",
     [](cp_al_parameters_t &p, const char *) { return p.has_pock_chambolle_alpha = false, true; }},
    {"no_bound_obj_rescaling", 0, nullptr, "skip the scaling of bounds and objective",
     [](cp_al_parameters_t &p, const char *) { return p.bound_objective_rescaling = false, true; }},
    {"sv_max_iter", 0, "N", "cap on power-iteration steps for the largest singular value (5000)",
     [](cp_al_parameters_t &p, const char *v) { return p.sv_max_iter = atoi(v), true; }},
    {"sv_tol", 0, "TOL", "power-iteration stopping tolerance (1e-4)",
     [](cp_al_parameters_t &p, const char *v) { return p.sv_tol = atof(v), true; }},
    {"feasibility_polishing", 'f', nullptr, "run the primal and dual polishing phases after the solve",
     [](cp_al_parameters_t &p, const char *) { return p.feasibility_polishing = true, true; }},
    {"eps_feas_polish", 0, "TOL", "residual target of the polishing phases (1e-6)",
     [](cp_al_parameters_t &p, const char *v) {
         return p.termination_criteria.eps_feas_polish_relative = atof(v), true;
     }},
    {"matrix_zero_tol", 0, "TOL", "treat constraint entries below TOL in magnitude as zero",
     [](cp_al_parameters_t &p, const char *v) { return p.matrix_zero_tol = atof(v), true; }},
    {"no_presolve", 0, nullptr, "accepted for compatibility; this build never presolves",
     [](cp_al_parameters_t &p, const char *) { return p.presolve = false, true; }},
    {"verbose", 'v', nullptr, "print progress while solving",
     [](cp_al_parameters_t &p, const char *) { return p.verbose = true, true; }},
};
constexpr int kNumOptions = sizeof(kOptions) / sizeof(kOptions[0]);
constexpr int kHelpCode = 'h';
constexpr int kFirstCode = 0x200; /* getopt return value of option i: kFirstCode + i */

void usage(const char *prog) {
    fprintf(stderr, "Usage: %s [OPTIONS] <mps_file> <output_dir>\n\n", prog);
    fprintf(stderr, "Solves the linear program in <mps_file> (MPS text, optionally gzip-compressed) on the GPU\n");
    fprintf(stderr, "and writes into <output_dir>, for an input named NAME.mps:\n");
    fprintf(stderr, "  NAME_summary.txt          status, iterations, objectives, residuals, times\n");
    fprintf(stderr, "  NAME_primal_solution.txt  one value of x per line\n");
    fprintf(stderr, "  NAME_dual_solution.txt    one value of y per line\n\n");
    fprintf(stderr, "Options (defaults in parentheses):\n");
    fprintf(stderr, "  -h, --help  show this text\n");
    for (const Option &o : kOptions) {
        char head[64];
        snprintf(head, sizeof head, "--%s%s%s", o.name, o.value ? " " : "", o.value ? o.value : "");
        if (o.letter)
            fprintf(stderr, "  -%c, %-34s %s\n", o.letter, head, o.help);
        else
            fprintf(stderr, "      %-34s %s\n", head, o.help);
    }
    fprintf(stderr, "\nCP_AL_* environment variables are read as the solver library reads them.\n");
    fprintf(stderr, "CP_AL_UNIFIED_POLICY, CP_AL_FEATURE_AUTO_POLICY and CP_AL_STRUCTURAL_TAIL_CUT switch on the\n"
                    "benchmark policy layer (features of the LP pick the settings; CP_AL_FEATURE_AUDIT_ONLY stops\n"
                    "after printing them).\n");
}

} // namespace

int main(int argc, char *argv[]) {
    cp_al_parameters_t params;
    set_default_parameters(&params);

    struct option long_options[kNumOptions + 2];
    std::string shorts = "h";
    long_options[0] = {"help", no_argument, nullptr, kHelpCode};
    for (int i = 0; i < kNumOptions; ++i) {
        const Option &o = kOptions[i];
        long_options[i + 1] = {o.name, o.value ? required_argument : no_argument, nullptr, kFirstCode + i};
        if (o.letter) shorts += o.letter;
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
    lp_problem_t *problem = read_mps_file(filename);
    if (!problem) {
        fprintf(stderr, "Failed to read or parse the file.\n");
        return 1;
    }
    /* the policy layer, in the reference's order (cli.c:1031-1071) */
    const bool need_stats = env_flag("CP_AL_UNIFIED_POLICY") || env_flag("CP_AL_FEATURE_AUTO_POLICY") ||
                            env_flag("CP_AL_STRUCTURAL_TAIL_CUT");
    cp_al_feature_stats_t stats;
    memset(&stats, 0, sizeof(stats));
    const clock_t policy_start = clock();
    if (need_stats) cp_al_feature_stats(problem, &stats);
    cp_al_unified_policy(need_stats ? &stats : nullptr);
    const bool feature_policy = env_flag("CP_AL_FEATURE_AUTO_POLICY");
    const bool tail = env_flag("CP_AL_STRUCTURAL_TAIL_CUT");
    const bool tail_pulse = env_flag("CP_AL_TAIL_ONLY_PULSE");
    if (need_stats)
        fprintf(stderr, "[feature-matrix-stats] computed=1 feature_policy=%d structural_tail=%d\n",
                feature_policy ? 1 : 0, tail ? 1 : 0);
    cp_al_feature_policy(problem, &params, need_stats ? &stats : nullptr);
    if (feature_policy)
        fprintf(stderr, "[feature-auto-policy-time] seconds=%.12g\n",
                (double)(clock() - policy_start) / CLOCKS_PER_SEC);
    if (env_flag("CP_AL_FEATURE_AUDIT_ONLY")) {
        lp_problem_free(problem);
        return 0;
    }
    cp_al_result_t *result =
        tail ? cp_al_structural_tail(problem, &params, &stats, tail_pulse ? 1 : 0) : solve_lp_problem(problem, &params);
    if (!result) {
        fprintf(stderr, "Solver failed.\n");
    } else {
        save_summary(result, output_dir, name);
        save_vector(result->primal_solution, problem->num_variables, output_dir, name, "_primal_solution.txt");
        save_vector(result->dual_solution, problem->num_constraints, output_dir, name, "_dual_solution.txt");
        cp_al_result_free(result);
    }
    lp_problem_free(problem);
    return 0;
}
