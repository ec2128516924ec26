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
 * solve_lp_problem does.  Not built: the feature / unified / structural-tail
 * policies the reference runs when CP_AL_UNIFIED_POLICY,
 * CP_AL_FEATURE_AUTO_POLICY, CP_AL_STRUCTURAL_TAIL_CUT or
 * CP_AL_FEATURE_AUDIT_ONLY is set (the command refuses to run with exit
 * code 2) and presolve (PSLP is not part of this build).
 */
#include "../../include/cp_al.h"
#include "../../include/cp_al_mps_parser.h"

#include <getopt.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
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

void usage(const char *prog) {
    fprintf(stderr, "Usage: %s [OPTIONS] <mps_file> <output_dir>\n\n", prog);
    fprintf(stderr, "Arguments:\n");
    fprintf(stderr, "  <mps_file>               Path to the input problem in MPS format (.mps or .mps.gz).\n");
    fprintf(stderr, "  <output_dir>             Directory where output files will be saved. It will contain:\n");
    fprintf(stderr, "                             - <basename>_summary.txt\n");
    fprintf(stderr, "                             - <basename>_primal_solution.txt\n");
    fprintf(stderr, "                             - <basename>_dual_solution.txt\n\n");
    fprintf(stderr, "Options:\n");
    fprintf(stderr, "  -h, --help                          Display this help message.\n");
    fprintf(stderr, "  -v, --verbose                       Enable verbose logging (default: false).\n");
    fprintf(stderr, "      --time_limit <seconds>          Time limit in seconds (default: 3600.0).\n");
    fprintf(stderr, "      --iter_limit <iterations>       Iteration limit (default: %d).\n", INT32_MAX);
    fprintf(stderr, "      --eps_opt <tolerance>           Relative optimality tolerance (default: 1e-4).\n");
    fprintf(stderr, "      --eps_feas <tolerance>          Relative feasibility tolerance (default: 1e-4).\n");
    fprintf(stderr, "      --l_inf_ruiz_iter <int>         Iterations for L-inf Ruiz rescaling (default: 10).\n");
    fprintf(stderr, "      --no_pock_chambolle             Disable Pock-Chambolle rescaling (default: enabled).\n");
    fprintf(stderr, "      --pock_chambolle_alpha <float>  Value for Pock-Chambolle alpha (default: 1.0).\n");
    fprintf(stderr, "      --no_bound_obj_rescaling        Disable bound objective rescaling (default: enabled).\n");
    fprintf(stderr, "      --eval_freq <int>               Termination evaluation frequency (default: 200).\n");
    fprintf(stderr, "      --sv_max_iter <int>             Max iterations for singular value estimation "
                    "(default: 5000).\n");
    fprintf(stderr, "      --sv_tol <float>                Tolerance for singular value estimation (default: 1e-4).\n");
    fprintf(stderr, "  -f  --feasibility_polishing         Enable feasibility use feasibility polishing "
                    "(default: false).\n");
    fprintf(stderr, "      --eps_feas_polish <tolerance>   Relative feasibility polish tolerance (default: 1e-6).\n");
    fprintf(stderr, "      --opt_norm <norm_type>          Norm for optimality criteria: l2 or linf (default: l2).\n");
    fprintf(stderr, "      --no_presolve                   Disable presolve (presolve is not built; accepted).\n");
    fprintf(stderr, "      --matrix_zero_tol <tolerance>.  Zero tolerance in constraint matrix.\n");
}

} // namespace

int main(int argc, char *argv[]) {
    cp_al_parameters_t params;
    set_default_parameters(&params);

    static struct option long_options[] = {{"help", no_argument, 0, 'h'},
                                           {"verbose", no_argument, 0, 'v'},
                                           {"time_limit", required_argument, 0, 1001},
                                           {"iter_limit", required_argument, 0, 1002},
                                           {"eps_opt", required_argument, 0, 1003},
                                           {"eps_feas", required_argument, 0, 1004},
                                           {"eps_feas_polish", required_argument, 0, 1006},
                                           {"feasibility_polishing", no_argument, 0, 'f'},
                                           {"l_inf_ruiz_iter", required_argument, 0, 1007},
                                           {"pock_chambolle_alpha", required_argument, 0, 1008},
                                           {"no_pock_chambolle", no_argument, 0, 1009},
                                           {"no_bound_obj_rescaling", no_argument, 0, 1010},
                                           {"sv_max_iter", required_argument, 0, 1011},
                                           {"sv_tol", required_argument, 0, 1012},
                                           {"eval_freq", required_argument, 0, 1013},
                                           {"opt_norm", required_argument, 0, 1014},
                                           {"no_presolve", no_argument, 0, 1015},
                                           {"matrix_zero_tol", required_argument, 0, 1016},
                                           {0, 0, 0, 0}};
    int opt;
    while ((opt = getopt_long(argc, argv, "hvfp", long_options, nullptr)) != -1) {
        switch (opt) {
        case 'h': usage(argv[0]); return 0;
        case 'v': params.verbose = true; break;
        case 1001: params.termination_criteria.time_sec_limit = atof(optarg); break;
        case 1002: params.termination_criteria.iteration_limit = atoi(optarg); break;
        case 1003: params.termination_criteria.eps_optimal_relative = atof(optarg); break;
        case 1004: params.termination_criteria.eps_feasible_relative = atof(optarg); break;
        case 1006: params.termination_criteria.eps_feas_polish_relative = atof(optarg); break;
        case 'f': params.feasibility_polishing = true; break;
        case 1007: params.l_inf_ruiz_iterations = atoi(optarg); break;
        case 1008: params.pock_chambolle_alpha = atof(optarg); break;
        case 1009: params.has_pock_chambolle_alpha = false; break;
        case 1010: params.bound_objective_rescaling = false; break;
        case 1011: params.sv_max_iter = atoi(optarg); break;
        case 1012: params.sv_tol = atof(optarg); break;
        case 1013: params.termination_evaluation_frequency = atoi(optarg); break;
        case 1014:
            if (strcmp(optarg, "l2") == 0) {
                params.optimality_norm = NORM_TYPE_L2;
            } else if (strcmp(optarg, "linf") == 0) {
                params.optimality_norm = NORM_TYPE_L_INF;
            } else {
                fprintf(stderr, "Error: opt_norm must be 'l2' or 'linf'\n");
                return 1;
            }
            break;
        case 1015: params.presolve = false; break;
        case 1016: params.matrix_zero_tol = atof(optarg); break;
        case '?': return 1;
        default: break;
        }
    }
    if (argc - optind != 2) {
        fprintf(stderr, "Error: You must specify an input file and an output directory.\n\n");
        usage(argv[0]);
        return 1;
    }
    const char *filename = argv[optind];
    const char *output_dir = argv[optind + 1];

    for (const char *flag : {"CP_AL_UNIFIED_POLICY", "CP_AL_FEATURE_AUTO_POLICY", "CP_AL_STRUCTURAL_TAIL_CUT",
                             "CP_AL_FEATURE_AUDIT_ONLY"}) {
        if (env_flag(flag)) {
            fprintf(stderr, "Error: %s is set, but the benchmark policy layer is not part of this build.\n", flag);
            return 2;
        }
    }
    const std::string name = instance_name(filename);
    lp_problem_t *problem = read_mps_file(filename);
    if (!problem) {
        fprintf(stderr, "Failed to read or parse the file.\n");
        return 1;
    }
    cp_al_result_t *result = solve_lp_problem(problem, &params);
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
