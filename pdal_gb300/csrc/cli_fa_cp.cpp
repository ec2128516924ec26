/*
 * cli_fa_cp.cpp -- the `fa_cp` command: drop-in for the FA_CP binary
 * (QP/FA_CP/src/cli.c:261-455) on top of libfa_cp_gb300.so.
 *
 *     fa_cp [OPTIONS] <mps_or_qps_file> <output_dir>
 *
 * Same options, defaults and exit codes; writes <name>_summary.txt,
 * <name>_primal_solution.txt and <name>_dual_solution.txt into output_dir in
 * the reference's formats (cli.c:112-170), <name> being the file name up to
 * its first dot, and the per-evaluation CSV of --trajectory_csv.  Not built:
 * feasibility polishing (-f prints a warning and solves without it).
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

void usage(const char *prog) {
    fprintf(stderr, "Usage: %s [OPTIONS] <mps_file> <output_dir>\n\n", prog);
    fprintf(stderr, "Arguments:\n");
    fprintf(stderr, "  <mps_file>               Path to the input problem in MPS format (.mps .QPS or .mps.gz).\n");
    fprintf(stderr, "  <output_dir>             Directory where output files will be saved. It will contain:\n");
    fprintf(stderr, "                             - <basename>_summary.txt\n");
    fprintf(stderr, "                             - <basename>_primal_solution.txt\n");
    fprintf(stderr, "                             - <basename>_dual_solution.txt\n\n");
    fprintf(stderr, "Options:\n");
    fprintf(stderr, "  -h, --help                          Display this help message.\n");
    fprintf(stderr, "  -v, --verbose <int>                 Verbosity level: 0=silent, 1=summary, 2=detailed "
                    "(default: 1).\n");
    fprintf(stderr, "      --time_limit <seconds>          Time limit in seconds (default: 3600.0).\n");
    fprintf(stderr, "      --iter_limit <iterations>       Iteration limit (default: %d).\n", INT32_MAX);
    fprintf(stderr, "      --eps_opt <tolerance>           Relative optimality tolerance (default: 1e-4).\n");
    fprintf(stderr, "      --eps_feas <tolerance>          Relative feasibility tolerance (default: 1e-4).\n");
    fprintf(stderr, "      --eps_infeas_detect <tolerance> Infeasibility detection tolerance (default: 1e-10).\n");
    fprintf(stderr, "      --l_inf_ruiz_iter <int>         Iterations for L-inf Ruiz rescaling (default: 10).\n");
    fprintf(stderr, "      --no_pock_chambolle             Disable Pock-Chambolle rescaling (default: enabled).\n");
    fprintf(stderr, "      --pock_chambolle_alpha <float>  Value for Pock-Chambolle alpha (default: 1.0).\n");
    fprintf(stderr, "      --no_bound_obj_rescaling        Disable bound objective rescaling (default: enabled).\n");
    fprintf(stderr, "      --no_al_qp                      Disable the AL primal-dual update and use the "
                    "non-augmented baseline branch.\n");
    fprintf(stderr, "      --al_sigma <float>              AL penalty parameter used in the full AL primal "
                    "subproblem (default: 0).\n");
    fprintf(stderr, "      --sigma_update <rule>           Restart-only sigma rule: fixed, residual, kkt, "
                    "displacement, progress, greedy, guarded, or balanced_guarded (default: guarded).\n");
    fprintf(stderr, "      --sigma_update_gain <float>     Log-domain damping gain for sigma updates "
                    "(default: 0.5).\n");
    fprintf(stderr, "      --sigma_clip_low <float>        Lower per-restart multiplicative clip (default: 0.6).\n");
    fprintf(stderr, "      --sigma_clip_high <float>       Upper per-restart multiplicative clip (default: 1.7).\n");
    fprintf(stderr, "      --sigma_min <float>             Minimum positive sigma for adaptive rules "
                    "(default: 1e-8).\n");
    fprintf(stderr, "      --sigma_max <float>             Maximum sigma for adaptive rules (default: 10).\n");
    fprintf(stderr, "      --sigma_rollback_tol <float>    Rollback to the best sigma if restart score worsens by "
                    "this factor (default: 1.25; nonpositive disables rollback).\n");
    fprintf(stderr, "      --sigma_zero_threshold <float>  Set guarded sigma to exactly zero below this value "
                    "(default: 1e-8).\n");
    fprintf(stderr, "      --sigma_activation_threshold <float> Primal bottleneck ratio needed to activate guarded "
                    "sigma (default: 2).\n");
    fprintf(stderr, "      --sigma_normal_motion_threshold <float> Minimum ||A dx||/||dx|| for guarded activation "
                    "(default: 1e-10).\n");
    fprintf(stderr, "      --sigma_activation_value <float> Positive sigma used when guarded mode activates from "
                    "zero; for balanced_guarded this is theta in sigma = theta * dual_step (default: 0.1).\n");
    fprintf(stderr, "      --eval_freq <int>               Termination evaluation frequency (default: 200).\n");
    fprintf(stderr, "      --trajectory_csv <path>         Write iteration trajectory CSV for plotting.\n");
    fprintf(stderr, "      --sv_max_iter <int>             Max iterations for singular value estimation "
                    "(default: 5000).\n");
    fprintf(stderr, "      --sv_tol <float>                Tolerance for singular value estimation (default: 1e-4).\n");
    fprintf(stderr, "      --opt_norm <norm_type>          Norm for optimality criteria: l2 or linf "
                    "(default: linf).\n");
}

} // namespace

int main(int argc, char *argv[]) {
    fa_cp_parameters_t params;
    set_default_parameters(&params);

    static struct option long_options[] = {{"help", no_argument, 0, 'h'},
                                           {"verbose", required_argument, 0, 'v'},
                                           {"time_limit", required_argument, 0, 1001},
                                           {"iter_limit", required_argument, 0, 1002},
                                           {"eps_opt", required_argument, 0, 1003},
                                           {"eps_feas", required_argument, 0, 1004},
                                           {"eps_infeas_detect", required_argument, 0, 1005},
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
                                           {"no_al_qp", no_argument, 0, 1015},
                                           {"al_sigma", required_argument, 0, 1016},
                                           {"trajectory_csv", required_argument, 0, 1017},
                                           {"sigma_update", required_argument, 0, 1018},
                                           {"sigma_update_gain", required_argument, 0, 1019},
                                           {"sigma_clip_low", required_argument, 0, 1020},
                                           {"sigma_clip_high", required_argument, 0, 1021},
                                           {"sigma_min", required_argument, 0, 1022},
                                           {"sigma_max", required_argument, 0, 1023},
                                           {"sigma_rollback_tol", required_argument, 0, 1024},
                                           {"sigma_zero_threshold", required_argument, 0, 1025},
                                           {"sigma_activation_threshold", required_argument, 0, 1026},
                                           {"sigma_normal_motion_threshold", required_argument, 0, 1027},
                                           {"sigma_activation_value", required_argument, 0, 1028},
                                           {0, 0, 0, 0}};
    int opt;
    while ((opt = getopt_long(argc, argv, "hv:fp", long_options, nullptr)) != -1) {
        switch (opt) {
        case 'h': usage(argv[0]); return 0;
        case 'v': params.verbose = atoi(optarg); break;
        case 1001: params.termination_criteria.time_sec_limit = atof(optarg); break;
        case 1002: params.termination_criteria.iteration_limit = atoi(optarg); break;
        case 1003: params.termination_criteria.eps_optimal_relative = atof(optarg); break;
        case 1004: params.termination_criteria.eps_feasible_relative = atof(optarg); break;
        case 1005: params.termination_criteria.eps_infeasible = atof(optarg); break;
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
        case 1015: params.use_al_qp = false; break;
        case 1016: params.al_sigma = atof(optarg); break;
        case 1017: params.trajectory_csv = optarg; break;
        case 1018:
            if (!parse_rule(optarg, &params.sigma_update_rule)) {
                fprintf(stderr, "Error: sigma_update must be fixed, residual, kkt, displacement, progress, greedy, "
                                "guarded, or balanced_guarded\n");
                return 1;
            }
            break;
        case 1019: params.sigma_update_gain = atof(optarg); break;
        case 1020: params.sigma_clip_low = atof(optarg); break;
        case 1021: params.sigma_clip_high = atof(optarg); break;
        case 1022: params.sigma_min = atof(optarg); break;
        case 1023: params.sigma_max = atof(optarg); break;
        case 1024: params.sigma_rollback_tol = atof(optarg); break;
        case 1025: params.sigma_zero_threshold = atof(optarg); break;
        case 1026: params.sigma_activation_threshold = atof(optarg); break;
        case 1027: params.sigma_normal_motion_threshold = atof(optarg); break;
        case 1028: params.sigma_activation_value = atof(optarg); break;
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
    if (params.feasibility_polishing) {
        fprintf(stderr, "Warning: feasibility polishing is not part of this build; solving without it.\n");
        params.feasibility_polishing = false;
    }
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
