/*
 * ref_solve.c -- runs the reference's own CP_AL (LP) or FA_CP (QP) solver
 * through its public C API on one problem file, and prints the result as one
 * JSON object with every double at full precision.
 *
 * Test infrastructure only: oracle/build.py (build_ref_solvers) compiles this
 * file against the reference's public headers (LP/CP_AL/include/cp_al.h or
 * QP/FA_CP/include/fa_cp.h) and links it with the reference's own solver
 * sources, compiled unmodified where they lie.  The reference's command-line
 * programs print their summaries with six digits (LP/CP_AL/src/cli.c:526-586,
 * QP/FA_CP/src/cli.c:120-170); parity at a relative objective of 1e-8 needs
 * the full double, hence this driver.  It calls exactly what the CLI calls
 * (set_default_parameters, create_*_problem, solve_*_problem; the CLI's
 * feature policies are inert unless their environment switches are set,
 * LP/CP_AL/src/cli.c:1032-1062).
 *
 *   ref_solve <problem.bin> [key=value ...]
 *
 * Problem file (little-endian, written by tests/golden/make_ref_solver_golden.py):
 *   char[8] "PDALPRB1"; int32 m, n, nnzA, has_Q, nnzQ, has_R, kR, nnzR;
 *   double obj_const; double c[n], var_lb[n], var_ub[n], con_lb[m], con_ub[m];
 *   A: int32 rp[m+1], ci[nnzA], double v[nnzA];
 *   Q (if has_Q): int32 rp[n+1], ci[nnzQ], double v[nnzQ];
 *   R (if has_R): int32 rp[kR+1], ci[nnzR], double v[nnzR].
 * Keys: eps, eps_opt, eps_feas, eps_polish, iter_limit, time_limit, ruiz,
 * pc_alpha, no_pc, no_bo, eval_freq, linf, sv_max_iter, sv_tol, reflection,
 * polish, artificial, sufficient, necessary, k_p, k_i, k_d, i_smooth,
 * verbose, out_x, out_y; QP only: sigma_rule, al_sigma, use_al_qp.
 */
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cuda_runtime_api.h>

#if defined(REF_QP)
#include "fa_cp.h"
typedef fa_cp_parameters_t params_t;
typedef fa_cp_result_t result_t;
#else
#include "cp_al.h"
typedef cp_al_parameters_t params_t;
typedef cp_al_result_t result_t;
#endif

static void die(const char *msg) {
    fprintf(stderr, "ref_solve: %s\n", msg);
    exit(2);
}

static void *read_exact(FILE *f, size_t bytes) {
    void *p = malloc(bytes > 0 ? bytes : 1);
    if (!p) die("out of memory");
    if (bytes > 0 && fread(p, 1, bytes, f) != bytes) die("truncated problem file");
    return p;
}

typedef struct {
    int rows;
    int nnz;
    int *rp, *ci;
    double *v;
} csr_t;

static void read_csr(FILE *f, int rows, int nnz, csr_t *out) {
    out->rows = rows;
    out->nnz = nnz;
    out->rp = (int *)read_exact(f, sizeof(int) * (size_t)(rows + 1));
    out->ci = (int *)read_exact(f, sizeof(int) * (size_t)nnz);
    out->v = (double *)read_exact(f, sizeof(double) * (size_t)nnz);
}

static void desc_of(const csr_t *a, int cols, matrix_desc_t *d) {
    memset(d, 0, sizeof(*d));
    d->m = a->rows;
    d->n = cols;
    d->fmt = matrix_csr;
    d->data.csr.nnz = a->nnz;
    d->data.csr.row_ptr = a->rp;
    d->data.csr.col_ind = a->ci;
    d->data.csr.vals = a->v;
}

static void put_double(const char *key, double v, int comma) {
    if (isnan(v))
        printf("\"%s\": \"nan\"", key);
    else if (isinf(v))
        printf("\"%s\": \"%s\"", key, v > 0 ? "inf" : "-inf");
    else
        printf("\"%s\": %.17g", key, v);
    if (comma) printf(", ");
}

static void dump(const char *path, const double *v, int len) {
    if (!path || !v) return;
    FILE *f = fopen(path, "wb");
    if (!f) die("cannot write a vector file");
    if (len > 0 && fwrite(v, sizeof(double), (size_t)len, f) != (size_t)len) die("short vector write");
    fclose(f);
}

int main(int argc, char **argv) {
    if (argc < 2) die("usage: ref_solve <problem.bin> [key=value ...]");
    FILE *f = fopen(argv[1], "rb");
    if (!f) die("cannot open the problem file");
    char magic[8];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "PDALPRB1", 8) != 0) die("not a problem file");
    int32_t hdr[8];
    if (fread(hdr, sizeof(int32_t), 8, f) != 8) die("truncated header");
    const int m = hdr[0], n = hdr[1], nnzA = hdr[2], has_q = hdr[3], nnzQ = hdr[4], has_r = hdr[5], kR = hdr[6],
              nnzR = hdr[7];
    double obj_const;
    if (fread(&obj_const, sizeof(double), 1, f) != 1) die("truncated header");
    double *c = (double *)read_exact(f, sizeof(double) * (size_t)n);
    double *vlb = (double *)read_exact(f, sizeof(double) * (size_t)n);
    double *vub = (double *)read_exact(f, sizeof(double) * (size_t)n);
    double *clb = (double *)read_exact(f, sizeof(double) * (size_t)m);
    double *cub = (double *)read_exact(f, sizeof(double) * (size_t)m);
    csr_t A, Q, R;
    read_csr(f, m, nnzA, &A);
    if (has_q) read_csr(f, n, nnzQ, &Q);
    if (has_r) read_csr(f, kR, nnzR, &R);
    fclose(f);

    params_t P;
    set_default_parameters(&P);
#if !defined(REF_QP)
    P.presolve = false; /* every reference benchmark runs with --no_presolve */
#endif
    const char *out_x = NULL, *out_y = NULL;
    for (int i = 2; i < argc; ++i) {
        char key[64];
        const char *eq = strchr(argv[i], '=');
        if (!eq || (size_t)(eq - argv[i]) >= sizeof(key)) die("arguments are key=value");
        memcpy(key, argv[i], (size_t)(eq - argv[i]));
        key[eq - argv[i]] = '\0';
        const char *val = eq + 1;
        const double d = atof(val);
        if (!strcmp(key, "eps")) {
            P.termination_criteria.eps_optimal_relative = d;
            P.termination_criteria.eps_feasible_relative = d;
        } else if (!strcmp(key, "eps_opt"))
            P.termination_criteria.eps_optimal_relative = d;
        else if (!strcmp(key, "eps_feas"))
            P.termination_criteria.eps_feasible_relative = d;
        else if (!strcmp(key, "eps_polish"))
            P.termination_criteria.eps_feas_polish_relative = d;
        else if (!strcmp(key, "iter_limit"))
            P.termination_criteria.iteration_limit = atoi(val);
        else if (!strcmp(key, "time_limit"))
            P.termination_criteria.time_sec_limit = d;
        else if (!strcmp(key, "ruiz"))
            P.l_inf_ruiz_iterations = atoi(val);
        else if (!strcmp(key, "pc_alpha"))
            P.pock_chambolle_alpha = d;
        else if (!strcmp(key, "no_pc"))
            P.has_pock_chambolle_alpha = atoi(val) == 0;
        else if (!strcmp(key, "no_bo"))
            P.bound_objective_rescaling = atoi(val) == 0;
        else if (!strcmp(key, "eval_freq"))
            P.termination_evaluation_frequency = atoi(val);
        else if (!strcmp(key, "linf"))
            P.optimality_norm = atoi(val) ? NORM_TYPE_L_INF : NORM_TYPE_L2;
        else if (!strcmp(key, "sv_max_iter"))
            P.sv_max_iter = atoi(val);
        else if (!strcmp(key, "sv_tol"))
            P.sv_tol = d;
        else if (!strcmp(key, "reflection"))
            P.reflection_coefficient = d;
        else if (!strcmp(key, "polish"))
            P.feasibility_polishing = atoi(val) != 0;
        else if (!strcmp(key, "artificial"))
            P.restart_params.artificial_restart_threshold = d;
        else if (!strcmp(key, "sufficient"))
            P.restart_params.sufficient_reduction_for_restart = d;
        else if (!strcmp(key, "necessary"))
            P.restart_params.necessary_reduction_for_restart = d;
        else if (!strcmp(key, "k_p"))
            P.restart_params.k_p = d;
        else if (!strcmp(key, "k_i"))
            P.restart_params.k_i = d;
        else if (!strcmp(key, "k_d"))
            P.restart_params.k_d = d;
        else if (!strcmp(key, "i_smooth"))
            P.restart_params.i_smooth = d;
#if defined(REF_QP)
        else if (!strcmp(key, "sigma_rule"))
            P.sigma_update_rule = (sigma_update_rule_t)atoi(val);
        else if (!strcmp(key, "al_sigma"))
            P.al_sigma = d;
        else if (!strcmp(key, "use_al_qp"))
            P.use_al_qp = atoi(val) != 0;
#endif
        else if (!strcmp(key, "verbose"))
            P.verbose = atoi(val);
        else if (!strcmp(key, "out_x"))
            out_x = val;
        else if (!strcmp(key, "out_y"))
            out_y = val;
        else
            die("unknown key");
    }

    matrix_desc_t dA;
    desc_of(&A, n, &dA);
    /* create the CUDA context before the clock starts: wall_sec is the solve */
    cudaFree(0);
    struct timespec t0, t1;
#if defined(REF_QP)
    matrix_desc_t dQ, dR;
    if (!has_q) {
        /* An empty n x n Q, not NULL: for a missing Q create_qp_problem keeps a
         * one-entry row pointer (QP/FA_CP/src/fa_cp.c:197) that the Ruiz pass
         * then reads n + 1 entries of (QP/FA_CP/src/preconditioner.c:167-170),
         * past its end.  An empty Q is the same problem without that read. */
        Q.rows = n;
        Q.nnz = 0;
        Q.rp = (int *)calloc((size_t)n + 1, sizeof(int));
        Q.ci = (int *)malloc(sizeof(int));
        Q.v = (double *)malloc(sizeof(double));
        if (!Q.rp || !Q.ci || !Q.v) die("out of memory");
    }
    desc_of(&Q, n, &dQ);
    if (has_r) desc_of(&R, n, &dR);
    qp_problem_t *prob = create_qp_problem(c, &dQ, has_r ? &dR : NULL, m > 0 ? &dA : NULL, clb, cub,
                                           vlb, vub, &obj_const);
    if (!prob) die("create_qp_problem failed");
    clock_gettime(CLOCK_MONOTONIC, &t0);
    result_t *r = solve_qp_problem(prob, &P);
    clock_gettime(CLOCK_MONOTONIC, &t1);
#else
    (void)Q;
    (void)R;
    (void)nnzQ;
    (void)nnzR;
    (void)kR;
    lp_problem_t *prob = create_lp_problem(c, &dA, clb, cub, vlb, vub, &obj_const);
    if (!prob) die("create_lp_problem failed");
    clock_gettime(CLOCK_MONOTONIC, &t0);
    result_t *r = solve_lp_problem(prob, &P);
    clock_gettime(CLOCK_MONOTONIC, &t1);
#endif
    if (!r) die("solve failed");
    const double wall = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    printf("{\"termination_reason\": %d, \"iterations\": %d, ", (int)r->termination_reason, r->total_count);
#if defined(REF_QP)
    printf("\"inner_iterations\": %d, \"sigma_update_count\": %d, ", r->total_inner_count, r->sigma_update_count);
    put_double("final_al_sigma", r->final_al_sigma, 1);
#endif
    put_double("primal_objective", r->primal_objective_value, 1);
    put_double("dual_objective", r->dual_objective_value, 1);
    put_double("relative_primal_residual", r->relative_primal_residual, 1);
    put_double("relative_dual_residual", r->relative_dual_residual, 1);
    put_double("absolute_primal_residual", r->absolute_primal_residual, 1);
    put_double("absolute_dual_residual", r->absolute_dual_residual, 1);
    put_double("objective_gap", r->objective_gap, 1);
    put_double("relative_objective_gap", r->relative_objective_gap, 1);
    put_double("rescaling_time_sec", r->rescaling_time_sec, 1);
    put_double("cumulative_time_sec", r->cumulative_time_sec, 1);
    put_double("feasibility_polishing_time", r->feasibility_polishing_time, 1);
    printf("\"feasibility_iteration\": %d, ", r->feasibility_iteration);
    put_double("wall_sec", wall, 0);
    printf("}\n");
    dump(out_x, r->primal_solution, n);
    dump(out_y, r->dual_solution, m);
#if defined(REF_QP)
    fa_cp_result_free(r);
    qp_problem_free(prob);
#else
    cp_al_result_free(r);
    lp_problem_free(prob);
#endif
    return 0;
}
