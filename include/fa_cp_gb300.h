/*
 * fa_cp_gb300.h -- additions of libfa_cp_gb300.so beyond the FA_CP interface
 * of fa_cp.h: per-call options instead of environment variables, statistics
 * of the last solve on the calling thread, and the last error message.
 *
 * None of these has a counterpart function in the reference; the options
 * replace the environment variables QP/FA_CP/src/fa_cp_core_op.cu:908-916 and
 * 1130-1169 read (FA_CP_RESTART_SELECT and its companions).
 */
#pragma once

#include "fa_cp_types.h"

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int device;        /* CUDA device ordinal; -1 keeps the current device */
    int blocks_per_sm; /* resident blocks of the persistent kernel per SM; 0 = as many as fit */
    /* restart target selection (QP/FA_CP/src/fa_cp_core_op.cu:1130-1169):
     * 0 restarts to the averaged iterate (default), 1 to the Halpern iterate
     * when its fixed-point score is below margin x the current one, 2 always
     * to the Halpern iterate */
    int restart_select;
    double restart_select_margin;
    int restart_select_min_iters;
    double restart_select_min_time;
    /* precision (options of this implementation): 0 = FP64 throughout (the
     * reference's arithmetic); 1 = FP32 iteration segments -- products,
     * projections, the BB inner solve and Halpern updates in FP32 with
     * (hi, lo) anchors and FP64 reductions, evaluation, restarts and
     * termination in FP64 -- until the relative KKT error is below
     * fp32_switch_tol or has not halved over fp32_stall_evals evaluations,
     * then FP64 from that iterate (the refinement phase) */
    int precision;
    double fp32_switch_tol;  /* default 1e-5 */
    int fp32_stall_evals;    /* default 25 */
    /* The persistent kernel's grid barriers give up after barrier_spin_limit
     * polls (0 = the default, about two seconds) and the solve then fails
     * with a message instead of hanging.  barrier_extra_arrivals makes every
     * barrier wait for that many blocks more than the launch has, so that
     * the bounded wait runs out: it exists to test that failure path, never
     * set it in a real solve. */
    long long barrier_spin_limit;
    int barrier_extra_arrivals;
} fa_cp_gb300_options_t;

typedef struct {
    double setup_sec;  /* equilibration, upload, power iterations */
    double loop_sec;   /* iterations and evaluations */
    double total_sec;
    double max_singular_value; /* power-iteration estimate of sigma_max(A) (scaled) */
    double q_norm;             /* estimate of the largest eigenvalue of the scaled Q */
    double q_nonconvexity;     /* estimate of its smallest eigenvalue (or 0) */
    int q_type;                /* quad_obj_type_t of the objective */
    int grid_blocks;           /* CUDA blocks of the persistent kernel */
    int restarts;
    int evaluations;
    int64_t kernel_launches;
    int64_t inner_iterations;  /* projected Barzilai-Borwein steps */
    double primal_weight;
    double step_size;
    double device_loop_ms;     /* device time of the iteration segments (CUDA events) */
    double equilibration_sec;  /* transposes on the host and equilibration on the device */
    double upload_sec;         /* plans, device arena and copies */
    double power_sec;          /* power iterations (sigma_max(A), eigenvalues of Q) */
    int power_iterations_a;
    int power_iterations_q;
    int fp32_iterations;       /* iterations run in FP32 segments (precision 1) */
    int polish_primal_status;  /* feasibility polishing: termination_reason_t of the primal and the */
    int polish_dual_status;    /* dual phase (7 = FEAS_POLISH_SUCCESS), -1 when not run */
} fa_cp_gb300_stats_t;

/* Defaults: current device, automatic grid and block budget, restart to the
 * averaged iterate. */
void fa_cp_gb300_default_options(fa_cp_gb300_options_t *opts);

/* The options solve_qp_problem uses: the defaults, overridden by the
 * environment variables the reference reads (FA_CP_RESTART_SELECT, with
 * FA_CP_RESTART_SELECT_LEGACY as fallback, FA_CP_RESTART_SELECT_MARGIN,
 * FA_CP_RESTART_SELECT_MIN_ITERS, FA_CP_RESTART_SELECT_MIN_TIME) and by
 * FA_CP_GB300_PRECISION ("fp64" or "fp32_refine", this implementation's). */
void fa_cp_gb300_options_from_env(fa_cp_gb300_options_t *opts);

/* solve_qp_problem with explicit options; params == NULL selects the
 * defaults, opts == NULL the default options.  NULL on error. */
fa_cp_result_t *fa_cp_gb300_solve(const qp_problem_t *prob, const fa_cp_parameters_t *params,
                                  const fa_cp_gb300_options_t *opts);

/* Statistics of the last solve on this thread. */
void fa_cp_gb300_last_stats(fa_cp_gb300_stats_t *stats);

/* The first `count` values of the C library's rand() sequence after
 * srand(seed), from the library's own generator: the start vectors of the
 * eigenvalue estimates of Q use it (QP/FA_CP/src/utils.cu:182-184 draws them
 * with rand() in a fresh process), without touching the process-wide
 * rand() state. */
void fa_cp_gb300_rand_sequence(unsigned seed, int count, int *out);

/* Message of the last failure on this thread ("" if none). */
const char *fa_cp_gb300_last_error(void);

/* The equilibration of a solve without the solve: column scales (n), row
 * scales (m) and the bound/objective factors {cbr, ovr} the solver computes
 * on the device before its first iteration (QP/FA_CP/src/preconditioner.c).
 * For tests and diagnostics; 0 on success, -1 on failure. */
int fa_cp_gb300_scaling(const qp_problem_t *prob, const fa_cp_parameters_t *params,
                        const fa_cp_gb300_options_t *opts, double *dcum, double *rcum, double *cbr_ovr);

#ifdef __cplusplus
} /* extern "C" */
#endif
