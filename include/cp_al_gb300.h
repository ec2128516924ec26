/*
 * cp_al_gb300.h -- entry points of libcp_al_gb300.so beyond the reference's
 * cp_al.h.
 *
 * The reference solver reads a second set of options from CP_AL_* environment
 * variables inside the library (LP/CP_AL/src/solver.cu:3141-3164, 3563-3579,
 * 2857-2966; LP/CP_AL/src/utils.cu:324-332, 370-372).  That plane is made
 * explicit here as cp_al_gb300_options_t.  solve_lp_problem() fills it from the
 * environment with cp_al_gb300_options_from_env(), so a caller of the
 * reference interface sees the same behaviour for the same environment.
 *
 * Only the options of the iteration itself are carried.  The reference's
 * benchmark controllers (alpha trial/pulse, adaptive lambda tiers, dynamic
 * evaluation frequency, Curtis-Reid scaling, diagnostics) are not.
 */
#pragma once

#include "cp_al_types.h"
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CP_AL_GB300_FP64 = 0,        /* plain FP64 everywhere */
    CP_AL_GB300_FP32_REFINE = 1  /* FP32 matrix/vectors, FP64 anchors and
                                    reductions, then an FP64 refinement phase */
} cp_al_gb300_precision_t;

typedef struct {
    /* --- the reference's CP_AL_* environment plane (same names, defaults) --- */
    double al_lambda;             /* CP_AL_LAMBDA, default 0.05 (solver.cu:3579) */
    int sigma_mode;               /* CP_AL_SIGMA_MODE!=0 or CP_AL_SIGMA set (solver.cu:3563-3564) */
    int sigma_set;                /* 1 when CP_AL_SIGMA gives sigma explicitly */
    double sigma;                 /* CP_AL_SIGMA */
    int sigma_adaptive;           /* CP_AL_SIGMA_ADAPTIVE; default 1 unless sigma_set (solver.cu:3158-3161) */
    double sigma_init_factor;     /* CP_AL_SIGMA_INIT_FACTOR, 6.0 */
    double sigma_min_factor;      /* CP_AL_SIGMA_MIN_FACTOR, 1e-4 */
    double sigma_max_factor;      /* CP_AL_SIGMA_MAX_FACTOR, 100 */
    double lambda_factor;         /* CP_AL_LAMBDA_FACTOR, 2.01 */
    int lambda_param_set;         /* 1 when CP_AL_LAMBDA_PARAM is given */
    double lambda_param;          /* CP_AL_LAMBDA_PARAM */
    double sigma_balance_gain;    /* CP_AL_SIGMA_BALANCE_GAIN, 0.15 */
    double sigma_i_smooth;        /* CP_AL_SIGMA_I_SMOOTH; NaN = restart_params.i_smooth */
    double sigma_kp;              /* CP_AL_SIGMA_KP; NaN = restart_params.k_p */
    double sigma_ki;              /* CP_AL_SIGMA_KI; NaN = restart_params.k_i */
    double sigma_kd;              /* CP_AL_SIGMA_KD; NaN = restart_params.k_d */
    double sigma_update_min;      /* CP_AL_SIGMA_UPDATE_MIN, 0.60 */
    double sigma_update_max;      /* CP_AL_SIGMA_UPDATE_MAX, 1.70 */
    double step_margin;           /* CP_AL_STEP_MARGIN, 0.998^2 */
    double restart_sufficient;    /* CP_AL_RESTART_SUFFICIENT; NaN = params */
    double restart_necessary;     /* CP_AL_RESTART_NECESSARY; NaN = params */
    double restart_artificial;    /* CP_AL_RESTART_ARTIFICIAL; NaN = params */
    int restart_select;           /* CP_AL_RESTART_SELECT (solver.cu:2749-2819): 0 = off; 1 = restart
                                     to the reflected Halpern iterate when its score wins; 2 = always
                                     to it; 3 = best of the current point, the reflected and the
                                     plain Halpern iterate */
    double restart_select_margin; /* CP_AL_RESTART_SELECT_MARGIN, 1.0 */
    int restart_select_min_iters; /* CP_AL_RESTART_SELECT_MIN_ITERS, 0 */
    int restart_select_threepoint;/* CP_AL_RESTART_SELECT_THREEPOINT, 0 (nonzero: mode 1 also scores
                                     the plain Halpern iterate) */
    double restart_select_min_time;/* CP_AL_RESTART_SELECT_MIN_TIME, 0.0 seconds */
    int cr_iterations;            /* Curtis-Reid passes before Ruiz (preconditioner.cu:162-270,
                                     403-425): CP_AL_CR_SCALING nonzero -> 20, CP_AL_CR_ITERS
                                     overrides; 0 = off */
    int cr_early_stop;            /* CP_AL_CR_EARLY_STOP: with 20 passes, stop after 5 when the
                                     largest change of a scaled entry's log is <= the threshold */
    double cr_early_stop_threshold; /* CP_AL_CR_EARLY_STOP_THRESHOLD, 0.1 */

    /* --- options of this implementation --- */
    int precision;                /* cp_al_gb300_precision_t */
    double fp32_switch_tol;       /* FP32 phase ends when rel KKT < this (default 1e-5) */
    int fp32_max_iterations;      /* FP32 phase iteration cap (default: none, -1) */
    int spmv_nnz_per_block;       /* row-block nonzero budget; 0 = automatic (single LP: by
                                     size; batch: autotuned, see batch_blocks_per_sm) */
    int device;                   /* CUDA device ordinal, -1 = current */
    int graph_blocks;             /* evaluation blocks per host check (default 1) */
    int timing;                   /* 1: time one primal and one dual launch per
                                     block with CUDA events (stats avg_*_ms) */
    int fp32_stall_evals;         /* FP32 phase ends after this many evaluations
                                     without halving its best KKT error (default 25) */
    int batch_blocks_per_sm;      /* batch: resident blocks per SM (2-4); 0 = autotune.
                                     When this or spmv_nnz_per_block is 0, the batch
                                     solver times each candidate schedule (row-block
                                     budget 1,024 / 2,048 x 2-4 blocks per SM) on a probe
                                     of the largest instances (200 iterations) and keeps
                                     the fastest, remembered per batch shape */
    int dual_panels;              /* rows with more nonzeros than the row-block budget in the
                                     iteration's A x product: 1 = by column panels (x staged in
                                     shared memory, one partial per row and panel), 0 = as
                                     row pieces, -1 (default) = panels when those rows hold at
                                     least 2^20 nonzeros */
    int panel_width;              /* columns per panel, a multiple of 4 up to 65536; 0 = 16384 */
    int primal_hot_rows;          /* with the panel path: the primal product A^T u takes the long
                                     rows' entries of u from a compact copy in shared memory (at
                                     most 1,536 long rows).  1 = in both phases, 0 = never (global
                                     memory like the rest), -1 (default) = in the FP64 phase only
                                     (measured faster there, slower in FP32) */
    int power_method;             /* sigma_max(A)^2 before the iteration: 0 = the reference's power
                                     iteration (LP/CP_AL/src/utils.cu:87-228, sv_max_iter, sv_tol);
                                     otherwise (default -1) the FP32_REFINE form uses Lanczos on
                                     A A^T with FP32 products -- at most min(128, sv_max_iter)
                                     steps, stopping when the largest Ritz value moves by less than
                                     1e-8 relative over 16 steps -- and the FP64 form the power
                                     iteration */
    int primal_staged;            /* the iteration's A^T u as a grid of one wave whose blocks walk
                                     the row blocks and copy the next one into shared memory with
                                     TMA bulk copies while they work on the current one: 1 = its
                                     matrix slice, 2 = also its rows' epilogue inputs, 0 = off
                                     (a block per row block, loads issued by the threads);
                                     -1 (default) = off.  Results are bit-identical in every mode */
    int infeasibility_detection;  /* nonzero: at every evaluation, test the iterates' displacement from
                                     the restart anchor as infeasibility certificates and stop with
                                     TERMINATION_REASON_PRIMAL_INFEASIBLE or _DUAL_INFEASIBLE (the ray
                                     fields of the result filled).  The reference has the formulas
                                     (LP/CP_AL/src/utils.cu:919-1029, 281-297) but never calls them:
                                     default 0, as there.  Single-LP solver only */
    double eps_infeasible;        /* tolerance of those tests (default 1e-8) */
    int persistent_loop;          /* small LPs: run the iteration, evaluation and restart loop inside one
                                     cooperative launch (grid barriers between the products) instead of a
                                     CUDA graph of per-iteration launches.  1 = when the problem allows it
                                     (row blocks of at most 1,024 nonzeros, no column panels, staged or
                                     hot-row product, restart target selection, infeasibility detection or
                                     timing); 0 or -1 (default) = never (measured no faster than the
                                     graph path with programmatic launches, which hides the launches) */
    int dual_fused_finish;        /* with the panel path: the group that writes a long row's last panel
                                     partial also sums the row's partials (fixed order) and runs its
                                     dual epilogue, instead of a separate launch.  1 = fused; 0 or -1
                                     (default) = a separate launch (measured twice as fast: the fused
                                     form fences and counts once per segment, 160,000 times on the
                                     large LP) */
    int device_transpose;         /* A^T built on the device (scatter, then a sort by row per column;
                                     exactly the host transpose) when no column has more than 2,048
                                     nonzeros: -1 (default) or 1 = so, 0 = on the host threads */

    /* --- benchmark controllers of the reference (off by default there and here; single-LP
     *     solver only) --- */
    int alpha_direct_pulse;       /* CP_AL_ALPHA_DIRECT_PULSE (LP/CP_AL/src/solver.cu:885-1032): at the
                                     first restart after 10,000 iterations with two recorded
                                     zero-alpha epochs (evaluation frequency 200, at least 400
                                     iterations left) the gate is evaluated once; when it passes, one
                                     evaluation block runs at alpha = 0.002 outside sigma mode, then
                                     alpha returns to 0 */
    int pulse_force;              /* CP_AL_DETERMINISTIC_PULSE_FORCE: the gate passes (it never passes
                                     otherwise, as in the reference) */
    int pulse_trace;              /* CP_AL_ALPHA_DIRECT_PULSE_TRACE (the pulse's stderr lines are printed
                                     whenever the pulse is enabled, as there) */
    int pulse_test_limit;         /* CP_AL_ALPHA_DIRECT_PULSE_TEST_TRAJECTORY_LIMIT: > 0 ends the solve
                                     (ITERATION_LIMIT) once the pulse is over and this many iterations
                                     are done */
    int sigma_trigger;            /* CP_AL_SIGMA_TRIGGER (solver.cu:1496-1527): outside sigma mode, at an
                                     evaluation after sigma_trigger_min_iters, switch sigma mode on
                                     (the sigma initialisation of solver.cu:3141-3164) and restart when
                                     rel. primal >= sigma_trigger_primal, rel. dual <=
                                     sigma_trigger_dual and their ratio >= sigma_trigger_ratio */
    int sigma_trigger_min_iters;  /* CP_AL_SIGMA_TRIGGER_MIN_ITERS, 200 */
    double sigma_trigger_primal;  /* CP_AL_SIGMA_TRIGGER_PRIMAL, 1e-2 */
    double sigma_trigger_dual;    /* CP_AL_SIGMA_TRIGGER_DUAL, 1e-6 */
    double sigma_trigger_ratio;   /* CP_AL_SIGMA_TRIGGER_RATIO, 1e6 */
    int dynamic_eval;             /* CP_AL_DYNAMIC_EVAL (solver.cu:1229-1255, 1529-1583): outside sigma mode,
                                     once the iterations reach dynamic_eval_min_iters, evaluation blocks
                                     of dynamic_eval_fast iterations instead of the evaluation frequency
                                     from the first evaluation whose residuals are one-sided (the smaller
                                     <= small_res, the larger >= large_res) or lopsided (ratio >= ratio,
                                     the larger >= large_res); the switch is kept */
    int dynamic_eval_fast;        /* CP_AL_DYNAMIC_EVAL_FAST, 50 (clamped to [3, evaluation frequency]) */
    double dynamic_eval_after_sec;/* CP_AL_DYNAMIC_EVAL_AFTER_SEC, -1: > 0 switches after this many seconds
                                     (unless Curtis-Reid stopped early) */
    int dynamic_eval_after_iters; /* CP_AL_DYNAMIC_EVAL_AFTER_ITERS, -1: > 0 switches after this many
                                     iterations (unless Curtis-Reid stopped early) */
    int dynamic_eval_min_iters;   /* CP_AL_DYNAMIC_EVAL_MIN_ITERS, 0 = the evaluation frequency (at least
                                     that) */
    double dynamic_eval_small_res;/* CP_AL_DYNAMIC_EVAL_SMALL_RES, 1e-6 */
    double dynamic_eval_large_res;/* CP_AL_DYNAMIC_EVAL_LARGE_RES, 1e-4 */
    double dynamic_eval_ratio;    /* CP_AL_DYNAMIC_EVAL_RATIO, 1e4 */
    int dynamic_eval_bootstrap_iters; /* CP_AL_DYNAMIC_EVAL_BOOTSTRAP_ITERS, 0: > 0 starts with short blocks
                                     and returns to the evaluation frequency at this many iterations unless
                                     the switch was taken */

    /* --- options of this implementation (continued) --- */
    int dual_concurrent;          /* with the panel path: the dual step's short-row launch and its
                                     long rows' panel launch run concurrently on two streams (also in
                                     the captured graphs).  1 = in both phases, -1 (default) = in the
                                     FP64 phase only (measured faster there, no faster in FP32), 0 =
                                     one after the other.  Results are bit-identical either way */
} cp_al_gb300_options_t;

/* Statistics of the last solve on this thread (for benchmarks and tests). */
typedef struct {
    double setup_sec;             /* device setup: scaling, power iteration, initial iterate */
    double loop_sec;              /* iteration loop (wall) */
    double total_sec;             /* whole call, including result download */
    double lambda_est;            /* power-iteration estimate of sigma_max(A)^2 */
    int power_iterations;
    int restarts;
    int fp32_iterations;          /* iterations run in the FP32 phase */
    int64_t kernel_launches;      /* kernels of this library launched by the loop */
    int64_t h2d_bytes;
    int64_t d2h_bytes;
    double primal_weight;
    double step_size;
    double al_penalty;
    /* timing == 1: mean duration of one primal / dual launch and of one
     * evaluation block, over the FP64 blocks and over the FP32 blocks */
    double avg_primal_ms;
    double avg_dual_ms;
    double avg_block_ms;
    int timed_blocks;
    double avg_primal32_ms;
    double avg_dual32_ms;
    double avg_block32_ms;
    int timed_blocks32;
    /* setup phases of the last solve (wall seconds): validation, transpose
     * and parameter checks on the host; row-block plans, allocation and
     * host-to-device copies; equilibration; power iteration */
    double prepare_sec;
    double upload_sec;
    double equilibration_sec;
    double power_sec;
    /* feasibility polishing of the last solve: termination_reason_t of its
     * primal and dual phases (-1: not run) */
    int polish_primal_status;
    int polish_dual_status;
    int cr_passes; /* Curtis-Reid passes run in the equilibration */
    int panel_rows; /* long rows the iteration's A x product runs by column panels (0: none) */
    int panels;     /* column panels of that product */
    /* timing == 1 with panels: the dual step's launch for the other rows and
     * its panel launch (the rest of avg_dual*_ms is the long rows' finishing
     * launch) */
    double avg_dual_rows_ms;
    double avg_dual_panels_ms;
    double avg_dual_rows32_ms;
    double avg_dual_panels32_ms;
    /* benchmark controllers: iteration at which the alpha pulse's positive
     * block started (-1: never), its gate (0 not evaluated, 1 passed, 2
     * rejected), iteration at which the sigma trigger fired (0: never) and
     * the dynamic evaluation frequency switched */
    int pulse_start_iteration;
    int pulse_gate;
    int sigma_trigger_iteration;
    int dynamic_eval_iteration;   /* iteration at which the blocks became dynamic_eval_fast long (0: never) */
    /* parts of upload_sec: the host-side row-block and panel plans, and the
     * device arena's allocation (the rest is copies and the device
     * transpose) */
    double upload_plan_sec;
    double upload_alloc_sec;
} cp_al_gb300_stats_t;

/* The reference defaults of every field, ignoring the environment. */
void cp_al_gb300_default_options(cp_al_gb300_options_t *opts);

/* Defaults, then each CP_AL_* variable that is set and parses overrides its
 * field exactly as the reference's getenv readers do. */
void cp_al_gb300_options_from_env(cp_al_gb300_options_t *opts);

/* Name of the first CP_AL_* environment switch that turns on a controller of
 * the reference this library does not implement -- adaptive lambda
 * (CP_AL_ADAPTIVE_LAMBDA, the race / auto CP_AL_LAMBDA_PROFILE values) or
 * the alpha rollback trial (CP_AL_ALPHA_ROLLBACK_TRIAL) -- or NULL.
 * solve_lp_problem
 * returns NULL with a message while one is set, instead of solving without
 * it.  Diagnostic and trace switches are ignored. */
const char *cp_al_gb300_unbuilt_switch(void);

/* solve_lp_problem with explicit options (opts == NULL -> from environment). */
cp_al_result_t *cp_al_gb300_solve(lp_problem_t *prob, const cp_al_parameters_t *params,
                                  const cp_al_gb300_options_t *opts);

/* Statistics of the last solve made by the calling thread. */
void cp_al_gb300_last_stats(cp_al_gb300_stats_t *out);

/* Last error message of the calling thread ("" if none). */
const char *cp_al_gb300_last_error(void);

/* --- device-resident solves (inputs already in HBM) ---------------------- */
/* ------------------------------------------------------------------ batch
 * Many independent LPs in one persistent launch: every resident CUDA block
 * takes the next instance from a device queue (largest first), runs the whole
 * solve -- equilibration, power iteration, iterations, restarts, termination
 * -- with its own controller state, and takes the next.  There is no
 * counterpart in the reference, whose benchmarks solve instances one at a
 * time through solve_lp_problem.  Every instance uses the same parameters and
 * options; precision CP_AL_GB300_FP32_REFINE runs each instance's FP32 phase
 * (FP64 anchors, evaluation and control) and then its FP64 refinement, as the
 * single-instance solver does. */
typedef struct {
    int instances;
    int optimal;          /* instances that reached OPTIMAL */
    int grid_blocks;      /* resident CUDA blocks of the launch */
    double host_prep_sec; /* validation, transposes, row-block plans, packing */
    double upload_sec;
    double kernel_sec;    /* the persistent launch (CUDA events) */
    double download_sec;
    double total_sec;
    double solves_per_sec; /* instances / total_sec */
    int iterations_p50, iterations_p99, iterations_max;
    long long total_iterations;
    long long device_bytes;
    int block_nnz;        /* schedule used: row-block nonzero budget */
    int blocks_per_sm;    /* schedule used: resident blocks per SM */
    double tune_sec;      /* time spent timing candidate schedules (0 when given or remembered) */
} cp_al_gb300_batch_stats_t;

/* Controller state of one instance at the end of its solve. */
typedef struct {
    double sigma;        /* sigma mode: the final sigma (0 otherwise) */
    double sigma_best;   /* sigma mode: the sigma of the best residual balance */
    double primal_weight;
    double step_size;
    double lambda_est;   /* sigma_max(A)^2 estimate of the scaled matrix */
    int restarts;
    int power_iterations;
    int fp32_iterations; /* iterations run in the FP32 phase */
} cp_al_gb300_instance_info_t;

/* Solves problems[0..count) and stores one result per instance in
 * results[0..count) (free each with cp_al_result_free); info (may be NULL)
 * receives count entries.  sigma0 (may be NULL) gives a per-instance initial
 * sigma for sigma mode (entries <= 0 keep the options' rule).  params / opts
 * may be NULL (defaults).  Returns 0, or -1 with nothing allocated (message
 * in cp_al_gb300_last_error). */
int cp_al_gb300_batch_solve(int count, lp_problem_t *const *problems, const cp_al_parameters_t *params,
                            const cp_al_gb300_options_t *opts, const double *sigma0, cp_al_result_t **results,
                            cp_al_gb300_instance_info_t *info, cp_al_gb300_batch_stats_t *stats);

/* Runs only the schedule autotuner of cp_al_gb300_batch_solve for this batch
 * (a no-op when opts fix the schedule or the batch shape was tuned before)
 * and reports the schedule in stats (block_nnz, blocks_per_sm, tune_sec); a
 * later cp_al_gb300_batch_solve of a batch of the same shape reuses it.
 * Returns 0, or -1 (message in cp_al_gb300_last_error). */
int cp_al_gb300_batch_tune(int count, lp_problem_t *const *problems, const cp_al_parameters_t *params,
                           const cp_al_gb300_options_t *opts, cp_al_gb300_batch_stats_t *stats);

typedef struct cp_al_gb300_session cp_al_gb300_session_t;

/* Uploads and prepares the problem (transpose, scaling, power iteration are
 * done by cp_al_gb300_session_solve, not here, so that a solve is complete). */
cp_al_gb300_session_t *cp_al_gb300_session_create(const lp_problem_t *prob, const cp_al_parameters_t *params,
                                                  const cp_al_gb300_options_t *opts);
/* Solves from the device-resident copy; the result stays on the device except
 * for the scalar summary written to *summary (vectors are not downloaded). */
int cp_al_gb300_session_solve(cp_al_gb300_session_t *s, cp_al_result_t *summary);
/* Starts a solve (equilibration, power iteration, initial iterate) without
 * iterating; iterations then run with cp_al_gb300_session_iterate. */
int cp_al_gb300_session_start(cp_al_gb300_session_t *s);
/* Runs `iterations` more iterations (rounded up to whole evaluation blocks)
 * of the solve in progress, or none if it has terminated for any reason but
 * the iteration limit; writes the scalar summary. */
int cp_al_gb300_session_iterate(cp_al_gb300_session_t *s, int iterations, cp_al_result_t *summary);
/* Downloads the unscaled solution of the last session solve. */
int cp_al_gb300_session_fetch(cp_al_gb300_session_t *s, double *primal, double *dual, double *reduced_cost);
void cp_al_gb300_session_free(cp_al_gb300_session_t *s);

/* Runs only the setup of a solve (equilibration and power iteration) and
 * returns the equilibrated constraint values in CSR order, the cumulative row
 * and column scales, {constraint-bound factor, objective factor} and the
 * power-iteration estimate of sigma_max(A)^2 (any output may be NULL). */
int cp_al_gb300_session_scaling(cp_al_gb300_session_t *s, double *scaled_values, double *row_scale,
                                double *col_scale, double *bound_obj_factors, double *lambda_est);

/* --- allocation-free evaluation ----------------------------------------- */

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory (an allocator owned by another framework, a memory pool that forbids
 * cudaMalloc while active, a loop where a cudaMalloc would synchronise the
 * device, a fixed device-memory budget): evaluates, for
 *     min c'x  s.t.  con_lb <= A x <= con_ub
 * and a candidate x, out[0] = ||A x - P(A x)||_2, out[1] = max |A x - P(A x)|
 * and out[2] = c'x, P the projection onto [con_lb, con_ub].  Every pointer is
 * a device pointer; A is CSR with m rows and n columns; stream may be NULL.
 * The call allocates nothing: its scratch is a fixed 2 MiB device array
 * inside the library, which every device that loads the library holds until
 * the process exits, so at most 524,288 rows are accepted (larger m returns
 * -1 with a message).  The first call on a device looks up that array's
 * device address (cudaGetSymbolAddress) and keeps it with the id of the
 * current context; a call under another context of that device (after
 * cudaDeviceReset, say) looks it up again.  Make the first call on each
 * device, and the first after a reset, before any stream capture.
 * All calls share the array, so calls that overlap on the GPU (different
 * streams, or several host threads) race; serialise them.  A NaN in the
 * inputs shows as NaN in out[0] and out[1].  The launch is asynchronous on
 * `stream`; returns 0, or -1 on a bad argument or CUDA error, with the
 * message in cp_al_gb300_last_error(). */
int cp_al_gb300_primal_kkt_noalloc(int m, int n, const int *row_ptr, const int *col_ind, const double *vals,
                                   const double *con_lb, const double *con_ub, const double *c, const double *x,
                                   double *out, void *stream);

#ifdef __cplusplus
} /* extern "C" */
#endif
