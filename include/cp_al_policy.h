/*
 * cp_al_policy.h -- the CP_AL command's benchmark policy layer, exported by
 * libcp_al_gb300.so and run by the `cp_al` command.
 *
 * The reference keeps this layer inside its command (LP/CP_AL/src/cli.c):
 * anonymous features of the parsed LP (52-214), the feature policy (216-399),
 * the unified decision list (401-470) and the structural tail, a two-phase
 * solve whose second phase is warm-started from the first and may run the
 * alpha pulse (588-833).  The policies only set CP_AL_* environment variables
 * and a few solver parameters; the solver reads the variables as
 * solve_lp_problem does.  The same switches turn them on:
 * CP_AL_UNIFIED_POLICY, CP_AL_FEATURE_AUTO_POLICY, CP_AL_STRUCTURAL_TAIL_CUT
 * (with CP_AL_TAIL_ONLY_PULSE), and the same stderr lines report them.
 */
#pragma once

#include "cp_al_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* LP/CP_AL/src/cli.c:53-67, same members in the same order. */
typedef struct {
    double coeff_log_range;            /* log10(max |a| / min |a|) over the finite nonzeros */
    double row_logmax_std;             /* std of log10(max |a|) over the nonempty rows */
    double col_logmax_std;             /* the same over the nonempty columns */
    double row_logspan_mean;           /* mean of log10(max |a| / min |a|) per nonempty row */
    double col_logspan_mean;
    double row_span2_fraction;         /* nonempty rows whose span is at least 2 decades */
    double col_span2_fraction;
    double row_nnz_cv;                 /* coefficient of variation of the stored entries per row */
    double col_nnz_cv;                 /* of the finite nonzero entries per column */
    double equality_fraction;          /* rows with finite, equal bounds */
    double two_sided_variable_fraction;/* variables with both bounds finite */
    double objective_density;          /* variables with c_j != 0 */
} cp_al_feature_stats_t;

/* LP/CP_AL/src/cli.c:90-214.  All zero when the problem has no rows, no
 * columns or no nonzeros.  Returns 0, or -1 for NULL arguments. */
int cp_al_feature_stats(const lp_problem_t *prob, cp_al_feature_stats_t *out);

/* LP/CP_AL/src/cli.c:401-470: with CP_AL_UNIFIED_POLICY set (non-zero),
 * choose the route from the features and set the variables the feature
 * policy and the structural tail read; prints the [unified-policy] line.
 * Returns the route's name, or NULL when the switch is off (or stats is
 * NULL, with the reference's error line). */
const char *cp_al_unified_policy(const cp_al_feature_stats_t *stats);

/* LP/CP_AL/src/cli.c:216-399: with CP_AL_FEATURE_AUTO_POLICY set, set the
 * evaluation frequency (200, or CP_AL_UNIFIED_EVAL_FREQ) and reflection
 * coefficient (1) in params and the CP_AL_* variables of the variant named by
 * CP_AL_FEATURE_POLICY_VARIANT (default safe0); prints the
 * [feature-auto-policy] line.  Returns 1 when applied, else 0. */
int cp_al_feature_policy(const lp_problem_t *prob, cp_al_parameters_t *params, const cp_al_feature_stats_t *stats);

/* LP/CP_AL/src/cli.c:607-831: the structural tail.  On LPs whose features
 * match its predicate (dense objective, uniform row scale, all or no
 * equality rows) a base solve gets 5% (all equality rows) or 75% of the time
 * limit; if it ends without OPTIMAL, a rescue solve warm-started from its
 * point gets the rest, with Curtis-Reid off, the feature policy re-applied,
 * evaluation frequency 200 and, with tail_pulse, the forced alpha pulse.
 * The result adds both solves' times and iteration counts.  Other LPs get one
 * solve.  prob keeps the warm start of a rescue.  The result is freed with
 * cp_al_result_free; NULL when a solve fails. */
cp_al_result_t *cp_al_structural_tail(lp_problem_t *prob, const cp_al_parameters_t *params,
                                      const cp_al_feature_stats_t *stats, int tail_pulse);

/* The solve the structural tail runs (default, or NULL: solve_lp_problem);
 * lets a test script the phases' results without a GPU. */
typedef cp_al_result_t *(*cp_al_solve_fn)(lp_problem_t *prob, const cp_al_parameters_t *params);
void cp_al_policy_set_solver(cp_al_solve_fn fn);

#ifdef __cplusplus
} /* extern "C" */
#endif
