/*
 * Presolve entry points of the reference's CP_AL library
 * (LP/CP_AL/internal/presolve.h:23-34) for the reference-solver build without
 * the PSLP library.  The reference's optimize() calls them only when
 * params->presolve is true (LP/CP_AL/src/solver.cu:1183-1194, 1726-1730);
 * the driver (ref_driver/ref_solve.c) always sets it false, so reaching one
 * of these is an error.
 */
#include <stdio.h>
#include <stdlib.h>

#include "presolve.h"

static void no_presolve(void) {
    fprintf(stderr, "reference build without PSLP: presolve is unavailable\n");
    exit(3);
}

cp_al_presolve_info_t *pslp_presolve(const lp_problem_t *original_prob, const cp_al_parameters_t *params) {
    (void)original_prob;
    (void)params;
    no_presolve();
    return NULL;
}

cp_al_result_t *create_result_from_presolve(const cp_al_presolve_info_t *info, const lp_problem_t *original_prob) {
    (void)info;
    (void)original_prob;
    no_presolve();
    return NULL;
}

const char *get_presolve_status_str(enum PresolveStatus_ status) {
    (void)status;
    return "presolve unavailable";
}

void pslp_postsolve(const cp_al_presolve_info_t *info, cp_al_result_t *reduced_result,
                    const lp_problem_t *original_prob) {
    (void)info;
    (void)reduced_result;
    (void)original_prob;
    no_presolve();
}

void cp_al_presolve_info_free(cp_al_presolve_info_t *info) { (void)info; }
