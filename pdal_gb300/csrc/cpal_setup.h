/*
 * cpal_setup.h -- host-side setup shared by the single-instance and the
 * batched CP_AL solvers.
 */
#pragma once

#include "../../include/cp_al_gb300.h"
#include "../../include/cp_al_types.h"
#include "cpal_control.h"

#include <string>

namespace pdal {

/* Controller parameters of one solve: the options resolved against the
 * parameters, and the norms of the unscaled problem. */
CpalParams resolve_cpal_params(const cp_al_parameters_t &P, const cp_al_gb300_options_t &O, const lp_problem_t *prob);

/* The message cp_al_gb300_last_error returns on this thread (also printed). */
void set_last_error(const std::string &msg);
void clear_last_error();

} // namespace pdal
