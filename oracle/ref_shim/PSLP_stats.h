/*
 * Empty stand-in for the presolve library's PSLP_stats.h, which
 * LP/CP_AL/include/cp_al_types.h:20 includes but no declaration the MPS
 * reader uses depends on.  Only the reference-reader build recipe
 * (oracle/build.py, build_ref) puts this directory on the include path.
 */
#pragma once
