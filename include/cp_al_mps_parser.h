/*
 * cp_al_mps_parser.h -- the MPS reader of libcp_al_gb300.so.
 *
 * Replaces LP/CP_AL/include/mps_parser.h:22 (read_mps_file, implemented in
 * LP/CP_AL/src/mps_parser.c:402): same name, signature and result.  The
 * problem is allocated with malloc and released with lp_problem_free
 * (cp_al.h).  Returns NULL (message on stderr and in cp_al_gb300_last_error)
 * when the file cannot be opened or parsed.  Files ending in ".gz" are read
 * through zlib.
 */
#pragma once

#include "cp_al_types.h"

#ifdef __cplusplus
extern "C" {
#endif

lp_problem_t *read_mps_file(const char *filename);

#ifdef __cplusplus
} /* extern "C" */
#endif
