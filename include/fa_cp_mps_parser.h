/*
 * fa_cp_mps_parser.h -- the MPS / QPS reader of libfa_cp_gb300.so.
 *
 * Replaces QP/FA_CP/include/mps_parser.h:23 (read_mps_file, implemented in
 * QP/FA_CP/src/mps_parser.c:371): same name, signature and result, including
 * the QUADOBJ (one triangle, mirrored) and QMATRIX (full) sections and the
 * empty low-rank component.  The problem is allocated with malloc and
 * released with qp_problem_free (fa_cp.h).  Returns NULL (message on stderr
 * and in fa_cp_gb300_last_error) when the file cannot be opened or parsed.
 */
#pragma once

#include "fa_cp_types.h"

#ifdef __cplusplus
extern "C" {
#endif

qp_problem_t *read_mps_file(const char *filename);

#ifdef __cplusplus
} /* extern "C" */
#endif
