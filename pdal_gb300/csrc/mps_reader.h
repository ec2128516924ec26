/*
 * mps_reader.h -- free-format MPS / QPS reader shared by the LP and QP
 * libraries (read_mps_file in cp_al_api.cpp and fa_cp_api.cpp).
 *
 * It accepts exactly the dialect of the CP_AL and FA_CP readers
 * (LP/CP_AL/src/mps_parser.c:402-830, QP/FA_CP/src/mps_parser.c:371-740):
 * whitespace-separated tokens, at most six per line; a line of one token
 * starting with a letter is a section header; the first N row is the
 * objective; RHS, RANGES and BOUNDS take the set name as their first token;
 * QUADOBJ lists one triangle of Q (mirrored), QMATRIX all of it.  A file whose
 * name ends in ".gz" is read through zlib.
 */
#pragma once

#include <string>
#include <vector>

namespace pdal {
namespace mps {

struct Csr {
    std::vector<int> row_ptr;  /* rows + 1 */
    std::vector<int> col_ind;
    std::vector<double> val;
};

struct Model {
    int num_rows = 0;  /* constraints: E, L and G rows other than the objective */
    int num_cols = 0;
    std::vector<double> c, var_lb, var_ub, con_lb, con_ub;
    double objective_constant = 0.0; /* sign already applied for maximisation */
    bool maximize = false;
    Csr A;                      /* num_rows x num_cols, entries in file order within a row */
    Csr Q;                      /* num_cols x num_cols (quadratic sections only) */
};

/* Reads `path` (".gz": gzip).  quadratic: also read QUADOBJ / QMATRIX.  On
 * failure returns false with a message in err. */
bool read_file(const char *path, bool quadratic, Model &out, std::string &err);

/* Parses an in-memory file; buf[len] must be writable (the parser writes
 * token terminators into the buffer). */
bool parse_buffer(char *buf, size_t len, bool quadratic, Model &out, std::string &err);

}  // namespace mps
}  // namespace pdal
