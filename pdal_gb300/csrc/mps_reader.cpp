/*
 * mps_reader.cpp -- the MPS / QPS reader behind read_mps_file.
 *
 * The whole file is read into one buffer (gzip through zlib), split into
 * lines and tokens in place, and parsed by one pass of a section state
 * machine with the rules of LP/CP_AL/src/mps_parser.c:402-830 and
 * QP/FA_CP/src/mps_parser.c:371-740.  Rules that are easy to get wrong, each
 * kept as the reference has it:
 *   - a line whose first character is '*', '\n' or '\r' is skipped; tokens
 *     split on space, tab, CR and LF, and only the first six count;
 *   - a line of exactly one token that starts with a letter is a section
 *     header; an unknown header (NAME, or OBJSENSE's "MAX" on a line of its
 *     own) switches to "no section", whose lines are ignored;
 *   - the first N row is the objective (with no N row, the first row of
 *     any type); the other N rows and rows of unknown type are dropped;
 *     a repeated row name keeps its first type;
 *   - COLUMNS: an odd token count starts with a column name, an even count
 *     continues the previous column; 'MARKER' lines are skipped;
 *     objective entries add up; entries of unknown rows are dropped; the
 *     matrix keeps every entry (duplicates are not summed) in file order;
 *   - RHS and RANGES pairs start at the second token (the first is the set
 *     name); an RHS on the objective row sets the constant to minus it;
 *   - RANGES: G rows get ub = lb + |R|, L rows lb = ub - |R|, E rows
 *     ub = rhs + R for R >= 0, else lb = rhs + R;
 *   - BOUNDS: LO UP FX FR MI PL BV on the column named by the third token,
 *     the value is the fourth (0 when absent); other types are ignored, and
 *     UP with a negative value leaves the lower bound alone;
 *   - QUADOBJ adds (i,j) and (j,i) for an off-diagonal entry, QMATRIX only
 *     (i,j); zero values and unknown columns are skipped;
 *   - maximisation negates c, Q and the objective constant.
 * Numbers are read with strtod (as atof does).  One deliberate difference:
 * a line of 4,096 or more characters is an error here, where the reference
 * reader prints an error and stops reading as if the file ended there.
 */
#include "mps_reader.h"

#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string_view>
#include <unordered_map>

#ifdef PDAL_HAVE_ZLIB
#include <zlib.h>
#endif

namespace pdal {
namespace mps {
namespace {

constexpr size_t kLineBuffer = 4096; /* the reference's line buffer, terminator included */
constexpr int kMaxTokens = 6;

enum class Sec { None, Rows, Columns, Rhs, Ranges, Bounds, ObjSense, QuadObj, QMatrix, EndData };

inline bool ascii_alpha(char ch) { return (ch >= 'A' && ch <= 'Z') || (ch >= 'a' && ch <= 'z'); }
inline bool delim(char ch) { return ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r'; }

using NameMap = std::unordered_map<std::string_view, int>;

struct Coo {
    std::vector<int> r, c;
    std::vector<double> v;
    void add(int i, int j, double x) {
        r.push_back(i);
        c.push_back(j);
        v.push_back(x);
    }
};

bool to_csr(int rows, const Coo &coo, Csr &out, std::string &err) {
    if (coo.v.size() > (size_t)INT_MAX) {
        err = "more than 2^31-1 matrix entries";
        return false;
    }
    out.row_ptr.assign((size_t)rows + 1, 0);
    for (int i : coo.r) ++out.row_ptr[(size_t)i + 1];
    for (int i = 0; i < rows; ++i) out.row_ptr[(size_t)i + 1] += out.row_ptr[i];
    std::vector<int> next(out.row_ptr.begin(), out.row_ptr.end() - 1);
    out.col_ind.resize(coo.v.size());
    out.val.resize(coo.v.size());
    for (size_t k = 0; k < coo.v.size(); ++k) {
        const int d = next[coo.r[k]]++;
        out.col_ind[d] = coo.c[k];
        out.val[d] = coo.v[k];
    }
    return true;
}

struct Parser {
    bool quadratic;
    Model &M;
    std::string &err;

    Sec sec = Sec::None;
    bool rows_done = false;
    std::vector<std::pair<char, std::string_view>> declared_rows;
    bool have_obj = false;
    std::string_view obj_name;
    NameMap rows, cols;
    std::vector<char> row_type;
    bool have_col = false;
    std::string_view col_name;
    double obj_constant = 0.0;
    bool maximize = false;
    Coo A, Q;

    Parser(bool q, Model &m, std::string &e) : quadratic(q), M(m), err(e) {}

    bool is_obj(std::string_view name) const { return have_obj && name == obj_name; }

    int row_of(std::string_view name) const {
        auto it = rows.find(name);
        return it == rows.end() ? -1 : it->second;
    }
    int col_of(std::string_view name) const {
        auto it = cols.find(name);
        return it == cols.end() ? -1 : it->second;
    }

    /* mps_parser.c finalize_rows: pick the objective, number the E/L/G rows,
     * default their sides from the row type. */
    void finalize_rows() {
        int obj = -1;
        for (size_t i = 0; i < declared_rows.size(); ++i)
            if (declared_rows[i].first == 'N') {
                obj = (int)i;
                break;
            }
        if (obj < 0 && !declared_rows.empty()) obj = 0;
        if (obj >= 0) {
            have_obj = true;
            obj_name = declared_rows[obj].second;
        }
        for (size_t i = 0; i < declared_rows.size(); ++i) {
            if ((int)i == obj) continue;
            const char t = declared_rows[i].first;
            if (t != 'E' && t != 'L' && t != 'G') continue;
            if (rows.emplace(declared_rows[i].second, (int)row_type.size()).second) row_type.push_back(t);
        }
        const size_t m = row_type.size();
        M.con_lb.resize(m);
        M.con_ub.resize(m);
        for (size_t i = 0; i < m; ++i) {
            const char t = row_type[i];
            M.con_lb[i] = t == 'L' ? -INFINITY : 0.0;
            M.con_ub[i] = t == 'G' ? INFINITY : 0.0;
        }
    }

    Sec header(std::string_view t) const {
        if (t == "ROWS") return Sec::Rows;
        if (t == "COLUMNS") return Sec::Columns;
        if (t == "RHS") return Sec::Rhs;
        if (t == "RANGES") return Sec::Ranges;
        if (t == "BOUNDS") return Sec::Bounds;
        if (t == "OBJSENSE") return Sec::ObjSense;
        if (quadratic && t == "QUADOBJ") return Sec::QuadObj;
        if (quadratic && t == "QMATRIX") return Sec::QMatrix;
        if (t == "ENDATA") return Sec::EndData;
        return Sec::None;
    }

    bool columns(char **tok, int n) {
        if (n < 2) return true;
        if (std::strcmp(tok[1], "'MARKER'") == 0) return true;
        int first = 0;
        if (n % 2 != 0) {
            col_name = tok[0];
            have_col = true;
            first = 1;
        } else if (!have_col) {
            err = "Column data found before any column name was defined.";
            return false;
        }
        auto ins = cols.emplace(col_name, (int)M.c.size());
        if (ins.second) {
            M.c.push_back(0.0);
            M.var_lb.push_back(0.0);
            M.var_ub.push_back(INFINITY);
        }
        const int j = ins.first->second;
        for (int k = first; k + 1 < n; k += 2) {
            const std::string_view row = tok[k];
            const double v = std::strtod(tok[k + 1], nullptr);
            if (is_obj(row)) {
                M.c[j] += v;
            } else {
                const int i = row_of(row);
                if (i >= 0) A.add(i, j, v);
            }
        }
        return true;
    }

    void rhs(char **tok, int n) {
        for (int k = 1; k + 1 < n; k += 2) {
            const std::string_view row = tok[k];
            const double v = std::strtod(tok[k + 1], nullptr);
            if (is_obj(row)) {
                obj_constant = -v;
                continue;
            }
            const int i = row_of(row);
            if (i < 0) continue;
            if (row_type[i] == 'L') {
                M.con_ub[i] = v;
            } else if (row_type[i] == 'G') {
                M.con_lb[i] = v;
            } else {
                M.con_lb[i] = v;
                M.con_ub[i] = v;
            }
        }
    }

    void ranges(char **tok, int n) {
        for (int k = 1; k + 1 < n; k += 2) {
            const double r = std::strtod(tok[k + 1], nullptr);
            const int i = row_of(tok[k]);
            if (i < 0) continue;
            const char t = row_type[i];
            const double base = t == 'L' ? M.con_ub[i] : M.con_lb[i];
            if (t == 'G')
                M.con_ub[i] = base + std::fabs(r);
            else if (t == 'L')
                M.con_lb[i] = base - std::fabs(r);
            else if (r >= 0)
                M.con_ub[i] = base + r;
            else
                M.con_lb[i] = base + r;
        }
    }

    void bounds(char **tok, int n) {
        if (n < 3) return;
        const double v = n > 3 ? std::strtod(tok[3], nullptr) : 0.0;
        const int j = col_of(tok[2]);
        if (j < 0) return;
        const std::string_view t = tok[0];
        double &lo = M.var_lb[j], &up = M.var_ub[j];
        if (t == "LO") {
            lo = v;
        } else if (t == "UP") {
            up = v;
        } else if (t == "FX") {
            lo = v;
            up = v;
        } else if (t == "FR") {
            lo = -INFINITY;
            up = INFINITY;
        } else if (t == "MI") {
            lo = -INFINITY;
        } else if (t == "PL") {
            up = INFINITY;
        } else if (t == "BV") {
            lo = 0.0;
            up = 1.0;
        }
    }

    void quad(char **tok, int n, bool mirror) {
        if (n < 3) return;
        const double v = std::strtod(tok[2], nullptr);
        if (v == 0.0) return;
        const int i = col_of(tok[0]), j = col_of(tok[1]);
        if (i < 0 || j < 0) {
            fprintf(stderr, "Warning: Variable '%s' or '%s' not found in COLUMNS. Skipping Q-entry.\n", tok[0],
                    tok[1]);
            return;
        }
        Q.add(i, j, v);
        if (i != j && mirror) Q.add(j, i, v);
    }

    bool line(char **tok, int n) {
        if (n == 1 && ascii_alpha(tok[0][0])) {
            const Sec next = header(tok[0]);
            if (sec == Sec::Rows && next != Sec::Rows && !rows_done) {
                finalize_rows();
                rows_done = true;
            }
            sec = next;
            return true;
        }
        switch (sec) {
        case Sec::ObjSense:
            if (std::strcmp(tok[0], "MAX") == 0 || std::strcmp(tok[0], "MAXIMIZE") == 0) maximize = true;
            break;
        case Sec::Rows:
            if (n >= 2) declared_rows.emplace_back(tok[0][0], std::string_view(tok[1]));
            break;
        case Sec::Columns:
            return columns(tok, n);
        case Sec::Rhs:
            rhs(tok, n);
            break;
        case Sec::Ranges:
            ranges(tok, n);
            break;
        case Sec::Bounds:
            bounds(tok, n);
            break;
        case Sec::QuadObj:
            quad(tok, n, true);
            break;
        case Sec::QMatrix:
            quad(tok, n, false);
            break;
        default:
            break;
        }
        return true;
    }

    bool finish() {
        M.num_cols = (int)M.c.size();
        M.num_rows = (int)row_type.size();
        M.con_lb.resize(M.num_rows);
        M.con_ub.resize(M.num_rows);
        M.maximize = maximize;
        M.objective_constant = maximize ? -obj_constant : obj_constant;
        if (maximize) {
            for (double &v : M.c) v = -v;
            for (double &v : Q.v) v = -v;
        }
        if (!to_csr(M.num_rows, A, M.A, err)) return false;
        if (quadratic && !to_csr(M.num_cols, Q, M.Q, err)) return false;
        return true;
    }
};

}  // namespace

bool parse_buffer(char *buf, size_t len, bool quadratic, Model &out, std::string &err) {
    out = Model{};
    Parser P(quadratic, out, err);
    buf[len] = '\0';
    size_t pos = 0, lineno = 0;
    char *tok[kMaxTokens];
    while (pos < len) {
        char *ln = buf + pos;
        const char *nl = static_cast<const char *>(std::memchr(ln, '\n', len - pos));
        const size_t L = nl ? (size_t)(nl - ln) + 1 : len - pos; /* newline included */
        ++lineno;
        if (L >= kLineBuffer) {
            err = "line " + std::to_string(lineno) + " is longer than " + std::to_string(kLineBuffer - 1) +
                  " characters";
            return false;
        }
        pos += L;
        if (ln[0] == '*' || ln[0] == '\n' || ln[0] == '\r') continue;
        /* the line is a C string to the reference: it ends at a NUL byte */
        int n = 0;
        size_t k = 0;
        while (k < L && ln[k] != '\0' && n < kMaxTokens) {
            while (k < L && delim(ln[k])) ++k;
            if (k >= L || ln[k] == '\0') break;
            tok[n++] = ln + k;
            while (k < L && ln[k] != '\0' && !delim(ln[k])) ++k;
            if (k < L && ln[k] != '\0') {
                ln[k] = '\0';
                ++k;
            }
        }
        if (n == 0) continue;
        if (!P.line(tok, n)) return false;
        if (P.sec == Sec::EndData) break;
    }
    return P.finish();
}

bool read_file(const char *path, bool quadratic, Model &out, std::string &err) {
    if (!path) {
        err = "no file name";
        return false;
    }
    std::vector<char> data;
    const size_t plen = std::strlen(path);
    const bool gz = plen > 3 && std::strcmp(path + plen - 3, ".gz") == 0;
    constexpr size_t kChunk = (size_t)4 << 20;
    if (gz) {
#ifdef PDAL_HAVE_ZLIB
        gzFile g = gzopen(path, "rb");
        if (!g) {
            err = std::string("Could not open file ") + path;
            return false;
        }
        for (;;) {
            const size_t at = data.size();
            data.resize(at + kChunk);
            const int got = gzread(g, data.data() + at, (unsigned)kChunk);
            if (got < 0) {
                int code = 0;
                err = std::string("gzip read error in ") + path + ": " + gzerror(g, &code);
                gzclose(g);
                return false;
            }
            data.resize(at + (size_t)got);
            if (got == 0) break;
        }
        gzclose(g);
#else
        err = std::string("cannot read ") + path + ": this build has no zlib";
        return false;
#endif
    } else {
        FILE *f = std::fopen(path, "rb");
        if (!f) {
            err = std::string("Could not open file ") + path;
            return false;
        }
        for (;;) {
            const size_t at = data.size();
            data.resize(at + kChunk);
            const size_t got = std::fread(data.data() + at, 1, kChunk, f);
            data.resize(at + got);
            if (got < kChunk) break;
        }
        const bool bad = std::ferror(f) != 0;
        std::fclose(f);
        if (bad) {
            err = std::string("read error in ") + path;
            return false;
        }
    }
    const size_t len = data.size();
    data.push_back('\0');
    return parse_buffer(data.data(), len, quadratic, out, err);
}

}  // namespace mps
}  // namespace pdal
