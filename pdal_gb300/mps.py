"""MPS / QPS files: reading through the libraries' read_mps_file (the C
reader of the CP_AL and FA_CP interfaces) and writing.

    d = mps.read_lp("afiro.mps")          # LPData (libcp_al_gb300.so)
    q = mps.read_qp("qafiro.qps")         # QPData (libfa_cp_gb300.so)
    mps.write_lp(d, "copy.mps")
    mps.write_qp(q, "copy.qps")

The writer emits free-format MPS in the dialect the reader accepts: rows R0..,
columns C0.., numbers printed with repr() (strtod reads them back bit for
bit).  Row kinds: E for lb == ub, L for lb = -inf, G for ub = +inf, G with a
RANGES entry for two finite sides (ub is then read back as lb + (ub - lb),
which can differ from ub in the last bit), and L with RHS "inf" for a free
row.  The objective constant c0 is written as the RHS -c0 of the objective
row.  For a QP, Q is written to QUADOBJ as its lower triangle (the reader
mirrors it), so Q must be symmetric.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

from . import _native as N
from .lp import LPData

__all__ = ["read_lp", "read_qp", "write_lp", "write_qp", "lp_arrays", "qp_arrays"]


def _arr(ptr, n, dtype):
    if n <= 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def lp_arrays(p: N.LpProblem) -> dict:
    """Copies of every array of an lp_problem_t (keys follow its fields)."""
    n, m, nnz = p.num_variables, p.num_constraints, p.constraint_matrix_num_nonzeros
    return {
        "num_variables": n, "num_constraints": m, "nnz": nnz, "objective_constant": p.objective_constant,
        "c": _arr(p.objective_vector, n, np.float64), "var_lb": _arr(p.variable_lower_bound, n, np.float64),
        "var_ub": _arr(p.variable_upper_bound, n, np.float64),
        "con_lb": _arr(p.constraint_lower_bound, m, np.float64),
        "con_ub": _arr(p.constraint_upper_bound, m, np.float64),
        "row_ptr": _arr(p.constraint_matrix_row_pointers, m + 1, np.int32),
        "col_ind": _arr(p.constraint_matrix_col_indices, nnz, np.int32),
        "val": _arr(p.constraint_matrix_values, nnz, np.float64),
    }


def _component(c, rows, nnz):
    if not c:
        return None
    c = c.contents
    return (_arr(c.row_ptr, rows + 1, np.int32), _arr(c.col_ind, nnz, np.int32), _arr(c.val, nnz, np.float64))


def qp_arrays(p: N.QpProblem) -> dict:
    """Copies of every array of a qp_problem_t."""
    n, m = p.num_variables, p.num_constraints
    return {
        "num_variables": n, "num_constraints": m, "objective_constant": p.objective_constant,
        "num_rank_lowrank_obj": p.num_rank_lowrank_obj,
        "c": _arr(p.objective_vector, n, np.float64), "var_lb": _arr(p.variable_lower_bound, n, np.float64),
        "var_ub": _arr(p.variable_upper_bound, n, np.float64),
        "con_lb": _arr(p.constraint_lower_bound, m, np.float64),
        "con_ub": _arr(p.constraint_upper_bound, m, np.float64),
        "A": _component(p.constraint_matrix, m, p.constraint_matrix_num_nonzeros),
        "Q": _component(p.objective_sparse_matrix, n, p.objective_sparse_matrix_num_nonzeros),
        "lowrank_nnz": p.objective_lowrank_matrix_num_nonzeros,
    }


def _read(lib, path) -> C.POINTER:
    ptr = lib.read_mps_file(str(path).encode())
    if not ptr:
        raise ValueError(f"cannot read {path}: {N.last_error(lib)}")
    return ptr


def read_lp(path) -> LPData:
    """LP from an MPS file (gzip when the name ends in .gz)."""
    lib = N.load_lp()
    ptr = _read(lib, path)
    try:
        a = lp_arrays(ptr.contents)
    finally:
        lib.lp_problem_free(ptr)
    m, n = a["num_constraints"], a["num_variables"]
    return LPData(a["c"], (a["row_ptr"], a["col_ind"], a["val"], (m, n)), a["con_lb"], a["con_ub"], a["var_lb"],
                  a["var_ub"], c0=float(a["objective_constant"]))


def read_qp(path):
    """QP from an MPS / QPS file (QUADOBJ, QMATRIX)."""
    from .qp import QPData

    lib = N.load_qp()
    ptr = _read(lib, path)
    try:
        a = qp_arrays(ptr.contents)
    finally:
        lib.qp_problem_free(ptr)
    m, n = a["num_constraints"], a["num_variables"]
    A = (*a["A"], (m, n))
    Q = (*a["Q"], (n, n)) if a["Q"][1].size else None
    return QPData(a["c"], A, a["con_lb"], a["con_ub"], a["var_lb"], a["var_ub"], Q=Q,
                  c0=float(a["objective_constant"]))


# ---------------------------------------------------------------- writer

def _num(v: float) -> str:
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    return repr(float(v))


def _csr(M, shape):
    import scipy.sparse as sp

    if isinstance(M, tuple):
        rp, ci, v = M[:3]
        return sp.csr_matrix((np.asarray(v, np.float64), np.asarray(ci), np.asarray(rp)), shape=shape)
    return sp.csr_matrix(M, shape=shape)


def _write(path, name, c, c0, A, con_lb, con_ub, var_lb, var_ub, Q=None):
    m, n = A.shape
    A = A.tocsc()
    lines = [f"NAME {name}", "ROWS", " N OBJ"]
    kinds = []
    for i in range(m):
        lo, up = float(con_lb[i]), float(con_ub[i])
        if lo == up:
            k = "E"
        elif math.isinf(lo) and lo < 0:
            k = "L"
        elif math.isinf(up) and up > 0:
            k = "G"
        else:
            k = "G"
        kinds.append(k)
        lines.append(f" {k} R{i}")
    lines.append("COLUMNS")
    for j in range(n):
        s, e = A.indptr[j], A.indptr[j + 1]
        entries = []
        if c[j] != 0.0:
            entries.append(("OBJ", float(c[j])))
        entries += [(f"R{int(i)}", float(v)) for i, v in zip(A.indices[s:e], A.data[s:e])]
        if not entries:
            entries = [("OBJ", 0.0)]
        for r, v in entries:
            lines.append(f" C{j} {r} {_num(v)}")
    lines.append("RHS")
    if c0 != 0.0:
        lines.append(f" RHS OBJ {_num(-c0)}")
    ranges = []
    for i, k in enumerate(kinds):
        lo, up = float(con_lb[i]), float(con_ub[i])
        if k == "E":
            v = lo
        elif k == "L":
            v = up
        else:
            v = lo
        if math.isinf(lo) and math.isinf(up):
            v = math.inf  # free row: L with an infinite right-hand side
        if v != 0.0:
            lines.append(f" RHS R{i} {_num(v)}")
        if k == "G" and not math.isinf(up):
            ranges.append(f" RNG R{i} {_num(up - lo)}")
    if ranges:
        lines.append("RANGES")
        lines += ranges
    lines.append("BOUNDS")
    for j in range(n):
        lo, up = float(var_lb[j]), float(var_ub[j])
        if lo == up:
            lines.append(f" FX BND C{j} {_num(lo)}")
            continue
        if math.isinf(lo) and math.isinf(up):
            lines.append(f" FR BND C{j}")
            continue
        if math.isinf(lo):
            lines.append(f" MI BND C{j}")
        elif lo != 0.0:
            lines.append(f" LO BND C{j} {_num(lo)}")
        if not math.isinf(up):
            lines.append(f" UP BND C{j} {_num(up)}")
    if Q is not None and Q.nnz:
        lines.append("QUADOBJ")
        T = Q.tocoo()
        for i, j, v in zip(T.row, T.col, T.data):
            if i >= j and v != 0.0:
                lines.append(f" C{int(j)} C{int(i)} {_num(float(v))}")
    lines.append("ENDATA")
    text = "\n".join(lines) + "\n"
    path = Path(path)
    if path.suffix == ".gz":
        import gzip

        with gzip.open(path, "wt") as f:
            f.write(text)
    else:
        path.write_text(text)
    return path


def write_lp(d: LPData, path, name: str = "PDAL") -> Path:
    rp, ci, v, (m, n) = d.csr()
    A = _csr((rp, ci, v), (m, n))
    return _write(path, name, np.asarray(d.c, np.float64), float(d.c0), A, d.con_lb, d.con_ub, d.var_lb,
                  d.var_ub)


def write_qp(q, path, name: str = "PDAL") -> Path:
    if q.R is not None:
        raise ValueError("the MPS / QPS format has no low-rank objective term")
    m, n = q.dims()
    A = _csr(q.A, (m, n)) if q.A is not None else _csr((np.zeros(m + 1, np.int32), [], []), (m, n))
    Q = _csr(q.Q, (n, n)) if q.Q is not None else None
    lb = q.var_lb if q.var_lb is not None else np.full(n, -np.inf)
    ub = q.var_ub if q.var_ub is not None else np.full(n, np.inf)
    cl = q.con_lb if q.con_lb is not None else np.full(m, -np.inf)
    cu = q.con_ub if q.con_ub is not None else np.full(m, np.inf)
    return _write(path, name, np.asarray(q.c, np.float64), float(q.c0), A, cl, cu, lb, ub, Q)
