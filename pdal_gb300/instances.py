"""Seeded synthetic LP/QP instances with the shapes and value distributions of
the benchmark workloads (numpy default_rng; same seed -> same arrays).

  random_lp(m, n, nnz_per_col)   random sparse LP with a planted feasible
                                 primal point and a dual-feasible point
                                 (2,000 x 5,000, 8 per column, is the small
                                 plain CP_AL case)
  zipf_lp(m, n, nnz)             large LP, Zipf(1.5) row lengths capped at
                                 20,000, entries N(0,1)*10^U[-3,3] per row
                                 and per column, 5% free variables
  batch_lps(count)               uneven batch, m log-uniform in [50, 5000]
  transport_lp(S, D)             min-cost transportation LP on a complete
                                 bipartite graph with arc capacities
  sparse_objective_lp(m, n)      feasibility-type LP: Zipf column lengths,
                                 0.5% of the costs nonzero
"""
from __future__ import annotations

import numpy as np

from .lp import LPData


def _csr_from_coo(rows, cols, vals, m, n):
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rp = np.zeros(m + 1, dtype=np.int64)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp)
    return rp.astype(np.int32), cols.astype(np.int32), vals.astype(np.float64)


def _distinct_rows_per_col(rng, m, n, k):
    """k distinct uniform rows for each of n columns (k may vary per column)."""
    k = np.broadcast_to(np.asarray(k), (n,)).astype(np.int64)
    kmax = int(k.max()) if n else 0
    kmax = min(kmax, m)
    k = np.minimum(k, m)
    rows = rng.integers(0, m, size=(n, kmax))
    for _ in range(64):
        srt = np.sort(rows, axis=1)
        dup = np.zeros_like(rows, dtype=bool)
        dup[:, 1:] = srt[:, 1:] == srt[:, :-1]
        bad = dup.any(axis=1)
        rows = srt
        if not bad.any():
            break
        rows[dup] = rng.integers(0, m, size=int(dup.sum()))
    mask = np.arange(kmax)[None, :] < k[:, None]
    cols = np.broadcast_to(np.arange(n)[:, None], rows.shape)
    return rows[mask], cols[mask]


def _plant(rng, A_csr, m, n, eq_rows, lb, ub, free_mask=None):
    """b from a feasible x0, c from a dual-feasible (y0, s) pair."""
    rp, ci, v = A_csr
    lo = np.where(np.isfinite(lb), lb, 0.0)
    hi = np.where(np.isfinite(ub), ub, lo + 5.0)
    x0 = lo + rng.random(n) * np.minimum(hi - lo, 5.0)
    Ax0 = np.zeros(m)
    row_of = np.repeat(np.arange(m), np.diff(rp))
    np.add.at(Ax0, row_of, v * x0[ci])
    slack = rng.random(m)
    is_eq = np.zeros(m, dtype=bool)
    is_eq[eq_rows] = True
    b = Ax0 + np.where(is_eq, 0.0, slack)
    con_lb = np.where(is_eq, b, -np.inf)
    con_ub = b.copy()
    y0 = rng.standard_normal(m)
    y0 = np.where(is_eq, y0, np.minimum(y0, 0.0))  # <= rows need y <= 0
    Aty = np.zeros(n)
    np.add.at(Aty, ci, v * y0[row_of])
    s = rng.random(n)
    if free_mask is not None:
        s = np.where(free_mask, 0.0, s)
    c = Aty + s
    return c, con_lb, con_ub


def random_lp(m: int = 2000, n: int = 5000, nnz_per_col=8, seed: int = 0, eq_fraction: float = 0.5,
              ub: float = 10.0) -> LPData:
    """Plain CP_AL benchmark LP: each column has nnz_per_col distinct uniform
    rows with N(0,1) entries; the first half of the rows are equalities, the
    rest <= rows; 0 <= x <= ub; b = A x0 + slack (x0 ~ U[0,5]); c = A'y0 + s
    with s ~ U[0,1] and y0 ~ N(0,1) clipped to <= 0 on the <= rows."""
    rng = np.random.default_rng(seed)
    rows, cols = _distinct_rows_per_col(rng, m, n, nnz_per_col)
    vals = rng.standard_normal(rows.shape[0])
    A = _csr_from_coo(rows, cols, vals, m, n)
    lb = np.zeros(n)
    ubv = np.full(n, float(ub))
    neq = int(round(m * eq_fraction))
    c, cl, cu = _plant(rng, A, m, n, np.arange(neq), lb, ubv)
    return LPData(c, (A[0], A[1], A[2], (m, n)), cl, cu, lb, ubv)


def infeasible_lp(kind: str, m: int = 300, n: int = 800, nnz_per_col: int = 6, seed: int = 0) -> LPData:
    """random_lp made infeasible.  kind "primal": row 0 (an equality) is
    asked to exceed its largest value over the variable box (10 * the sum of
    its positive entries) by 1, so no x satisfies it.  kind "dual": one more
    variable, 0 <= x_new unbounded above, with cost -1 and negative entries in
    three <= rows only, so x_new -> infinity stays feasible and the objective
    is unbounded below."""
    d = random_lp(m, n, nnz_per_col, seed=seed)
    rp, ci, v, _ = d.csr()
    if kind == "primal":
        row0 = v[rp[0]:rp[1]]
        top = 10.0 * np.maximum(row0, 0.0).sum() + 1.0
        d.con_lb = d.con_lb.copy()
        d.con_ub = d.con_ub.copy()
        d.con_lb[0], d.con_ub[0] = top, np.inf
        return d
    if kind != "dual":
        raise ValueError(kind)
    rng = np.random.default_rng(seed + 1)
    le_rows = np.flatnonzero(np.isinf(d.con_lb))
    pick = np.sort(rng.choice(le_rows, 3, replace=False))
    rows = np.concatenate([np.repeat(np.arange(m), np.diff(rp)), pick])
    cols = np.concatenate([ci, np.full(3, n)])
    vals = np.concatenate([v, -rng.uniform(0.5, 1.5, 3)])
    A = _csr_from_coo(rows, cols, vals, m, n + 1)
    return LPData(np.append(d.c, -1.0), (A[0], A[1], A[2], (m, n + 1)), d.con_lb, d.con_ub, np.append(d.var_lb, 0.0),
                  np.append(d.var_ub, np.inf))


def zipf_lp(m: int = 1_000_000, n: int = 2_000_000, nnz: int = 20_000_000, seed: int = 1000,
            zipf_a: float = 1.5, max_row: int = 20_000, free_fraction: float = 0.05) -> LPData:
    """Large badly scaled LP: row lengths Zipf(zipf_a) capped at max_row and
    rescaled to about nnz in total, uniform columns, values
    N(0,1) * 10^U[-3,3] (row factor) * 10^U[-3,3] (column factor); bounds
    0 <= x <= U[1,100] with free_fraction free variables; b and c planted."""
    rng = np.random.default_rng(seed)
    z = rng.zipf(zipf_a, size=m).astype(np.float64)
    cap = min(max_row, n)
    # scale f so that sum(min(max(1, round(z f)), cap)) ~ nnz: the heaviest
    # rows reach the cap, the bulk keeps the power-law shape
    lo, hi = 1e-9, 1.0
    for _ in range(60):
        f = np.sqrt(lo * hi)
        tot = np.minimum(np.maximum(1.0, np.round(z * f)), cap).sum()
        lo, hi = (f, hi) if tot < nnz else (lo, f)
    lens = np.minimum(np.maximum(1.0, np.round(z * np.sqrt(lo * hi))), cap).astype(np.int64)
    total = int(lens.sum())
    rows = np.repeat(np.arange(m, dtype=np.int64), lens)
    cols = rng.integers(0, n, size=total, dtype=np.int64)
    key = rows * n + cols
    key.sort()
    key = key[np.concatenate(([True], key[1:] != key[:-1]))]
    rows, cols = key // n, key % n
    rf = 10.0 ** rng.uniform(-3, 3, size=m)
    cf = 10.0 ** rng.uniform(-3, 3, size=n)
    vals = rng.standard_normal(rows.shape[0]) * rf[rows] * cf[cols]
    rp = np.zeros(m + 1, dtype=np.int64)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    A = (rp, cols.astype(np.int32), vals)
    lb = np.zeros(n)
    ubv = rng.uniform(1, 100, size=n)
    free = rng.random(n) < free_fraction
    lb[free] = -np.inf
    ubv[free] = np.inf
    c, cl, cu = _plant(rng, A, m, n, np.arange(m // 2), lb, ubv, free_mask=free)
    return LPData(c, (A[0], A[1], A[2], (m, n)), cl, cu, lb, ubv)


def sparse_objective_lp(m: int = 3000, n: int = 6000, nnz: int = 40_000, seed: int = 5000, priced: float = 0.005,
                        max_col: int = 600) -> LPData:
    """Feasibility-type LP: column lengths Zipf(1.5) capped at max_col and
    rescaled to about nnz in total (a few dense columns, most with one or two
    entries), values N(0,1), 0 <= x <= 10, half the rows equalities, b
    planted, and only a `priced` fraction of the costs nonzero."""
    rng = np.random.default_rng(seed)
    z = rng.zipf(1.5, size=n).astype(np.float64)
    cap = min(max_col, m)
    lo, hi = 1e-9, 1.0
    for _ in range(60):
        f = np.sqrt(lo * hi)
        tot = np.minimum(np.maximum(1.0, np.round(z * f)), cap).sum()
        lo, hi = (f, hi) if tot < nnz else (lo, f)
    k = np.minimum(np.maximum(1.0, np.round(z * np.sqrt(lo * hi))), cap).astype(np.int64)
    rows, cols = _distinct_rows_per_col(rng, m, n, k)
    vals = rng.standard_normal(rows.shape[0])
    A = _csr_from_coo(rows, cols, vals, m, n)
    lb = np.zeros(n)
    ubv = np.full(n, 10.0)
    c, cl, cu = _plant(rng, A, m, n, np.arange(m // 2), lb, ubv)
    c = np.where(rng.random(n) < priced, c, 0.0)
    return LPData(c, (A[0], A[1], A[2], (m, n)), cl, cu, lb, ubv)


def batch_lps(count: int = 4096, seed: int = 3000, m_range=(50, 5000)) -> list[LPData]:
    """Uneven batch: m log-uniform in m_range, n = round(m * U[2,3]),
    3-20 nonzeros per column, otherwise as random_lp."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        m = int(round(np.exp(rng.uniform(np.log(m_range[0]), np.log(m_range[1])))))
        n = int(round(m * rng.uniform(2, 3)))
        k = rng.integers(3, 21, size=n)
        out.append(_random_lp_k(m, n, k, seed * 100003 + i))
    return out


def _random_lp_k(m, n, k, seed):
    rng = np.random.default_rng(seed)
    rows, cols = _distinct_rows_per_col(rng, m, n, k)
    vals = rng.standard_normal(rows.shape[0])
    A = _csr_from_coo(rows, cols, vals, m, n)
    lb = np.zeros(n)
    ubv = np.full(n, 10.0)
    c, cl, cu = _plant(rng, A, m, n, np.arange(m // 2), lb, ubv)
    return LPData(c, (A[0], A[1], A[2], (m, n)), cl, cu, lb, ubv)


def transport_lp(supplies: int = 200, demands: int = 200, seed: int = 4000, base_costs=None,
                 perturb: float = 0.2) -> LPData:
    """min sum c_ij x_ij over a complete bipartite graph: supply rows
    sum_j x_ij = s_i, demand rows sum_i x_ij = d_j (totals rebalanced to be
    equal), 0 <= x_ij <= cap_ij with cap ~ U[20,200]; costs
    base_ij * (1 + perturb * N(0,1)) with base ~ U[1,100]."""
    rng = np.random.default_rng(seed)
    S, D = supplies, demands
    n = S * D
    if base_costs is None:
        base_costs = np.random.default_rng(4000).uniform(1, 100, size=n)
    cost = base_costs * (1.0 + perturb * rng.standard_normal(n))
    s = rng.uniform(10, 100, size=S)
    d = rng.uniform(10, 100, size=D)
    d *= s.sum() / d.sum()
    cap = rng.uniform(20, 200, size=n)
    arc = np.arange(n)
    i = arc // D
    j = arc % D
    rows = np.concatenate([i, S + j])
    cols = np.concatenate([arc, arc])
    vals = np.ones(2 * n)
    A = _csr_from_coo(rows, cols, vals, S + D, n)
    b = np.concatenate([s, d])
    return LPData(cost, (A[0], A[1], A[2], (S + D, n)), b.copy(), b.copy(), np.zeros(n), cap)


def docs_example_lp() -> LPData:
    """The 3x2 example of the reference's C API documentation
    (LP/CP_AL/docs/C_API.md:41-89): min x1 + x2 s.t. x1 + 2 x2 = 5, x2 <= 2,
    3 x1 + 2 x2 <= 8, x free.  Optimum x = (1, 2), objective 3."""
    rp = np.array([0, 2, 3, 5], dtype=np.int32)
    ci = np.array([0, 1, 1, 0, 1], dtype=np.int32)
    v = np.array([1.0, 2.0, 1.0, 3.0, 2.0])
    return LPData(np.array([1.0, 1.0]), (rp, ci, v, (3, 2)), np.array([5.0, -np.inf, -np.inf]),
                  np.array([5.0, 2.0, 8.0]), np.full(2, -np.inf), np.full(2, np.inf))


def planted_qp(n: int = 200_000, m: int = 100_000, nnz_per_col: int = 10, b_rows: int = 50_000,
               b_nnz_per_row: int = 5, seed: int = 2000, eq_fraction: float = 0.5, diag_lo: float = 1e-4,
               q_form: str = "sparse"):
    """Convex QP with a known optimum (the FA_CP workload at its default sizes):
    A has nnz_per_col N(0,1) entries per column; Q = B'B + diag(U[diag_lo, 1])
    with B b_rows x n at b_nnz_per_row N(0,1) entries per row; box
    -U[0,10] <= x <= U[0,10].  x* lies strictly inside the box, y* ~ N(0,1)
    on equality rows and -|N(0,1)| or 0 on the <= rows (active rows get
    u = (Ax*)_i, the others a positive slack), and c = -Q x* + A'y*, so x*
    satisfies the KKT conditions exactly and f* = 1/2 x*'Qx* + c'x*.

    q_form "sparse" stores Q explicitly (SPARSE_Q path); "lowrank" passes
    R = B and the diagonal as a separate Q (LOW_RANK_PLUS_SPARSE_Q path).
    Returns (QPData, x_star, f_star)."""
    from .qp import QPData

    rng = np.random.default_rng(seed)
    rows, cols = _distinct_rows_per_col(rng, m, n, nnz_per_col)
    A = _csr_from_coo(rows, cols, rng.standard_normal(rows.shape[0]), m, n)
    br = np.repeat(np.arange(b_rows), b_nnz_per_row)
    bc = rng.integers(0, n, size=br.shape[0])
    key = br.astype(np.int64) * n + bc
    key = np.unique(key)
    br, bc = (key // n).astype(np.int64), (key % n).astype(np.int64)
    B = _csr_from_coo(br, bc, rng.standard_normal(br.shape[0]), b_rows, n)
    dq = diag_lo + rng.random(n) * (1.0 - diag_lo)
    lo = -10.0 * rng.random(n)
    hi = 10.0 * rng.random(n)
    x = lo + (0.1 + 0.8 * rng.random(n)) * (hi - lo)

    def csr_mv(M, v, nr):
        rp, ci, vals = M
        out = np.zeros(nr)
        np.add.at(out, np.repeat(np.arange(nr), np.diff(rp)), vals * v[ci])
        return out

    def csr_tmv(M, v, nr, nc):
        rp, ci, vals = M
        out = np.zeros(nc)
        np.add.at(out, ci, vals * v[np.repeat(np.arange(nr), np.diff(rp))])
        return out

    Bx = csr_mv(B, x, b_rows)
    Qx = csr_tmv(B, Bx, b_rows, n) + dq * x
    Ax = csr_mv(A, x, m)
    is_eq = rng.random(m) < eq_fraction
    active = rng.random(m) < 0.5
    y = rng.standard_normal(m)
    y = np.where(is_eq, y, np.where(active, -np.abs(y), 0.0))
    con_ub = Ax + np.where(is_eq | active, 0.0, rng.random(m))
    con_lb = np.where(is_eq, Ax, -np.inf)
    c = -Qx + csr_tmv(A, y, m, n)
    f = 0.5 * float(x @ Qx) + float(c @ x)
    Acsr = (A[0], A[1], A[2], (m, n))
    if q_form == "sparse":
        data = QPData(c=c, A=Acsr, con_lb=con_lb, con_ub=con_ub, var_lb=lo, var_ub=hi, Q=_gram_plus_diag(B, dq, n))
    elif q_form == "lowrank":
        diag = (np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), dq, (n, n))
        data = QPData(c=c, A=Acsr, con_lb=con_lb, con_ub=con_ub, var_lb=lo, var_ub=hi, Q=diag,
                      R=(B[0], B[1], B[2], (b_rows, n)))
    else:
        raise ValueError(q_form)
    return data, x, f


def _gram_plus_diag(B, dq, n):
    """CSR of B'B + diag(dq), summed in a fixed order with plain IEEE products
    and additions (rows of B in order, pairs of a row in order, then the
    diagonal), so that every platform builds the same bits: a library sparse
    product may fuse or reorder them."""
    rp, ci, v = B
    lens = np.diff(rp)
    keys, prods = [], []
    rows_all = np.arange(lens.shape[0])
    for L in np.unique(lens):
        if L == 0:
            continue
        rows = rows_all[lens == L]
        idx = rp[rows][:, None] + np.arange(L)[None, :]          # (R, L) positions
        cols, vals = ci[idx].astype(np.int64), v[idx]
        k = (cols[:, :, None] * n + cols[:, None, :]).reshape(rows.shape[0], -1)
        pv = (vals[:, :, None] * vals[:, None, :]).reshape(rows.shape[0], -1)
        keys.append((rows, k))
        prods.append(pv)
    # the pairs in row order of B, then the diagonal
    flat_k = np.concatenate([k.reshape(-1) for _, k in keys]) if keys else np.zeros(0, np.int64)
    flat_v = np.concatenate([p.reshape(-1) for p in prods]) if prods else np.zeros(0)
    owner = np.concatenate([np.repeat(r, k.shape[1]) for r, k in keys]) if keys else np.zeros(0, np.int64)
    seq = np.argsort(owner, kind="stable")
    flat_k, flat_v = flat_k[seq], flat_v[seq]
    dk = np.arange(n, dtype=np.int64) * n + np.arange(n, dtype=np.int64)
    all_k = np.concatenate([flat_k, dk])
    all_v = np.concatenate([flat_v, np.asarray(dq, dtype=np.float64)])
    uk, inv = np.unique(all_k, return_inverse=True)
    qv = np.bincount(inv, weights=all_v, minlength=uk.shape[0])
    qr, qc = uk // n, uk % n
    qrp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(qrp, qr + 1, 1)
    return (np.cumsum(qrp).astype(np.int32), qc.astype(np.int32), qv, (n, n))


def transport_family(supplies: int, demands: int, seeds, base_costs=None, perturb: float = 0.2) -> list[LPData]:
    """transport_lp for many seeds, sharing one CSR of the (unit, complete
    bipartite) constraint matrix: instance k equals
    transport_lp(supplies, demands, seeds[k], base_costs, perturb)."""
    S, D = supplies, demands
    n = S * D
    if base_costs is None:
        base_costs = np.random.default_rng(4000).uniform(1, 100, size=n)
    arc = np.arange(n)
    A = _csr_from_coo(np.concatenate([arc // D, S + arc % D]), np.concatenate([arc, arc]), np.ones(2 * n), S + D, n)
    Acsr = (A[0], A[1], A[2], (S + D, n))
    out = []
    for sd in seeds:
        rng = np.random.default_rng(sd)
        cost = base_costs * (1.0 + perturb * rng.standard_normal(n))
        s = rng.uniform(10, 100, size=S)
        d = rng.uniform(10, 100, size=D)
        d *= s.sum() / d.sum()
        cap = rng.uniform(20, 200, size=n)
        b = np.concatenate([s, d])
        out.append(LPData(cost, Acsr, b.copy(), b.copy(), np.zeros(n), cap))
    return out
