"""Parity of the CUDA CP_AL (LP) solver with the CPU oracle, through the C-ABI
(create_lp_problem / cp_al_gb300_solve / cp_al_result_free).

Bars (floating point, FP64 form): same termination status; iteration counts
within 2%; relative objective difference <= 1e-8 at relative KKT 1e-8; per-block
iterates equal to 1e-9 relative after a fixed number of iterations.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pdal_gb300 import instances as I
from pdal_gb300 import lp

pytestmark = pytest.mark.gpu

OBJ_RTOL = 1e-8
ITER_RTOL = 0.02


def rel(a, b):
    return abs(a - b) / (1.0 + abs(b))


def both(data, params=None, options=None):
    params = {"time_limit": 120.0, **(params or {})}
    g = lp.solve(data, params, options)
    o = O.solve_lp(data, params, options)
    return g, o


def assert_parity(g, o, obj_rtol=OBJ_RTOL, iter_rtol=ITER_RTOL):
    assert g.status == o.status, (g.status, o.status)
    assert abs(g.iterations - o.iterations) <= max(iter_rtol * o.iterations, 0), (g.iterations, o.iterations)
    assert rel(g.primal_objective, o.primal_objective) <= obj_rtol, (g.primal_objective, o.primal_objective)
    assert rel(g.dual_objective, o.dual_objective) <= obj_rtol


def test_docs_example_known_answer(lp_lib):
    g = lp.solve(I.docs_example_lp(), {"eps": 1e-9})
    assert g.status == "OPTIMAL"
    assert np.allclose(g.x, [1.0, 2.0], atol=1e-6)
    assert abs(g.primal_objective - 3.0) < 1e-7


@pytest.mark.parametrize("m,n,k,seed", [(150, 400, 6, 1), (2000, 5000, 8, 0)])
def test_random_lp_parity(lp_lib, m, n, k, seed):
    g, o = both(I.random_lp(m, n, k, seed=seed), {"eps": 1e-8, "l_inf_ruiz_iterations": 4})
    assert g.status == "OPTIMAL"
    assert_parity(g, o)


def test_fixed_iterations_iterates_match(lp_lib):
    d = I.random_lp(300, 700, 6, seed=11)
    for blocks in (1, 3, 8):
        p = {"eps": 1e-14, "iteration_limit": 200 * blocks, "l_inf_ruiz_iterations": 4}
        g, o = both(d, p)
        assert g.status == o.status == "ITERATION_LIMIT"
        assert g.iterations == o.iterations
        sx = 1 + np.abs(o.x).max()
        sy = 1 + np.abs(o.y).max()
        assert np.abs(g.x - o.x).max() / sx < 1e-9
        assert np.abs(g.y - o.y).max() / sy < 1e-9
        assert np.abs(g.reduced_cost - o.reduced_cost).max() / (1 + np.abs(o.reduced_cost).max()) < 1e-9


def test_sigma_mode_parity(lp_lib):
    opts = {"sigma_mode": 1, "sigma_init_factor": 0.5, "al_lambda": 0.0, "sigma_kp": 0.5, "sigma_ki": 0.0,
            "sigma_kd": 0.0, "sigma_balance_gain": 0.0, "sigma_update_min": 1e-6, "sigma_update_max": 1e6,
            "restart_necessary": 0.8}
    g, o = both(I.random_lp(400, 1000, 6, seed=3), {"eps": 1e-8}, opts)
    assert g.status == "OPTIMAL"
    assert_parity(g, o)


@pytest.mark.parametrize("variant", [
    {"options": {"al_lambda": 0.0}},                      # no augmentation: gather y directly
    {"params": {"reflection_coefficient": 0.7}},          # A x carried through the recurrence
    {"params": {"linf": True}},                           # L-infinity optimality norm
    {"params": {"bound_objective_rescaling": False, "has_pock_chambolle_alpha": False}},
])
def test_option_variants_parity(lp_lib, variant):
    p = {"eps": 1e-8, "l_inf_ruiz_iterations": 4, **variant.get("params", {})}
    g, o = both(I.random_lp(300, 800, 5, seed=21), p, variant.get("options"))
    assert g.status == "OPTIMAL"
    assert_parity(g, o)


def test_transport_and_warm_start(lp_lib):
    d = I.transport_lp(15, 20, seed=2)
    g, o = both(d, {"eps": 1e-8})
    assert_parity(g, o)
    d.primal_start, d.dual_start = g.x, g.y
    g2, o2 = both(d, {"eps": 1e-8})
    assert_parity(g2, o2)
    assert g2.iterations <= g.iterations


@pytest.mark.parametrize("S", [256, 512, 1024, 2048])
def test_long_rows_and_block_budgets(lp_lib, S):
    """A few dense rows longer than the block budget take the split-row path."""
    d = I.random_lp(200, 3000, 3, seed=5)
    rp, ci, v, (m, n) = d.csr()
    rng = np.random.default_rng(0)
    rows = [list(zip(ci[rp[i]:rp[i + 1]], v[rp[i]:rp[i + 1]])) for i in range(m)]
    for i in (3, 77):  # make two rows dense: 3000 nonzeros each
        rows[i] = [(j, rng.standard_normal()) for j in range(n)]
    rp2 = np.zeros(m + 1, np.int32)
    rp2[1:] = np.cumsum([len(r) for r in rows])
    ci2 = np.array([j for r in rows for j, _ in r], np.int32)
    v2 = np.array([x for r in rows for _, x in r])
    Ax = np.zeros(m)
    for i in (3, 77):
        Ax[i] = v2[rp2[i]:rp2[i + 1]].sum()
        d.con_lb[i] = Ax[i]
        d.con_ub[i] = Ax[i] + 1.0
    d.A = (rp2, ci2, v2, (m, n))
    p = {"eps": 1e-14, "iteration_limit": 600, "l_inf_ruiz_iterations": 4}
    g = lp.solve(d, p, {"spmv_nnz_per_block": S})
    o = O.solve_lp(d, p)
    assert np.abs(g.x - o.x).max() / (1 + np.abs(o.x).max()) < 1e-9
    assert np.abs(g.y - o.y).max() / (1 + np.abs(o.y).max()) < 1e-9


def _lp_with_dense_rows(rows_dense=(3, 77, 150), m=200, n=3000, seed=5):
    """random_lp with a few rows made dense (every first, second or third
    column), bounds kept feasible around the planted point."""
    d = I.random_lp(m, n, 3, seed=seed)
    rp, ci, v, _ = d.csr()
    rng = np.random.default_rng(0)
    rows = [list(zip(ci[rp[i]:rp[i + 1]], v[rp[i]:rp[i + 1]])) for i in range(m)]
    for i in rows_dense:
        rows[i] = [(j, rng.standard_normal()) for j in range(0, n, 1 + i % 3)]
    rp2 = np.zeros(m + 1, np.int32)
    rp2[1:] = np.cumsum([len(r) for r in rows])
    ci2 = np.array([j for r in rows for j, _ in r], np.int32)
    v2 = np.array([x for r in rows for _, x in r])
    for i in rows_dense:
        s_i = v2[rp2[i]:rp2[i + 1]].sum()
        d.con_lb[i] = s_i
        d.con_ub[i] = s_i + 1.0
    d.A = (rp2, ci2, v2, (m, n))
    return d


@pytest.mark.parametrize("width", [1024, 2048, 4096])
def test_long_rows_by_column_panels(lp_lib, width):
    """The long rows of the iteration's A x by column panels (x staged in
    shared memory, one partial per row and panel, then a warp per row): the
    iterates still follow the oracle, with one panel (4096), two and three."""
    d = _lp_with_dense_rows()
    n = d.A[3][1]
    p = {"eps": 1e-14, "iteration_limit": 600, "l_inf_ruiz_iterations": 4}
    g = lp.solve(d, p, {"spmv_nnz_per_block": 256, "dual_panels": 1, "panel_width": width})
    assert g.stats["panel_rows"] == 3 and g.stats["panels"] == (n + width - 1) // width
    o = O.solve_lp(d, p)
    assert np.abs(g.x - o.x).max() / (1 + np.abs(o.x).max()) < 1e-9
    assert np.abs(g.y - o.y).max() / (1 + np.abs(o.y).max()) < 1e-9


@pytest.mark.parametrize("opts", [{"al_lambda": 0.0}, {"al_lambda": 0.0, "sigma_mode": 1, "sigma_init_factor": 0.5}],
                         ids=["lambda0", "sigma"])
def test_badly_scaled_zipf_panels_iterates_match(lp_lib, opts):
    """The large-LP structure at 1/50 scale with its long rows by column
    panels (ten panels): iterates against the oracle after 1,000 iterations."""
    d = I.zipf_lp(20_000, 40_000, 400_000, seed=1002)
    p = {"eps": 1e-14, "iteration_limit": 1000, "sv_max_iter": 200, "time_limit": 120}
    g = lp.solve(d, p, {**opts, "dual_panels": 1, "panel_width": 4096})
    assert g.stats["panel_rows"] > 0 and g.stats["panels"] == 10
    o = O.solve_lp(d, p, opts)
    assert g.iterations == o.iterations
    for a, b in ((g.x, o.x), (g.y, o.y)):
        err = np.abs(a - b).max() / (1 + np.abs(b).max())
        assert err < 1e-8, err


@pytest.mark.parametrize("precision", ["fp64", "fp32_refine"])
def test_primal_hot_rows_change_nothing(lp_lib, precision):
    """Taking the long rows' entries of the gathered dual vector from shared
    memory in A^T u changes where a value is read, not the value or the order
    of the sums: bit-identical iterates with and without it, in both forms."""
    d = I.zipf_lp(20_000, 40_000, 400_000, seed=1002)
    p = {"eps": 1e-14, "iteration_limit": 1200, "sv_max_iter": 200, "time_limit": 120}
    base = {"al_lambda": 0.0, "precision": precision, "dual_panels": 1, "panel_width": 4096,
            "fp32_switch_tol": 1e-4, "fp32_stall_evals": 2}
    a = lp.solve(d, p, {**base, "primal_hot_rows": 0})
    b = lp.solve(d, p, {**base, "primal_hot_rows": 1})
    assert a.stats["panel_rows"] > 0
    assert a.iterations == b.iterations and a.stats["fp32_iterations"] == b.stats["fp32_iterations"]
    assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)


@pytest.mark.parametrize("precision", ["fp64", "fp32_refine"])
@pytest.mark.parametrize("budget", [256, 2048])
def test_staged_primal_product_changes_nothing(lp_lib, precision, budget):
    """The staged primal product (one wave of blocks, each row block's slice
    and row inputs copied ahead by TMA) keeps k_primal's lane groups and
    summation order: bit-identical iterates with and without it, on an LP
    with empty, one-entry and long columns (pieces of the row-block budget)."""
    d = I.zipf_lp(20_000, 40_000, 400_000, seed=1002)
    rp, ci, v, (m, n) = d.csr()
    # two dense columns: rows of A^T long enough to be split into pieces
    extra = np.arange(0, m, 3)
    rows = np.repeat(np.arange(m), np.diff(rp))
    keep = ~np.isin(ci, [5, 13])
    rows = np.concatenate([rows[keep], extra, extra])
    cols = np.concatenate([ci[keep], np.full(extra.size, 5), np.full(extra.size, 13)])
    vals = np.concatenate([v[keep], np.ones(extra.size), -np.ones(extra.size)])
    import scipy.sparse as sp

    A = sp.csr_matrix((vals, (rows, cols)), shape=(m, n))
    A.sort_indices()
    d.A = (A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data, (m, n))
    p = {"eps": 1e-14, "iteration_limit": 1000, "sv_max_iter": 200, "time_limit": 120}
    base = {"al_lambda": 0.0, "precision": precision, "spmv_nnz_per_block": budget, "fp32_switch_tol": 1e-4,
            "fp32_stall_evals": 2}
    a = lp.solve(d, p, {**base, "primal_staged": 0})
    for mode in (1, 2):
        b = lp.solve(d, p, {**base, "primal_staged": mode})
        assert a.iterations == b.iterations and a.stats["fp32_iterations"] == b.stats["fp32_iterations"]
        assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)


@pytest.mark.parametrize("precision", ["fp64", "fp32_refine"])
def test_concurrent_dual_launches_change_nothing(lp_lib, precision):
    """The dual step's short-row and panel launches on two streams
    (dual_concurrent) write disjoint outputs from the same x-bar: iterates
    bit-identical to the launches one after the other, also with the timing
    events bracketing the forked step."""
    d = _lp_with_dense_rows()
    p = {"eps": 1e-14, "iteration_limit": 2000, "time_limit": 120, "l_inf_ruiz_iterations": 4}
    base = {"precision": precision, "spmv_nnz_per_block": 256, "dual_panels": 1, "panel_width": 1024,
            "fp32_switch_tol": 1e-4, "fp32_stall_evals": 2}
    a = lp.solve(d, p, {**base, "dual_concurrent": 0})
    for extra in ({}, {"timing": 1}):
        b = lp.solve(d, p, {**base, "dual_concurrent": 1, **extra})
        assert b.stats["panel_rows"] == 3
        assert a.iterations == b.iterations and a.stats["fp32_iterations"] == b.stats["fp32_iterations"]
        assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)
    assert b.stats["avg_dual_ms" if precision == "fp64" else "avg_dual32_ms"] > 0


def test_panels_fp32_form_reaches_tolerance(lp_lib):
    """Chosen form (FP32 phase, then FP64) with the panel path: same status and
    objective as the oracle at relative KKT 1e-7."""
    d = _lp_with_dense_rows()
    p = {"eps": 1e-7, "iteration_limit": 200_000, "time_limit": 120, "l_inf_ruiz_iterations": 4}
    g = lp.solve(d, p, {"precision": "fp32_refine", "spmv_nnz_per_block": 256, "dual_panels": 1,
                        "panel_width": 1024})
    assert g.stats["panel_rows"] == 3 and g.stats["fp32_iterations"] > 0
    o = O.solve_lp(d, p)
    assert g.status == o.status == "OPTIMAL"
    assert g.kkt < 1e-7
    assert rel(g.primal_objective, o.primal_objective) <= 1e-6


def test_edge_rows_and_columns(lp_lib):
    """Empty rows, empty columns, free rows, free and fixed variables."""
    d = I.random_lp(120, 300, 4, seed=8)
    rp, ci, v, (m, n) = d.csr()
    keep = (ci % 17) != 0  # empties some columns
    row_of = np.repeat(np.arange(m), np.diff(rp))
    keep &= ~np.isin(row_of, [0, 5, 50])  # empties rows 0, 5, 50
    rp2 = np.zeros(m + 1, np.int32)
    np.add.at(rp2, row_of[keep] + 1, 1)
    rp2 = np.cumsum(rp2).astype(np.int32)
    d.A = (rp2, ci[keep].astype(np.int32), v[keep], (m, n))
    d.con_lb[[0, 5]] = -np.inf
    d.con_ub[[0, 5]] = np.inf
    d.con_lb[50], d.con_ub[50] = -1.0, 1.0
    d.con_lb[10], d.con_ub[10] = -np.inf, np.inf  # free row with entries
    d.var_lb[:10] = -np.inf
    d.var_ub[:10] = np.inf
    d.c[:10] = 0.0
    d.var_lb[10:15] = d.var_ub[10:15] = 2.0  # fixed
    p = {"eps": 1e-14, "iteration_limit": 1000, "l_inf_ruiz_iterations": 4}
    g, o = both(d, p)
    assert np.all(np.isfinite(g.x)) and np.all(np.isfinite(g.y))
    assert np.abs(g.x - o.x).max() / (1 + np.abs(o.x).max()) < 1e-9
    assert np.abs(g.y - o.y).max() / (1 + np.abs(o.y).max()) < 1e-9


def test_no_constraints(lp_lib):
    n = 50
    d = lp.LPData(np.linspace(-1, 1, n), (np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), (0, n)),
                  np.zeros(0), np.zeros(0), np.zeros(n), np.full(n, 3.0))
    g, o = both(d, {"eps": 1e-10})
    assert g.status == o.status == "OPTIMAL"
    assert np.allclose(g.x, np.where(d.c < 0, 3.0, 0.0), atol=1e-6)


def test_fp32_refine_matches_fp64(lp_lib):
    d = I.random_lp(2000, 5000, 8, seed=0)
    p = {"eps": 1e-8, "l_inf_ruiz_iterations": 4}
    g32 = lp.solve(d, p, {"precision": "fp32_refine"})
    o = O.solve_lp(d, p)
    assert g32.status == "OPTIMAL"
    assert g32.stats["fp32_iterations"] > 0
    assert rel(g32.primal_objective, o.primal_objective) <= 1e-8


def test_session_is_deterministic(lp_lib):
    d = I.random_lp(500, 1200, 6, seed=4)
    p = {"eps": 1e-8, "l_inf_ruiz_iterations": 4}
    s = lp.LPSession(d, p)
    try:
        r1 = s.solve()
        x1, y1, _ = s.fetch()
        r2 = s.solve()
        x2, y2, _ = s.fetch()
    finally:
        s.close()
    assert r1.iterations == r2.iterations
    assert np.array_equal(x1, x2) and np.array_equal(y1, y2)
    g = lp.solve(d, p)
    assert g.iterations == r1.iterations
    assert np.array_equal(g.x, x1)


@pytest.mark.parametrize("iters", [200, 1000])
def test_badly_scaled_zipf_iterates_match(lp_lib, iters):
    """Zipf row lengths (split rows), entries spread over 1e-6..1e6, free
    variables: the large-LP structure at 1/50 scale."""
    d = I.zipf_lp(20_000, 40_000, 400_000, seed=1002)
    p = {"eps": 1e-14, "iteration_limit": iters, "sv_max_iter": 200, "time_limit": 120}
    # CP_AL_LAMBDA=0: with the default augmentation (0.05) the reference
    # iteration itself amplifies 1e-13 input perturbations to 1e-5 within 200
    # iterations on this instance (oracle-only experiment), so no two
    # implementations can agree there beyond that level
    g, o = both(d, p, {"al_lambda": 0.0})
    assert g.iterations == o.iterations
    for a, b in ((g.x, o.x), (g.y, o.y)):
        err = np.abs(a - b).max() / (1 + np.abs(b).max())
        assert err < 1e-8, err


@pytest.mark.parametrize("options", [
    {"restart_select": 1},
    {"restart_select": 2},
    {"restart_select": 1, "sigma_mode": 1, "sigma_init_factor": 0.5, "al_lambda": 0.0, "sigma_kp": 0.5,
     "sigma_ki": 0.0, "sigma_kd": 0.0, "sigma_balance_gain": 0.0, "restart_necessary": 0.8},
], ids=["select1", "select2", "select1_sigma"])
def test_restart_target_selection_parity(lp_lib, options):
    """Restart to the Halpern iterate when its score wins (A13): iterates after
    fixed blocks and the full solve match the oracle."""
    d = I.random_lp(300, 700, 6, seed=21)
    p = {"eps": 1e-14, "iteration_limit": 1600, "l_inf_ruiz_iterations": 4}
    g, o = both(d, p, options)
    assert g.iterations == o.iterations
    assert np.abs(g.x - o.x).max() / (1 + np.abs(o.x).max()) < 1e-8
    assert np.abs(g.y - o.y).max() / (1 + np.abs(o.y).max()) < 1e-8
    g, o = both(d, {"eps": 1e-8, "l_inf_ruiz_iterations": 4}, options)
    assert g.status == "OPTIMAL"
    assert_parity(g, o)


SIGMA_OPTS = {"sigma_mode": 1, "sigma_init_factor": 0.5, "al_lambda": 0.0, "sigma_kp": 0.5, "sigma_ki": 0.0,
              "sigma_kd": 0.0, "sigma_balance_gain": 0.0, "restart_necessary": 0.8}


@pytest.mark.parametrize("refl,options,halpern_restarts", [
    (0.5, {"restart_select": 3}, 1),
    (0.3, {"restart_select": 1, "restart_select_threepoint": 1, "al_lambda": 0.0}, 4),
    (0.3, {"restart_select": 3, **SIGMA_OPTS}, 4),
], ids=["select3_beta", "select1_threepoint", "select3_sigma"])
def test_restart_three_point_parity(lp_lib, refl, options, halpern_restarts):
    """Three-point restart target selection (A13, LP/CP_AL/src/solver.cu:
    2749-2819, 3043-3075): the plain Halpern point w x^ + (1 - w) x0 wins
    the oracle's restarts as counted here within the first 1600 iterations;
    the iterates after those blocks and the full solve match the oracle."""
    d = I.random_lp(300, 700, 6, seed=3)
    base = {"l_inf_ruiz_iterations": 4, "reflection_coefficient": refl}
    g, o = both(d, {**base, "eps": 1e-14, "iteration_limit": 1600}, options)
    assert o.stats["restart_targets"][2] == halpern_restarts, o.stats["restart_targets"]
    assert g.iterations == o.iterations
    assert g.stats["restarts"] == sum(o.stats["restart_targets"])
    assert np.abs(g.x - o.x).max() / (1 + np.abs(o.x).max()) < 1e-8
    assert np.abs(g.y - o.y).max() / (1 + np.abs(o.y).max()) < 1e-8
    g, o = both(d, {**base, "eps": 1e-8}, options)
    assert g.status == "OPTIMAL"
    assert_parity(g, o)


@pytest.mark.parametrize("sv_max_iter", [5000, 60])
def test_fp32_power_iteration_matches_fp64(lp_lib, sv_max_iter):
    """The chosen form's fused FP32 power step (FP32 products, FP64 sums, the
    residual from the Rayleigh sums, alternating vector buffers) against the
    FP64 form's separate residual pass: the same number of power iterations
    (converged within 5,000, or at the 60 cap) within one, and the same
    sigma_max(A)^2 estimate within 1e-6 relative."""
    d = I.random_lp(300, 700, 6, seed=21)
    p = {"eps": 1e-4, "l_inf_ruiz_iterations": 4, "sv_max_iter": sv_max_iter, "iteration_limit": 400}
    g64 = lp.solve(d, p)
    g32 = lp.solve(d, p, {"precision": "fp32_refine", "power_method": 0})
    it64, it32 = g64.stats["power_iterations"], g32.stats["power_iterations"]
    assert abs(it32 - it64) <= 1, (it32, it64)
    if sv_max_iter == 60:
        assert it32 == it64 == 60
    else:
        assert it64 < 5000
    assert rel(g32.stats["lambda_est"], g64.stats["lambda_est"]) < 1e-6


@pytest.mark.parametrize("shape", [(300, 700, 6, 21), (2000, 5000, 8, 0)])
def test_lanczos_estimate(lp_lib, shape):
    """The chosen form's Lanczos estimate of sigma_max(A)^2 against the dense
    SVD of the same equilibrated matrix: within 1e-6 relative, never above it
    by more than FP32 rounding, and in far fewer steps than the power
    iteration of the FP64 form."""
    m, n, k, seed = shape
    d = I.random_lp(m, n, k, seed=seed)
    p = {"eps": 1e-4, "l_inf_ruiz_iterations": 4, "iteration_limit": 200}
    s = lp.LPSession(d, p, {"precision": "fp32_refine"})
    vals, rsc, csc, cbr, ovr, lam = s.scaling()
    s.close()
    rp, ci, _, _ = d.csr()
    A = np.zeros((m, n))
    A[np.repeat(np.arange(m), np.diff(rp)), ci] = vals
    true = np.linalg.svd(A, compute_uv=False)[0] ** 2
    assert lam <= true * (1 + 1e-6)
    assert rel(lam, true) < 1e-6 * (1 + true)
    g = lp.solve(d, p, {"precision": "fp32_refine"})
    g64 = lp.solve(d, p)
    assert g.stats["power_iterations"] <= 128
    assert g.stats["power_iterations"] < g64.stats["power_iterations"] or g64.stats["power_iterations"] < 64


def test_restart_three_point_fp32_form(lp_lib):
    """The three-point selection in the FP32 form (anchors rebuilt as (hi, lo)
    pairs at a restart to the plain Halpern point) reaches the oracle's
    optimum at 1e-8."""
    d = I.random_lp(300, 700, 6, seed=3)
    p = {"eps": 1e-8, "l_inf_ruiz_iterations": 4, "reflection_coefficient": 0.3}
    g = lp.solve(d, p, {"restart_select": 3, "precision": "fp32_refine"})
    o = O.solve_lp(d, p, {"restart_select": 3})
    assert g.status == "OPTIMAL" and o.stats["restart_targets"][2] > 0
    assert rel(g.primal_objective, o.primal_objective) <= 1e-6


@pytest.mark.parametrize("opts,passes", [
    ({"cr_iterations": 20}, 20),
    ({"cr_iterations": 20, "cr_early_stop": 1, "cr_early_stop_threshold": 1e9}, 5),
    ({"cr_iterations": 7}, 7),
], ids=["cr20", "cr_early_stop", "cr7"])
def test_curtis_reid_scaling_matches_oracle(lp_lib, opts, passes):
    """The device Curtis-Reid passes before Ruiz (LP/CP_AL/src/
    preconditioner.cu:162-270, 553-624) on a badly scaled LP: the same number
    of passes as the oracle and the same cumulative scales, scaled matrix and
    bound/objective factors to 1e-11 relative (log and exp of the device and
    the host libraries may differ in the last bit)."""
    d = I.zipf_lp(400, 900, nnz=6000, seed=3, max_row=300)
    prm = {"l_inf_ruiz_iterations": 4}
    s = lp.LPSession(d, prm, opts)
    try:
        s.start()
        vals, r, c, cbr, ovr, _ = s.scaling()
    finally:
        s.close()
    ro, co, cbro, ovro, svo, po = O.rescale(d, prm, opts, with_passes=True)
    assert po == passes
    for a, b in ((r, ro), (c, co), (vals, svo)):
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-11
    assert rel(cbr, cbro) < 1e-11 and rel(ovr, ovro) < 1e-11


def test_curtis_reid_solve_parity(lp_lib):
    """A solve with Curtis-Reid scaling on: the oracle's status, iterations
    and objectives."""
    d = I.random_lp(300, 700, 6, seed=21)
    g, o = both(d, {"eps": 1e-8, "l_inf_ruiz_iterations": 4}, {"cr_iterations": 20})
    assert g.status == "OPTIMAL" and g.stats["cr_passes"] == 20
    assert_parity(g, o)


@pytest.mark.parametrize("kind", ["random", "transport"])
def test_feasibility_polishing_matches_oracle(kind):
    """Feasibility polishing (LP/CP_AL/src/solver.cu:3912-4456) after a loose
    solve: both phases reach eps_feas_polish_relative on the GPU and in the
    oracle, the polished solution has the oracle's residual scale and
    objective, and the phases take the same number of iterations within one
    evaluation block."""
    data = I.random_lp(300, 800, 6, seed=17) if kind == "random" else I.transport_lp(15, 12, seed=5)
    prm = {"eps": 1e-3, "l_inf_ruiz_iterations": 4, "feasibility_polishing": True, "eps_feas_polish": 1e-8}
    g = lp.solve(data, prm)
    o = O.solve_lp(data, prm)
    assert g.status == o.status
    assert (g.stats["polish_primal_status"], g.stats["polish_dual_status"]) == (7, 7)
    assert o.stats["polish_status"] == ("FEAS_POLISH_SUCCESS", "FEAS_POLISH_SUCCESS")
    assert g.relative_primal_residual <= 1e-8 and g.relative_dual_residual <= 1e-8
    assert abs(g.primal_objective - o.primal_objective) <= 1e-6 * (1 + abs(o.primal_objective))
    assert abs(g.stats["feasibility_iteration"] - o.stats["feasibility_iteration"]) <= 400
    # the polished point is primal feasible for the original problem
    rp, ci, v, (m, n) = data.csr()
    import scipy.sparse as sp

    A = sp.csr_matrix((v, ci, rp), shape=(m, n))
    ax = A @ g.x
    viol = np.maximum(np.asarray(data.con_lb) - ax, 0) + np.maximum(ax - np.asarray(data.con_ub), 0)
    assert np.linalg.norm(viol) <= 1e-6 * (1 + np.linalg.norm(np.nan_to_num(data.con_ub, posinf=0)))


@pytest.mark.parametrize("kind,status", [("primal", "PRIMAL_INFEASIBLE"), ("dual", "DUAL_INFEASIBLE")])
@pytest.mark.parametrize("seed", [3, 8])
def test_infeasibility_detection_matches_oracle(lp_lib, kind, status, seed):
    """Opt-in infeasibility certificates, evaluated on the device at every
    evaluation: same status, same evaluation and certificate values as the
    oracle in FP64; the chosen form reaches the same status."""
    d = I.infeasible_lp(kind, seed=seed)
    p = {"eps": 1e-8, "iteration_limit": 20_000, "time_limit": 120}
    g = lp.solve(d, p, {"infeasibility_detection": 1})
    o = O.solve_lp(d, p, {"infeasibility_detection": 1})
    assert g.status == o.status == status
    assert g.iterations == o.iterations
    for f in ("max_primal_ray_infeasibility", "max_dual_ray_infeasibility", "primal_ray_linear_objective",
              "dual_ray_objective"):
        assert abs(g.stats[f] - o.stats[f]) <= 1e-7 * (1 + abs(o.stats[f])), f
    g32 = lp.solve(d, p, {"infeasibility_detection": 1, "precision": "fp32_refine"})
    assert g32.status == status


def test_infeasibility_detection_leaves_feasible_solves_alone(lp_lib):
    d = I.random_lp(300, 800, 6, seed=21)
    a = lp.solve(d, {"eps": 1e-8}, {"infeasibility_detection": 0})
    b = lp.solve(d, {"eps": 1e-8}, {"infeasibility_detection": 1})
    assert a.status == b.status == "OPTIMAL" and a.iterations == b.iterations
    assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)


@pytest.mark.parametrize("precision", ["fp64", "fp32_refine"])
@pytest.mark.parametrize("opts", [{}, {"al_lambda": 0.0}, {"al_lambda": 0.0, "sigma_mode": 1, "sigma_init_factor": 0.5}],
                         ids=["default", "lambda0", "sigma"])
def test_persistent_loop_matches_graph_path(lp_lib, precision, opts):
    """The small-LP persistent loop (one cooperative launch, grid barriers)
    runs the graph path's row blocks, epilogues, controller and restart:
    bit-identical iterates, iteration counts and phase switch."""
    d = I.random_lp(2000, 5000, 8, seed=0)
    p = {"eps": 1e-7, "l_inf_ruiz_iterations": 4, "iteration_limit": 30_000}
    base = {**opts, "precision": precision}
    a = lp.solve(d, p, {**base, "persistent_loop": 0})
    b = lp.solve(d, p, {**base, "persistent_loop": 1})
    assert a.status == b.status and a.iterations == b.iterations
    assert a.stats["fp32_iterations"] == b.stats["fp32_iterations"]
    assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)
    assert b.stats["kernel_launches"] < a.stats["kernel_launches"]


@pytest.mark.parametrize("case", ["zipf_panels_hot", "dense_columns", "random"])
def test_device_transpose_is_the_host_transpose(lp_lib, case):
    """A^T built on the device (atomic scatter, then every column sorted by
    row: one thread for short columns, a block's bitonic sort for long ones)
    is the host transpose exactly: bit-identical iterates with either, also
    with the long rows' hot-index copy of A^T (FP64 panel path)."""
    if case == "zipf_panels_hot":
        d = I.zipf_lp(20_000, 40_000, 400_000, seed=1002)
        opts = {"al_lambda": 0.0, "dual_panels": 1, "panel_width": 4096}
    elif case == "dense_columns":
        d = I.random_lp(2000, 5000, 8, seed=4)
        rp, ci, v, (m, n) = d.csr()
        rows = np.repeat(np.arange(m), np.diff(rp))
        # columns 7, 11 and 13 get 600, 1,900 and 2,000 entries: the block sort
        extra = [(7, np.arange(0, m, 3)[:600]), (11, np.arange(0, m, 1)[:1900]), (13, np.arange(0, m)[:2000])]
        keep = ~np.isin(ci, [7, 11, 13])
        rr, cc, vv = [rows[keep]], [ci[keep]], [v[keep]]
        for col, rws in extra:
            rr.append(rws)
            cc.append(np.full(rws.size, col))
            vv.append(np.random.default_rng(col).standard_normal(rws.size))
        import scipy.sparse as sp

        A = sp.csr_matrix((np.concatenate(vv), (np.concatenate(rr), np.concatenate(cc))), shape=(m, n))
        A.sort_indices()
        d.A = (A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data, (m, n))
        opts = {}
    else:
        d = I.random_lp(300, 800, 6, seed=9)
        opts = {}
    p = {"eps": 1e-14, "iteration_limit": 600, "sv_max_iter": 200, "time_limit": 120}
    a = lp.solve(d, p, {**opts, "device_transpose": 0})
    b = lp.solve(d, p, {**opts, "device_transpose": 1})
    assert a.iterations == b.iterations
    assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)
    assert b.stats["h2d_bytes"] < a.stats["h2d_bytes"]


def test_controllers_in_the_fp32_phase(lp_lib):
    """The sigma trigger and the alpha pulse switch the AL penalty on inside
    the chosen form's FP32 phase (the host then recomputes A x0 and the
    predictor in FP32 before the predictor form's graph): the trigger fires
    where the FP64 form's does and the solve reaches the oracle's optimum; the
    pulse runs its positive block inside a long FP32 phase and the iterate
    stays close to the FP64 form's."""
    trig = {"al_lambda": 0.0, "sigma_trigger": 1, "sigma_trigger_min_iters": 2000, "sigma_trigger_primal": 0.0,
            "sigma_trigger_dual": 1.0, "sigma_trigger_ratio": 0.0}
    d = I.random_lp(300, 800, 6, seed=17)
    p = {"eps": 1e-8, "l_inf_ruiz_iterations": 4}
    g = lp.solve(d, p, {**trig, "precision": "fp32_refine", "fp32_switch_tol": 1e-7})
    o = O.solve_lp(d, p, trig)
    assert g.status == o.status == "OPTIMAL"
    assert g.stats["sigma_trigger_iteration"] == o.stats["sigma_trigger_iteration"] == 2000
    assert g.stats["fp32_iterations"] > 2000
    assert rel(g.primal_objective, o.primal_objective) <= 1e-7
    d = I.random_lp(200, 500, 5, seed=5)
    p = {"eps": 1e-14, "iteration_limit": 12000, "l_inf_ruiz_iterations": 0, "has_pock_chambolle_alpha": False,
         "bound_objective_rescaling": False}
    pulse = {"al_lambda": 0.0, "alpha_direct_pulse": 1, "pulse_force": 1}
    g32 = lp.solve(d, p, {**pulse, "precision": "fp32_refine", "fp32_switch_tol": 1e-12,
                          "fp32_stall_evals": 1_000_000})
    g64 = lp.solve(d, p, pulse)
    assert g32.stats["fp32_iterations"] == 12000 and g32.stats["pulse_gate"] == 1
    assert 10000 <= g32.stats["pulse_start_iteration"] <= 11800
    assert np.all(np.isfinite(g32.x)) and rel(g32.primal_objective, g64.primal_objective) <= 1e-5
