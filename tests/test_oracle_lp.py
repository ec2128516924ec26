"""Pins of the CPU oracle (the checker of the CUDA library).

The reference ships no numeric golden vectors for this path, so the oracle is
pinned against known answers: the analytic optimum of the reference's own C API
example, independent LP optima from scipy's HiGHS, the dense SVD for the power
iteration, committed fixtures (tests/golden), and the reference defaults.
"""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.optimize import linprog

from oracle import oracle as O
from pdal_gb300 import instances as I
from pdal_gb300.lp import LPData


def highs_objective(d):
    rp, ci, v, (m, n) = d.csr()
    A = sp.csr_matrix((v, ci, rp), shape=(m, n))
    eq = np.isfinite(d.con_lb) & (d.con_lb == d.con_ub)
    ub_rows = ~eq & np.isfinite(d.con_ub)
    lb_rows = ~eq & np.isfinite(d.con_lb)
    A_ub = sp.vstack([A[ub_rows], -A[lb_rows]])
    b_ub = np.concatenate([d.con_ub[ub_rows], -d.con_lb[lb_rows]])
    bounds = list(zip(np.where(np.isfinite(d.var_lb), d.var_lb, None), np.where(np.isfinite(d.var_ub), d.var_ub, None)))
    res = linprog(d.c, A_ub=A_ub, b_ub=b_ub, A_eq=A[eq], b_eq=d.con_lb[eq], bounds=bounds, method="highs")
    assert res.status == 0
    return res.fun


def test_docs_example_known_answer():
    # LP/CP_AL/docs/C_API.md:41-89: optimum x = (1, 2), objective 3
    r = O.solve_lp(I.docs_example_lp(), {"eps": 1e-9})
    assert r.status == "OPTIMAL"
    assert np.allclose(r.x, [1.0, 2.0], atol=1e-6)
    assert abs(r.primal_objective - 3.0) < 1e-7
    assert abs(r.dual_objective - 3.0) < 1e-7


@pytest.mark.parametrize("seed", [1, 2])
def test_random_lp_matches_highs(seed):
    d = I.random_lp(150, 400, 6, seed=seed)
    r = O.solve_lp(d, {"eps": 1e-9, "l_inf_ruiz_iterations": 4})
    assert r.status == "OPTIMAL"
    f = highs_objective(d)
    assert abs(r.primal_objective - f) / (1 + abs(f)) < 1e-7


def test_transport_matches_highs():
    d = I.transport_lp(12, 15, seed=3)
    r = O.solve_lp(d, {"eps": 1e-9})
    assert r.status == "OPTIMAL"
    f = highs_objective(d)
    assert abs(r.primal_objective - f) / (1 + abs(f)) < 1e-7


def test_sigma_mode_matches_highs():
    d = I.random_lp(120, 300, 5, seed=7)
    opts = {"sigma_mode": 1, "sigma_init_factor": 0.5, "al_lambda": 0.0, "sigma_kp": 0.5, "sigma_ki": 0.0,
            "sigma_kd": 0.0, "sigma_balance_gain": 0.0, "sigma_update_min": 1e-6, "sigma_update_max": 1e6,
            "restart_necessary": 0.8}
    r = O.solve_lp(d, {"eps": 1e-9}, opts)
    assert r.status == "OPTIMAL"
    f = highs_objective(d)
    assert abs(r.primal_objective - f) / (1 + abs(f)) < 1e-7


def test_power_iteration_matches_svd():
    d = I.random_lp(60, 150, 4, seed=5)
    rp, ci, v, (m, n) = d.csr()
    A = sp.csr_matrix((v, ci, rp), shape=(m, n)).toarray()
    s, it = O.power_iteration(d, 5000, 1e-10)
    smax = np.linalg.svd(A, compute_uv=False)[0]
    assert abs(s - smax) / smax < 1e-6
    assert 1 <= it <= 5000


def test_ruiz_equilibrates_rows_and_columns():
    d = I.random_lp(80, 200, 5, seed=9)
    rp, ci, v, (m, n) = d.csr()
    r, c, cbr, ovr, sv = O.rescale(d, {"l_inf_ruiz_iterations": 25, "has_pock_chambolle_alpha": False,
                                      "bound_objective_rescaling": False})
    S = sp.csr_matrix((sv, ci, rp), shape=(m, n))
    row_max = abs(S).max(axis=1).toarray().ravel()
    col_max = abs(S).max(axis=0).toarray().ravel()
    assert np.all(abs(row_max[row_max > 0] - 1) < 1e-3)
    assert np.all(abs(col_max[col_max > 0] - 1) < 1e-3)
    # scaled entries are D_r^-1 A D_c^-1 of the original
    A = sp.csr_matrix((v, ci, rp), shape=(m, n))
    expect = sp.diags(1 / r) @ A @ sp.diags(1 / c)
    assert np.allclose(S.toarray(), expect.toarray(), rtol=1e-12, atol=0)
    assert cbr == 1.0 and ovr == 1.0


def test_defaults_are_the_reference_defaults(lp_lib):
    from pdal_gb300 import lp

    p_prod = lp.default_parameters(lp_lib)
    p_or = O.default_parameters()
    for name, _ in type(p_or)._fields_:
        a, b = getattr(p_prod, name), getattr(p_or, name)
        if hasattr(a, "_fields_"):
            for sub, _ in type(a)._fields_:
                assert getattr(a, sub) == getattr(b, sub), (name, sub)
        else:
            assert a == b, name
    o_prod = lp.default_options(lp_lib)
    o_or = O.default_options()
    for name, _ in type(o_or)._fields_:
        a, b = getattr(o_prod, name), getattr(o_or, name)
        assert (a == b) or (np.isnan(a) and np.isnan(b)), name


def test_oracle_feasibility_polishing():
    """The oracle's feasibility polishing (LP/CP_AL/src/solver.cu:3912-4456):
    after a loose solve both phases reach the polishing tolerance, the
    primal objective moves toward the optimum, and a solve that is already
    feasible enough runs no polishing iterations."""
    from pdal_gb300.instances import random_lp

    d = random_lp(300, 800, 6, seed=17)
    loose = O.solve_lp(d, {"eps": 1e-3, "l_inf_ruiz_iterations": 4})
    pol = O.solve_lp(d, {"eps": 1e-3, "l_inf_ruiz_iterations": 4, "feasibility_polishing": True,
                         "eps_feas_polish": 1e-8})
    assert pol.stats["polish_status"] == ("FEAS_POLISH_SUCCESS", "FEAS_POLISH_SUCCESS")
    assert pol.relative_primal_residual <= 1e-8 < loose.relative_primal_residual
    assert pol.relative_dual_residual <= 1e-8
    assert pol.iterations == loose.iterations and pol.stats["feasibility_iteration"] > 0
    tight = O.solve_lp(d, {"eps": 1e-9, "l_inf_ruiz_iterations": 4, "feasibility_polishing": True,
                           "eps_feas_polish": 1e-6})
    assert tight.stats["polish_status"] == (None, None) and tight.stats["feasibility_iteration"] == 0


def test_oracle_restart_three_point():
    """Restart target selection with the plain Halpern point as a third
    candidate (LP/CP_AL/src/solver.cu:2749-2819, 3043-3075): on this
    instance the plain Halpern point wins one restart, the solve reaches
    HiGHS's optimum, and the selection stays off before its minimum
    iteration count or time."""
    d = I.random_lp(300, 700, 6, seed=3)
    prm = {"eps": 1e-8, "l_inf_ruiz_iterations": 4, "reflection_coefficient": 0.5}
    r = O.solve_lp(d, prm, {"restart_select": 3})
    assert r.status == "OPTIMAL"
    assert r.stats["restart_targets"][2] >= 1
    f = highs_objective(d)
    assert abs(r.primal_objective - f) <= 1e-6 * (1 + abs(f))
    # the three-point switch with mode 1 is mode 3
    r1 = O.solve_lp(d, prm, {"restart_select": 1, "restart_select_threepoint": 1})
    assert (r1.iterations, r1.stats["restart_targets"]) == (r.iterations, r.stats["restart_targets"])
    plain = O.solve_lp(d, prm)
    for gate in ({"restart_select_min_iters": 10**8}, {"restart_select_min_time": 1e9}):
        g = O.solve_lp(d, prm, {"restart_select": 3, **gate})
        assert g.stats["restart_targets"][1:] == (0, 0)
        assert g.iterations == plain.iterations


def test_oracle_curtis_reid():
    """Curtis-Reid scaling before Ruiz (LP/CP_AL/src/preconditioner.cu:162-270,
    553-624): on a badly scaled LP its passes shrink the spread of log|a| of
    the scaled matrix to a fraction, early stop ends them after the fifth pass
    when the threshold allows it and never otherwise, and a solve with it
    reaches HiGHS's optimum."""
    d = I.zipf_lp(400, 900, nnz=6000, seed=3, max_row=300)
    base = {"l_inf_ruiz_iterations": 0, "has_pock_chambolle_alpha": False, "bound_objective_rescaling": False}
    raw = np.log10(np.abs(d.csr()[2]))
    *_, sv, p20 = O.rescale(d, base, {"cr_iterations": 20}, with_passes=True)
    assert p20 == 20
    assert np.log10(np.abs(sv)).std() < 0.3 * raw.std()
    *_, p5 = O.rescale(d, base, {"cr_iterations": 20, "cr_early_stop": 1, "cr_early_stop_threshold": 1e9},
                       with_passes=True)
    *_, pn = O.rescale(d, base, {"cr_iterations": 20, "cr_early_stop": 1, "cr_early_stop_threshold": -1.0},
                       with_passes=True)
    *_, p7 = O.rescale(d, base, {"cr_iterations": 7, "cr_early_stop": 1, "cr_early_stop_threshold": 1e9},
                       with_passes=True)
    assert (p5, pn, p7) == (5, 20, 7)
    case = I.random_lp(300, 700, 6, seed=21)
    res = O.solve_lp(case, {"eps": 1e-8, "l_inf_ruiz_iterations": 4}, {"cr_iterations": 20})
    f = highs_objective(case)
    assert res.status == "OPTIMAL" and abs(res.primal_objective - f) <= 1e-6 * (1 + abs(f))


@pytest.mark.parametrize("options", [
    {"restart_select": 1}, {"restart_select": 2}, {"restart_select": 3},
    {"restart_select": 1, "restart_select_margin": 0.9}, {"restart_select": 3, "al_lambda": 0.0},
], ids=["select1", "select2", "select3", "select1_margin", "select3_lambda0"])
def test_oracle_restart_selection_reaches_optimum(options):
    """Every restart target selection mode of the oracle
    (LP/CP_AL/src/solver.cu:2749-2819) still solves to HiGHS's optimum."""
    for d in (I.random_lp(300, 700, 6, seed=21), I.transport_lp(15, 12, seed=5)):
        r = O.solve_lp(d, {"eps": 1e-8, "l_inf_ruiz_iterations": 4, "reflection_coefficient": 0.5}, options)
        f = highs_objective(d)
        assert r.status == "OPTIMAL" and abs(r.primal_objective - f) <= 1e-6 * (1 + abs(f))


def test_oracle_curtis_reid_without_constraints():
    """Curtis-Reid on an LP without constraints: every scale stays 1 and early
    stop ends the passes after the fifth (the reference's maximum over no
    rows is the lowest double)."""
    n = 50
    d = LPData(np.linspace(-1, 1, n), (np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), (0, n)),
               np.zeros(0), np.zeros(0), np.zeros(n), np.full(n, 3.0))
    base = {"l_inf_ruiz_iterations": 0, "has_pock_chambolle_alpha": False, "bound_objective_rescaling": False}
    _, c, _, _, _, p = O.rescale(d, base, {"cr_iterations": 20, "cr_early_stop": 1}, with_passes=True)
    assert p == 5 and np.all(c == 1.0)
    *_, p20 = O.rescale(d, base, {"cr_iterations": 20}, with_passes=True)
    assert p20 == 20


def _highs_status(d):
    """HiGHS on the same LP: 0 optimal, 2 infeasible, 3 unbounded."""
    rp, ci, v, (m, n) = d.csr()
    A = sp.csr_matrix((v, ci, rp), shape=(m, n))
    lo, hi = np.asarray(d.con_lb), np.asarray(d.con_ub)
    eq = lo == hi
    ub_rows, lb_rows = np.isfinite(hi) & ~eq, np.isfinite(lo) & ~eq
    r = linprog(d.c, A_ub=sp.vstack([A[ub_rows], -A[lb_rows]]), b_ub=np.concatenate([hi[ub_rows], -lo[lb_rows]]),
                A_eq=A[eq], b_eq=lo[eq],
                bounds=[(l, u if np.isfinite(u) else None) for l, u in zip(d.var_lb, d.var_ub)], method="highs")
    return r.status


@pytest.mark.parametrize("kind,status,highs", [("primal", "PRIMAL_INFEASIBLE", 2), ("dual", "DUAL_INFEASIBLE", 3)])
@pytest.mark.parametrize("seed", [3, 8])
def test_oracle_infeasibility_detection(kind, status, highs, seed):
    """Opt-in certificates (the reference's utils.cu:281-297 tests on the
    displacement from the restart anchor): an infeasible LP stops with the
    status HiGHS confirms, with a certificate that passes the tolerance;
    without the option it runs to its iteration limit, as the reference's
    solver does."""
    d = I.infeasible_lp(kind, seed=seed)
    assert _highs_status(d) == highs
    p = {"eps": 1e-8, "iteration_limit": 20_000}
    on = O.solve_lp(d, p, {"infeasibility_detection": 1})
    off = O.solve_lp(d, p, {"infeasibility_detection": 0})
    assert on.status == status and on.iterations < 20_000
    assert off.status == "ITERATION_LIMIT"
    s = on.stats
    if kind == "primal":
        assert s["dual_ray_objective"] > 0
        assert s["max_dual_ray_infeasibility"] / s["dual_ray_objective"] <= 1e-8
    else:
        assert s["primal_ray_linear_objective"] < 0
        assert s["max_primal_ray_infeasibility"] / -s["primal_ray_linear_objective"] <= 1e-8


def test_oracle_infeasibility_detection_leaves_feasible_solves_alone():
    d = I.random_lp(300, 800, 6, seed=21)
    a = O.solve_lp(d, {"eps": 1e-8}, {"infeasibility_detection": 0})
    b = O.solve_lp(d, {"eps": 1e-8}, {"infeasibility_detection": 1})
    assert a.status == b.status == "OPTIMAL" and a.iterations == b.iterations
    assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)
