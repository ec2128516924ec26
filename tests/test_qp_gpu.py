"""FA_CP (convex QP) on the GPU through the C-ABI library, against the CPU
oracle and the known answers.

Tolerances: both sides compute in FP64 with different summation orders, so
iterates agree to ~1e-12 relative per step; after hundreds of iterations and
a few restart decisions the fixed-iteration iterates are compared at 1e-7
(relative to the vector's scale), objective values at the requested
tolerance, iteration counts exactly where both stop at the same evaluation.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O
from pdal_gb300 import qp
from pdal_gb300.instances import planted_qp, random_lp
from pdal_gb300.qp import QPData
from test_oracle_qp import A3, INF, docs_diag_qp, docs_lowrank_qp

pytestmark = pytest.mark.gpu


def both(data, params):
    g = qp.solve(data, {**params, "verbose": 0})
    o = O.solve_qp(data, params)
    return g, o


@pytest.mark.parametrize("make,f", [(docs_diag_qp, -20.0 / 3.0), (docs_lowrank_qp, -8.0)])
def test_docs_examples(make, f):
    g, o = both(make(), {"eps": 1e-9})
    assert g.status == o.status == "OPTIMAL"
    assert abs(g.primal_objective - f) < 1e-7 * abs(f)
    np.testing.assert_allclose(g.x, [2 / 3, 4 / 3], atol=1e-7)
    assert g.iterations == o.iterations


def test_model_interface_solves_readme_example():
    from pdal_gb300.fa_cp import FA_CP, Model

    m = Model(objective_matrix=sp.csc_matrix([[1.0, -1.0], [-1.0, 2.0]]),
              objective_matrix_low_rank=sp.csc_matrix([[1.0, 0.0]]), objective_vector=np.array([-2.0, -6.0]),
              constraint_matrix=sp.csc_matrix(A3), constraint_lower_bound=np.full(3, -INF),
              constraint_upper_bound=np.array([2.0, 2.0, 3.0]), variable_lower_bound=np.zeros(2),
              variable_upper_bound=np.full(2, INF))
    m.setParams(LogLevel=0, OptimalityTol=1e-8, FeasibilityTol=1e-8)
    m.optimize()
    assert m.Status == "OPTIMAL" and m.StatusCode == FA_CP.OPTIMAL
    assert abs(m.ObjVal + 8.0) < 1e-6
    np.testing.assert_allclose(m.X, [2 / 3, 4 / 3], atol=1e-6)
    # MAXIMIZE flips the sign of c and c0 only (QP/FA_CP/python/fa_cp/model.py:500-553)
    m.ModelSense = FA_CP.MAXIMIZE
    m.setObjectiveVector(np.array([2.0, 6.0]))
    m.optimize()
    assert m.Status == "OPTIMAL" and abs(m.ObjVal - 8.0) < 1e-6
    np.testing.assert_allclose(m.X, [2 / 3, 4 / 3], atol=1e-6)


@pytest.mark.parametrize("form", ["sparse", "lowrank"])
def test_planted_qp_matches_oracle(form):
    data, xs, fs = planted_qp(n=3000, m=1500, b_rows=750, seed=21, q_form=form)
    g, o = both(data, {"eps": 1e-7})
    assert g.status == o.status == "OPTIMAL"
    assert abs(g.primal_objective - fs) <= 1e-5 * (1 + abs(fs))
    assert abs(g.iterations - o.iterations) <= 0.05 * o.iterations + 10
    assert g.inner_iterations > 0


@pytest.mark.parametrize("form,al_sigma", [("sparse", 0.0), ("lowrank", 0.0), ("sparse", 0.3)])
def test_fixed_iterations_track_oracle(form, al_sigma):
    """Same seed, same iteration budget: the iterates agree."""
    data, _, _ = planted_qp(n=800, m=400, b_rows=200, seed=3, q_form=form)
    prm = {"eps": 1e-14, "iteration_limit": 600, "al_sigma": al_sigma,
           "sigma_update_rule": "fixed" if al_sigma else "guarded"}
    g, o = both(data, prm)
    assert g.iterations == o.iterations == 600
    sx = 1 + np.abs(o.x).max()
    sy = 1 + np.abs(o.y).max()
    assert np.abs(g.x - o.x).max() <= 1e-7 * sx
    assert np.abs(g.y - o.y).max() <= 1e-7 * sy
    assert abs(g.inner_iterations - o.inner_iterations) <= 0.02 * o.inner_iterations + 5


def test_lp_through_fa_cp_matches_oracle():
    d = random_lp(m=400, n=1000, nnz_per_col=5, seed=9)
    q = QPData(c=d.c, A=d.csr(), con_lb=d.con_lb, con_ub=d.con_ub, var_lb=d.var_lb, var_ub=d.var_ub)
    g, o = both(q, {"eps": 1e-8})
    assert g.status == o.status == "OPTIMAL"
    assert abs(g.primal_objective - o.primal_objective) <= 1e-7 * (1 + abs(o.primal_objective))
    assert abs(g.iterations - o.iterations) <= 0.05 * o.iterations + 10
    g2, o2 = both(q, {"eps": 1e-14, "iteration_limit": 500})
    assert np.abs(g2.x - o2.x).max() <= 1e-8 * (1 + np.abs(o2.x).max())


@pytest.mark.parametrize("rule", ["residual_balance", "kkt_balance", "displacement", "progress", "greedy_score",
                                  "balanced_guarded"])
def test_sigma_rules_match_oracle(rule):
    data, _, fs = planted_qp(n=600, m=300, b_rows=150, seed=5, q_form="sparse")
    prm = {"eps": 1e-7, "al_sigma": 0.1, "sigma_update_rule": rule}
    g, o = both(data, prm)
    assert g.status == o.status
    assert abs(g.sigma_update_count - o.sigma_update_count) <= 2
    if o.status == "OPTIMAL":
        assert abs(g.primal_objective - fs) <= 1e-5 * (1 + abs(fs))


def test_infeasibility_detection():
    d = QPData(c=np.array([1.0, 1.0]), A=np.array([[1.0, 1.0]]), con_lb=np.array([-INF]), con_ub=np.array([-1.0]),
               var_lb=np.zeros(2), var_ub=np.full(2, INF), Q=np.eye(2))
    g, o = both(d, {"eps": 1e-8, "iteration_limit": 20000})
    assert g.status == o.status == "PRIMAL_INFEASIBLE"
    d = QPData(c=np.array([-1.0, -1.0]), A=np.array([[1.0, -1.0]]), con_lb=np.array([0.0]), con_ub=np.array([0.0]),
               var_lb=np.zeros(2), var_ub=np.full(2, INF))
    g, o = both(d, {"eps": 1e-8, "iteration_limit": 20000})
    assert g.status == o.status == "DUAL_INFEASIBLE"


def test_long_rows_and_columns():
    """A dense row and a dense column longer than one row block (1,024), and
    a dense row of Q."""
    rng = np.random.default_rng(4)
    n, m = 3000, 200
    A = sp.random(m, n, density=0.003, random_state=5, format="lil")
    A[0, :] = rng.standard_normal(n)
    A = A.tocsr()
    Acol = sp.random(2500, n, density=0.002, random_state=6, format="lil")
    Acol[:, 7] = rng.standard_normal((2500, 1))
    A = sp.vstack([A, Acol.tocsr()]).tocsr()
    m = A.shape[0]
    B = sp.random(400, n, density=0.002, random_state=7, format="lil")
    B[3, :] = rng.standard_normal(n) * 0.1
    Q = (B.T @ B + sp.diags(rng.random(n) + 0.1)).tocsr()
    x = rng.uniform(-1, 1, n)
    Ax = A @ x
    data = QPData(c=rng.standard_normal(n), A=A, con_lb=Ax - 1.0, con_ub=Ax + 1.0, var_lb=-np.ones(n) * 3,
                  var_ub=np.ones(n) * 3, Q=Q)
    g, o = both(data, {"eps": 1e-14, "iteration_limit": 400})
    assert np.abs(g.x - o.x).max() <= 1e-7 * (1 + np.abs(o.x).max())
    assert np.abs(g.y - o.y).max() <= 1e-7 * (1 + np.abs(o.y).max())


def test_box_only_and_warm_start():
    rng = np.random.default_rng(8)
    n = 500
    Q = sp.diags(rng.random(n) + 0.5).tocsr() + sp.random(n, n, density=0.002, random_state=1) * 0.01
    Q = ((Q + Q.T) * 0.5).tocsr()
    data = QPData(c=rng.standard_normal(n), Q=Q, var_lb=-np.ones(n), var_ub=np.ones(n))
    g, o = both(data, {"eps": 1e-9})
    assert g.status == o.status == "OPTIMAL"
    assert abs(g.primal_objective - o.primal_objective) <= 1e-7 * (1 + abs(o.primal_objective))
    d2, _, _ = planted_qp(n=600, m=300, b_rows=150, seed=12, q_form="sparse")
    cold, _ = both(d2, {"eps": 1e-8})
    d2.primal_start, d2.dual_start = cold.x, cold.y
    g, o = both(d2, {"eps": 1e-8})
    assert g.status == o.status == "OPTIMAL" and g.iterations <= cold.iterations
    assert g.iterations == o.iterations


def test_restart_select_halpern_matches_oracle_objective():
    data, _, fs = planted_qp(n=600, m=300, b_rows=150, seed=13, q_form="sparse")
    g = qp.solve(data, {"eps": 1e-7, "verbose": 0}, {"restart_select": 1})
    assert g.status == "OPTIMAL" and abs(g.primal_objective - fs) <= 1e-5 * (1 + abs(fs))


def test_deterministic_repeat():
    data, _, _ = planted_qp(n=2000, m=1000, b_rows=500, seed=17, q_form="sparse")
    a = qp.solve(data, {"eps": 1e-6, "verbose": 0})
    b = qp.solve(data, {"eps": 1e-6, "verbose": 0})
    assert a.iterations == b.iterations and np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)


def _diag_qp(n=3000, m=1200, seed=5):
    rng = np.random.default_rng(seed)
    A = sp.random(m, n, density=8.0 / m, random_state=seed, format="csr") * 10.0 ** rng.uniform(-2, 2)
    Q = sp.diags(rng.uniform(1e-3, 10.0, n)).tocsr()
    b = A @ rng.uniform(-1, 1, n)
    return QPData(rng.standard_normal(n) * 100, A, b - 1.0, b + np.where(rng.random(m) < 0.5, 0.0, np.inf),
                  np.full(n, -5.0), np.where(rng.random(n) < 0.1, np.inf, 5.0), Q=Q)


@pytest.mark.parametrize("case", ["sparse", "lowrank", "diag", "lp", "pc_half"])
def test_device_equilibration_is_bit_identical_to_oracle(case):
    """The device equilibration (Ruiz passes, Pock-Chambolle, bound/objective
    scaling) gives the oracle's scale vectors bit for bit (the oracle follows
    QP/FA_CP/src/preconditioner.c:92-331); with alpha = 0.5 the |a|^alpha
    terms go through pow(), whose last bit may differ between the device and
    the host library, so that case is compared at 1e-14."""
    params = {"l_inf_ruiz_iterations": 10}
    if case in ("sparse", "lowrank", "pc_half"):
        data, _, _ = planted_qp(n=4000, m=2000, b_rows=1000, seed=31, q_form="lowrank" if case == "lowrank" else "sparse")
    elif case == "diag":
        data = _diag_qp()
    else:
        d = random_lp(800, 2000, 6, seed=4)
        data = QPData(d.c, d.A, d.con_lb, d.con_ub, d.var_lb, d.var_ub)
    if case == "pc_half":
        params["pock_chambolle_alpha"] = 0.5
    g = qp.scaling(data, params)
    o = O.qp_scaling(data, params)
    for a, b in zip(g, o):
        if case == "pc_half":
            np.testing.assert_allclose(a, b, rtol=1e-14, atol=0)
        else:
            assert np.array_equal(np.asarray(a), np.asarray(b)), case


@pytest.mark.parametrize("form", ["sparse", "lowrank", "diag", "lp"])
def test_fp32_refine_reaches_fp64_tolerance(form):
    """Chosen form: FP32 iteration segments (FP64 reductions, evaluation and
    control), then FP64 from the FP32 iterate.  It meets the same relative KKT
    tolerance as the FP64 solve, and two solutions that each meet 1e-8 along
    different trajectories agree in objective to that tolerance."""
    if form in ("sparse", "lowrank"):
        data, _, f_star = planted_qp(n=3000, m=1500, b_rows=750, seed=41, q_form=form)
    elif form == "diag":
        data, f_star = _diag_qp(n=3000, m=1200, seed=7), None
    else:
        d = random_lp(800, 2000, 6, seed=9)
        data, f_star = QPData(d.c, d.A, d.con_lb, d.con_ub, d.var_lb, d.var_ub), None
    params = {"eps": 1e-8, "verbose": 0, "iteration_limit": 200_000}
    g64 = qp.solve(data, params)
    g32 = qp.solve(data, params, {"precision": "fp32_refine"})
    assert g64.status == g32.status == "OPTIMAL"
    assert g32.kkt < 1e-8 and g32.stats["fp32_iterations"] > 0
    assert abs(g32.primal_objective - g64.primal_objective) <= 5e-8 * (1 + abs(g64.primal_objective))
    if f_star is not None:
        assert abs(g32.primal_objective - f_star) <= 1e-7 * (1 + abs(f_star))


def test_grid_barrier_wait_runs_out_and_recovers(qp_lib):
    """Failure detection without a GPU fault: every grid barrier of the
    persistent kernel is told to wait for one block more than the launch has,
    with a short poll limit, so each wait runs out; the kernel records the
    error and returns, the solve fails with a message instead of hanging, and
    the next solve on the same context succeeds."""
    qd, _, f_star = planted_qp(n=400, m=200, b_rows=100, seed=23, q_form="sparse")
    bad = {"device": 0, "barrier_extra_arrivals": 1, "barrier_spin_limit": 1 << 12}
    with pytest.raises(RuntimeError, match="grid barrier"):
        qp.solve(qd, {"eps": 1e-8, "verbose": 0}, bad)
    g = qp.solve(qd, {"eps": 1e-8, "verbose": 0}, {"device": 0})
    assert g.status == "OPTIMAL"
    assert abs(g.primal_objective - f_star) <= 1e-6 * (1 + abs(f_star))


@pytest.mark.parametrize("gen", [("random_lp", {"m": 300, "n": 800, "nnz_per_col": 6, "seed": 17}),
                                 ("transport_lp", {"supplies": 20, "demands": 20, "seed": 4001})],
                         ids=["random_lp", "transport"])
def test_feasibility_polishing_matches_oracle(qp_lib, gen):
    """FA_CP feasibility polishing of an LP solved through FA_CP
    (fa_cp_core_op.cu:1241-1735): both phases on the device against the
    oracle's restatement -- same phase statuses and iteration count, the
    polished residuals, objectives and solutions."""
    import ref_cases as RC

    d = RC.make_instance(gen, "qp")
    p = {"eps": 1e-4, "feasibility_polishing": True, "eps_feas_polish": 1e-8, "verbose": 0}
    g = qp.solve(d, p, {"device": 0})
    o = O.solve_qp(d, p)
    assert g.status == o.status == "OPTIMAL" and g.iterations == o.iterations
    assert (g.stats["polish_primal_status"], g.stats["polish_dual_status"]) == o.stats["polish_status"] == (7, 7)
    assert g.stats["feasibility_iteration"] == o.stats["feasibility_iteration"] > 0
    assert g.relative_primal_residual <= 1e-8 and g.relative_dual_residual <= 1e-8
    for a, b in ((g.primal_objective, o.primal_objective), (g.dual_objective, o.dual_objective)):
        assert abs(a - b) <= 1e-9 * (1 + abs(b))
    assert np.abs(g.x - o.x).max() <= 1e-9 * (1 + np.abs(o.x).max())
    assert np.abs(g.y - o.y).max() <= 1e-9 * (1 + np.abs(o.y).max())


def test_feasibility_polishing_skips_qps(qp_lib, capfd):
    """A QP is solved without the polishing phases, with a warning."""
    d, _, _ = planted_qp(n=400, m=200, b_rows=100, seed=23, q_form="sparse")
    g = qp.solve(d, {"eps": 1e-6, "feasibility_polishing": True, "verbose": 0}, {"device": 0})
    assert g.status == "OPTIMAL" and g.stats["feasibility_iteration"] == 0
    assert g.stats["polish_primal_status"] == g.stats["polish_dual_status"] == -1
    assert "built for problems without Q" in capfd.readouterr().err
