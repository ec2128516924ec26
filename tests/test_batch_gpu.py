"""The batched CP_AL solver (one persistent launch over many LPs) against the
single-instance GPU solver and the CPU oracle, instance by instance.

Both GPU paths run the same FP64 arithmetic on the same row-block products;
only the order of the reductions differs (block slots vs one block), so the
termination status and iteration count agree and objectives agree to 1e-9
relative; against the oracle the bar is the one the single solver meets
(objective 1e-8 relative, iterations within 2%)."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O
from pdal_gb300 import lp
from pdal_gb300.instances import batch_lps, random_lp
from pdal_gb300.lp import LPData

pytestmark = pytest.mark.gpu

SIGMA = {"sigma_mode": 1, "sigma_adaptive": 1, "sigma_init_factor": 0.5, "sigma_min_factor": 1e-4,
         "sigma_max_factor": 100.0, "sigma_balance_gain": 0.0, "sigma_kp": 0.5, "sigma_ki": 0.0, "sigma_kd": 0.0,
         "sigma_update_min": 1e-6, "sigma_update_max": 1e6, "lambda_factor": 2.01, "al_lambda": 0.0,
         "restart_sufficient": 0.2, "restart_necessary": 0.8, "restart_artificial": 0.36}


def long_row_lp(seed=2):
    """A dense row and a dense column, both longer than one row block."""
    rng = np.random.default_rng(seed)
    m, n = 300, 2500
    A = sp.random(m, n, density=0.004, random_state=seed, format="lil")
    A[0, :] = rng.standard_normal(n)
    A[:, 5] = rng.standard_normal((m, 1))
    A = A.tocsr()
    x0 = rng.uniform(0, 5, n)
    b = A @ x0
    y0 = rng.standard_normal(m)
    c = A.T @ y0 + rng.random(n)
    return LPData(c, A, b, b.copy(), np.zeros(n), np.full(n, 10.0))


@pytest.mark.parametrize("options", [{}, SIGMA], ids=["default", "sigma_protocol"])
def test_batch_matches_single_solver(options):
    items = batch_lps(count=20, seed=77, m_range=(50, 700)) + [long_row_lp()]
    params = {"eps": 1e-8, "l_inf_ruiz_iterations": 4, "iteration_limit": 200000}
    res, st = lp.solve_batch(items, params, options)
    assert st["instances"] == len(items) and st["grid_blocks"] > 0
    for d, b in zip(items, res):
        s = lp.solve(d, params, options)
        assert b.status == s.status == "OPTIMAL"
        assert abs(b.iterations - s.iterations) <= 0.02 * s.iterations, (b.iterations, s.iterations)
        assert abs(b.primal_objective - s.primal_objective) <= 1e-8 * (1 + abs(s.primal_objective))
        assert np.abs(b.x - s.x).max() <= 1e-5 * (1 + np.abs(s.x).max())
    its = sorted(r.iterations for r in res)
    assert st["iterations_max"] == its[-1] and st["optimal"] == len(items)


def test_batch_matches_oracle():
    items = batch_lps(count=6, seed=5, m_range=(60, 300))
    params = {"eps": 1e-8, "l_inf_ruiz_iterations": 4, "iteration_limit": 200000}
    res, _ = lp.solve_batch(items, params)
    for d, b in zip(items, res):
        o = O.solve_lp(d, params)
        assert b.status == o.status == "OPTIMAL"
        assert abs(b.primal_objective - o.primal_objective) <= 1e-8 * (1 + abs(o.primal_objective))
        assert abs(b.iterations - o.iterations) <= 0.02 * o.iterations


def test_batch_handles_iteration_limit_and_warm_start():
    items = batch_lps(count=4, seed=8, m_range=(80, 200))
    res, st = lp.solve_batch(items, {"eps": 1e-12, "iteration_limit": 400})
    assert all(r.status == "ITERATION_LIMIT" and r.iterations == 400 for r in res)
    cold, _ = lp.solve_batch(items, {"eps": 1e-8, "iteration_limit": 200000})
    for d, r in zip(items, cold):
        d.primal_start, d.dual_start = r.x, r.y
    warm, _ = lp.solve_batch(items, {"eps": 1e-8, "iteration_limit": 200000})
    assert all(w.status == "OPTIMAL" and w.iterations <= c.iterations for w, c in zip(warm, cold))


def test_batch_fp32_refine_matches_single_solver():
    """Chosen form: FP32 phase with FP64 anchors/evaluation, then FP64
    refinement; the result meets the FP64 tolerance and agrees with the
    single-instance FP32_REFINE solve."""
    items = batch_lps(count=12, seed=31, m_range=(80, 600)) + [long_row_lp(3)]
    params = {"eps": 1e-8, "l_inf_ruiz_iterations": 4, "iteration_limit": 200000}
    opts = {"precision": "fp32_refine"}
    res, st = lp.solve_batch(items, params, opts)
    for d, b in zip(items, res):
        s = lp.solve(d, params, opts)
        o = lp.solve(d, params)
        assert b.status == s.status == "OPTIMAL"
        assert b.kkt < 1e-8
        # two solutions that each meet relative KKT 1e-8 along different
        # trajectories agree in objective to the tolerance, not beyond it
        assert abs(b.primal_objective - o.primal_objective) <= 5e-8 * (1 + abs(o.primal_objective))
        assert abs(b.primal_objective - s.primal_objective) <= 5e-8 * (1 + abs(s.primal_objective))
        # FP32 trajectories depend on the reduction order, so the iteration
        # counts of the two FP32 paths differ; both run an FP32 phase
        assert b.stats["fp32_iterations"] > 0


def test_schedule_autotuner_and_fixed_schedules():
    """Every schedule solves the batch to the same optimum; with no schedule
    given the autotuner times the candidates once per batch shape and then
    reuses its choice."""
    items = batch_lps(count=40, seed=91, m_range=(100, 1500))
    params = {"eps": 1e-7, "l_inf_ruiz_iterations": 4, "iteration_limit": 200000}
    ref = None
    for bs, mb in ((2048, 2), (2048, 3), (1024, 2), (1024, 3), (1024, 4)):
        res, st = lp.solve_batch(items, params, {"spmv_nnz_per_block": bs, "batch_blocks_per_sm": mb})
        assert (st["block_nnz"], st["blocks_per_sm"]) == (bs, mb) and st["tune_sec"] == 0.0
        assert st["optimal"] == len(items)
        obj = np.array([r.primal_objective for r in res])
        if ref is None:
            ref = obj
        np.testing.assert_allclose(obj, ref, rtol=2e-7)
    res, st = lp.solve_batch(items, params)
    assert (st["block_nnz"], st["blocks_per_sm"]) in {(2048, 2), (2048, 3), (1024, 2), (1024, 3), (1024, 4)}
    assert st["tune_sec"] > 0.0 and st["optimal"] == len(items)
    res2, st2 = lp.solve_batch(items, params)
    assert st2["tune_sec"] == 0.0 and (st2["block_nnz"], st2["blocks_per_sm"]) == (st["block_nnz"], st["blocks_per_sm"])
    other = batch_lps(count=41, seed=92, m_range=(100, 1500))
    t = lp.tune_batch(other, params)
    assert t["tune_sec"] > 0.0
    _, st3 = lp.solve_batch(other, params)
    assert st3["tune_sec"] == 0.0 and (st3["block_nnz"], st3["blocks_per_sm"]) == (t["block_nnz"], t["blocks_per_sm"])
    with pytest.raises(RuntimeError):
        lp.solve_batch(items, params, {"spmv_nnz_per_block": 2048, "batch_blocks_per_sm": 4})


@pytest.mark.parametrize("opts", [{"restart_select": 1}, {"cr_iterations": 5}, {"alpha_direct_pulse": 1},
                                  {"sigma_trigger": 1}, {"dynamic_eval": 1}, {"dynamic_eval_after_iters": 400}],
                         ids=["restart_select", "curtis_reid", "pulse", "trigger", "dynamic_eval", "dynamic_eval_iters"])
def test_batch_refuses_single_solve_options(lp_lib, opts):
    """Options the batched launch cannot honour are refused with a message
    (an error, not a silent skip): restart target selection, Curtis-Reid
    scaling, and the benchmark controllers whose step or block-length changes
    would switch the kernel form a batch launch fixes."""
    items = [random_lp(30, 60, 3, seed=s) for s in range(2)]
    with pytest.raises(RuntimeError, match="not supported by the batched solver"):
        lp.solve_batch(items, {"eps": 1e-6}, {"device": 0, **opts})
