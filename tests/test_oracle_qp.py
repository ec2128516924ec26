"""The FA_CP oracle (CPU restatement of QP/FA_CP) against known answers, and
the host-side QP interface of libfa_cp_gb300.so (no GPU needed).

Known answers: the two small QPs of the reference's documentation
(QP/FA_CP/docs/C_API.md:45-123 and QP/FA_CP/README.md:223-268) have
closed-form optima (active constraints 1 and 2); planted QPs have an optimum
that satisfies the KKT conditions by construction; LPs solved through FA_CP
are checked against scipy's HiGHS."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O
from pdal_gb300 import _native as N
from pdal_gb300.instances import planted_qp, random_lp
from pdal_gb300.qp import QPData

INF = np.inf
A3 = np.array([[1.0, 1.0], [-1.0, 2.0], [2.0, 1.0]])


def docs_diag_qp():
    """min 1/2(4x0^2 + 2x1^2) - 2x0 - 6x1, Ax <= (2, 2, 3), x >= 0; optimum
    x = (2/3, 4/3), f = -20/3, duals (-2/3, -4/3, 0)."""
    return QPData(c=np.array([-2.0, -6.0]), A=A3, con_lb=np.full(3, -INF), con_ub=np.array([2.0, 2.0, 3.0]),
                  var_lb=np.zeros(2), var_ub=np.full(2, INF), Q=np.diag([4.0, 2.0]))


def docs_lowrank_qp():
    """Q = [[1,-1],[-1,2]] plus R = [[1,0]] (so Q + R'R = [[2,-1],[-1,2]]),
    same constraints; optimum x = (2/3, 4/3), f = -8, duals (-8/3, -2/3, 0)."""
    return QPData(c=np.array([-2.0, -6.0]), A=sp.csc_matrix(A3), con_lb=np.full(3, -INF),
                  con_ub=np.array([2.0, 2.0, 3.0]), var_lb=np.zeros(2), var_ub=np.full(2, INF),
                  Q=sp.csc_matrix([[1.0, -1.0], [-1.0, 2.0]]), R=sp.csc_matrix([[1.0, 0.0]]))


@pytest.mark.parametrize("make,f,x,y", [
    (docs_diag_qp, -20.0 / 3.0, [2 / 3, 4 / 3], [-2 / 3, -4 / 3, 0.0]),
    (docs_lowrank_qp, -8.0, [2 / 3, 4 / 3], [-8 / 3, -2 / 3, 0.0]),
])
def test_oracle_docs_examples(make, f, x, y):
    r = O.solve_qp(make(), {"eps": 1e-9})
    assert r.status == "OPTIMAL"
    assert abs(r.primal_objective - f) < 1e-7 * abs(f)
    np.testing.assert_allclose(r.x, x, atol=1e-7)
    np.testing.assert_allclose(r.y, y, atol=1e-6)


def test_oracle_sparse_q_only_and_r_only_agree():
    """The same objective as sparse Q, as R'R, and as Q + R'R."""
    B = np.array([[1.0, 2.0, 0.0], [0.0, 1.0, -1.0]])
    Qfull = B.T @ B + np.eye(3) * 0.5
    base = dict(c=np.array([1.0, -2.0, 0.5]), A=np.array([[1.0, 1.0, 1.0]]), con_lb=np.array([1.0]),
                con_ub=np.array([1.0]), var_lb=-np.ones(3) * 5, var_ub=np.ones(3) * 5)
    r1 = O.solve_qp(QPData(Q=sp.csr_matrix(Qfull), **base), {"eps": 1e-9})
    r2 = O.solve_qp(QPData(Q=sp.csr_matrix(np.eye(3) * 0.5), R=sp.csr_matrix(B), **base), {"eps": 1e-9})
    # closed form: KKT of the equality-constrained QP (box inactive)
    K = np.block([[Qfull, np.ones((3, 1))], [np.ones((1, 3)), np.zeros((1, 1))]])
    sol = np.linalg.solve(K, np.r_[-base["c"], 1.0])
    for r in (r1, r2):
        assert r.status == "OPTIMAL"
        np.testing.assert_allclose(r.x, sol[:3], atol=1e-6)


@pytest.mark.parametrize("form", ["sparse", "lowrank"])
def test_oracle_planted_qp(form):
    data, xs, fs = planted_qp(n=600, m=300, b_rows=150, seed=11, q_form=form)
    r = O.solve_qp(data, {"eps": 1e-8})
    assert r.status == "OPTIMAL"
    assert abs(r.primal_objective - fs) <= 1e-6 * (1 + abs(fs))
    assert r.inner_iterations > 0


def test_oracle_lp_through_fa_cp_matches_highs():
    from scipy.optimize import linprog

    d = random_lp(m=60, n=150, nnz_per_col=4, seed=5)
    rp, ci, v, (m, n) = d.csr()
    A = sp.csr_matrix((v, ci, rp), shape=(m, n))
    q = QPData(c=d.c, A=(rp, ci, v, (m, n)), con_lb=d.con_lb, con_ub=d.con_ub, var_lb=d.var_lb, var_ub=d.var_ub)
    r = O.solve_qp(q, {"eps": 1e-8})
    eq = np.isfinite(d.con_lb)
    h = linprog(d.c, A_ub=A[~eq], b_ub=d.con_ub[~eq], A_eq=A[eq], b_eq=d.con_ub[eq],
                bounds=list(zip(d.var_lb, d.var_ub)), method="highs")
    assert r.status == "OPTIMAL"
    assert abs(r.primal_objective - h.fun) <= 1e-6 * (1 + abs(h.fun))


def test_oracle_detects_primal_infeasibility():
    # x0 + x1 <= -1 with x >= 0
    d = QPData(c=np.array([1.0, 1.0]), A=np.array([[1.0, 1.0]]), con_lb=np.array([-INF]), con_ub=np.array([-1.0]),
               var_lb=np.zeros(2), var_ub=np.full(2, INF), Q=np.eye(2))
    r = O.solve_qp(d, {"eps": 1e-8, "iteration_limit": 20000})
    assert r.status == "PRIMAL_INFEASIBLE"


def test_oracle_detects_dual_infeasibility():
    # min -x0 - x1 s.t. x0 - x1 = 0, x >= 0: unbounded along (1, 1)
    d = QPData(c=np.array([-1.0, -1.0]), A=np.array([[1.0, -1.0]]), con_lb=np.array([0.0]), con_ub=np.array([0.0]),
               var_lb=np.zeros(2), var_ub=np.full(2, INF))
    r = O.solve_qp(d, {"eps": 1e-8, "iteration_limit": 20000})
    assert r.status == "DUAL_INFEASIBLE"


def test_default_parameters_equal_reference_defaults(qp_lib):
    """Library and oracle restate QP/FA_CP/src/utils.cu:494-537 identically."""
    a = N.FacpParameters()
    qp_lib.set_default_parameters(C.byref(a))
    b = O.qp_default_parameters()
    assert bytes(a) == bytes(b)
    assert a.termination_criteria.eps_infeasible == 1e-10 and a.optimality_norm == N.NORM_LINF
    assert a.restart_params.necessary_reduction_for_restart == 0.8 and a.sigma_update_rule == 6


def test_rand_sequence_is_the_c_library_sequence(qp_lib):
    libc = C.CDLL(None)
    out = (C.c_int * 64)()
    for seed in (1, 7, 123456):
        qp_lib.fa_cp_gb300_rand_sequence(seed, 64, out)
        libc.srand(seed)
        assert list(out) == [libc.rand() for _ in range(64)]


def _read_component(P, which, rows):
    comp = getattr(P, which).contents
    nnz = getattr(P, {"constraint_matrix": "constraint_matrix_num_nonzeros",
                      "objective_sparse_matrix": "objective_sparse_matrix_num_nonzeros",
                      "objective_lowrank_matrix": "objective_lowrank_matrix_num_nonzeros"}[which])
    rp = np.ctypeslib.as_array(comp.row_ptr, shape=(rows + 1,)).copy()
    ci = np.ctypeslib.as_array(comp.col_ind, shape=(nnz,)).copy() if nnz else np.zeros(0, int)
    v = np.ctypeslib.as_array(comp.val, shape=(nnz,)).copy() if nnz else np.zeros(0)
    return rp, ci, v


def test_create_qp_problem_formats_and_zero_tolerance(qp_lib):
    """Dense input drops |a| <= 1e-12 (or zero_tolerance); CSC/COO drop only
    with a positive zero_tolerance; absent Q/R become empty matrices."""
    from pdal_gb300.fa_cp._core import _desc

    rng = np.random.default_rng(1)
    m, n = 5, 6
    A = rng.standard_normal((m, n)) * (rng.random((m, n)) < 0.5)
    A[0, 0] = 1e-13
    A[1, 1] = 1e-5
    keep = []
    want = sp.csr_matrix(np.where(np.abs(A) > 1e-12, A, 0.0))
    for M, tol, expect in [(A, 0.0, want), (sp.csc_matrix(A), 0.0, sp.csr_matrix(A)),
                           (sp.coo_matrix(A), 1e-4, sp.csr_matrix(np.where(np.abs(A) > 1e-4, A, 0.0)))]:
        d = _desc(M, tol, keep)
        p = qp_lib.create_qp_problem(None, None, None, C.byref(d), None, None, None, None, None)
        assert p
        P = p.contents
        assert (P.num_variables, P.num_constraints, P.num_rank_lowrank_obj) == (n, m, 0)
        rp, ci, v = _read_component(P, "constraint_matrix", m)
        got = sp.csr_matrix((v, ci, rp), shape=(m, n)).toarray()
        np.testing.assert_array_equal(got, expect.toarray())
        qrp, _, _ = _read_component(P, "objective_sparse_matrix", n)
        assert P.objective_sparse_matrix_num_nonzeros == 0 and not qrp.any()
        assert np.all(np.isneginf(np.ctypeslib.as_array(P.variable_lower_bound, shape=(n,))))
        qp_lib.qp_problem_free(p)
    # n from Q when A is absent, R rows give the rank
    dq = _desc(np.eye(3), 0.0, keep)
    dr = _desc(np.ones((2, 3)), 0.0, keep)
    p = qp_lib.create_qp_problem(None, C.byref(dq), C.byref(dr), None, None, None, None, None, None)
    assert p and p.contents.num_variables == 3 and p.contents.num_constraints == 0
    assert p.contents.num_rank_lowrank_obj == 2 and p.contents.objective_lowrank_matrix_num_nonzeros == 6
    qp_lib.qp_problem_free(p)
    assert not qp_lib.create_qp_problem(None, None, None, None, None, None, None, None, None)


def test_model_interface_host_side():
    """Parameter aliases and argument checks of fa_cp.Model (no solve)."""
    from pdal_gb300.fa_cp import FA_CP, Model

    m = Model(objective_vector=[1.0, 2.0], constraint_matrix=A3, constraint_upper_bound=[2, 2, 3],
              objective_matrix=np.eye(2))
    m.setParams(LogLevel=0, TimeLimit=10.0, OptimalityTol=1e-7)
    assert m.getParam("verbose") == 0 and m.Params.TimeLimit == 10.0 and m.Params["eps_optimal_relative"] == 1e-7
    with pytest.raises(ValueError):
        m.setConstraintLowerBound([0.0])
    with pytest.raises(ValueError):
        Model(objective_vector=[1.0], constraint_matrix=A3)
    with pytest.warns(RuntimeWarning):
        m.setWarmStart(primal=[1.0, 2.0, 3.0])
    assert m.X is None and FA_CP.MAXIMIZE == -1


def _reference_precond():
    """The reference's own FA_CP equilibration (QP/FA_CP/src/preconditioner.c),
    compiled unmodified by oracle/build.py (build_ref); skipped where the
    reference sources are absent."""
    from oracle import build as ob

    built = {p.name: p for p in ob.build_ref()}
    if "libref_facp_precond.so" not in built:
        pytest.skip("reference sources absent")
    lib = C.CDLL(str(built["libref_facp_precond.so"]))
    _dp = C.POINTER(C.c_double)
    lib.ref_facp_rescale.restype = C.c_int
    lib.ref_facp_rescale.argtypes = [C.POINTER(N.QpProblem), C.POINTER(N.FacpParameters), _dp, _dp, _dp]
    return lib


def _scaling_cases():
    rng = np.random.default_rng(12)
    data_s, _, _ = planted_qp(n=900, m=400, b_rows=200, seed=13, q_form="sparse")
    data_r, _, _ = planted_qp(n=900, m=400, b_rows=200, seed=14, q_form="lowrank")
    n, m = 700, 300
    A = sp.random(m, n, density=0.02, random_state=15, format="csr")
    A.data *= 10.0 ** rng.uniform(-3, 3, A.nnz)
    Qd = sp.diags(rng.uniform(1e-4, 50.0, n)).tocsr()
    b = A @ rng.uniform(-1, 1, n)
    data_d = QPData(rng.standard_normal(n) * 30, A, b - rng.random(m), np.where(rng.random(m) < 0.5, b, np.inf),
                    np.where(rng.random(n) < 0.1, -np.inf, -3.0), np.full(n, 4.0), Q=Qd)
    d = random_lp(300, 700, 5, seed=16)
    data_l = QPData(d.c, d.A, d.con_lb, d.con_ub, d.var_lb, d.var_ub)
    return {"sparse": data_s, "lowrank": data_r, "diag": data_d, "lp": data_l}


@pytest.mark.parametrize("case", ["sparse", "lowrank", "diag", "lp"])
@pytest.mark.parametrize("prm", [{"l_inf_ruiz_iterations": 10}, {"l_inf_ruiz_iterations": 3, "pock_chambolle_alpha": 0.6},
                                 {"l_inf_ruiz_iterations": 0, "has_pock_chambolle_alpha": False,
                                  "bound_objective_rescaling": False}], ids=["default", "pc0.6", "off"])
def test_oracle_equilibration_is_the_reference_preconditioner(case, prm):
    """Pins the oracle's equilibration on the reference's own code: scale
    vectors and bound/objective factors bit for bit (the device equilibration
    is held to the oracle bit for bit by tests/test_qp_gpu.py)."""
    lib = _reference_precond()
    data = _scaling_cases()[case]
    d_o, r_o, cbr_o, ovr_o = O.qp_scaling(data, prm)
    prob = O._QpProblem(data)
    p = O._qp_apply_params(O.qp_default_parameters(), prm)
    n, m = prob.n, prob.m
    d, r, f = np.zeros(max(n, 1)), np.zeros(max(m, 1)), np.zeros(2)
    assert lib.ref_facp_rescale(C.byref(prob.p), C.byref(p), d.ctypes.data_as(C.POINTER(C.c_double)),
                                r.ctypes.data_as(C.POINTER(C.c_double)), f.ctypes.data_as(C.POINTER(C.c_double))) == 0
    assert np.array_equal(d[:n], d_o) and np.array_equal(r[:m], r_o)
    assert f[0] == cbr_o and f[1] == ovr_o
