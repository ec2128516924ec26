"""The warm-start MLP: the CPU oracle against finite differences (no GPU),
then the CUDA kernels against the oracle, training, BF16 inference, and the
learned warm start on a small transportation family (GPU)."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    inp, h, out, n = 7, 5, 4, 6
    nparam = inp * h + h + h * h + h + h * out + out
    p = rng.standard_normal(nparam) * 0.5
    X, Y = rng.standard_normal((n, inp)), rng.standard_normal((n, out))
    loss, g = MO.loss_grad(p, X, Y, inp, h, out)
    eps = 1e-6
    for k in rng.choice(nparam, 25, replace=False):
        e = np.zeros(nparam)
        e[k] = eps
        fd = (MO.loss_grad(p + e, X, Y, inp, h, out)[0] - MO.loss_grad(p - e, X, Y, inp, h, out)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * (1 + abs(fd))


def test_point_kkt_is_zero_at_an_optimum():
    from scipy.optimize import linprog

    from pdal_gb300.instances import transport_lp
    from pdal_gb300.learn import point_kkt

    d = transport_lp(6, 5, seed=3)
    rp, ci, v, (m, n) = d.csr()
    import scipy.sparse as sp

    A = sp.csr_matrix((v, ci, rp), shape=(m, n))
    r = linprog(d.c, A_eq=A, b_eq=d.con_ub, bounds=list(zip(d.var_lb, d.var_ub)), method="highs")
    y = r.eqlin.marginals
    assert point_kkt(d, r.x, y) < 1e-8
    assert point_kkt(d, np.zeros(n), np.zeros(m)) > 0.1


@pytest.mark.gpu
def test_gpu_gradient_matches_oracle():
    from pdal_gb300.learn import MLP

    rng = np.random.default_rng(1)
    inp, h, out, n = 70, 33, 21, 37  # not multiples of the 64 x 64 tile
    net = MLP(inp, h, out, seed=3)
    p = net.get_params()
    X, Y = rng.standard_normal((n, inp)).astype(np.float32), rng.standard_normal((n, out)).astype(np.float32)
    loss, g = net.loss_grad(X, Y)
    lo, go = MO.loss_grad(p, X, Y, inp, h, out)
    assert abs(loss - lo) <= 1e-5 * (1 + lo)
    assert np.abs(g - go).max() <= 1e-4 * (1 + np.abs(go).max())
    P32 = net.predict(X, bf16=False)
    Po, _ = MO.forward(p, X, inp, h, out)
    assert np.abs(P32 - Po).max() <= 1e-4 * (1 + np.abs(Po).max())
    Pb = net.predict(X, bf16=True)  # BF16 weights/activations, FP32 accumulation: ~3 significant digits
    assert np.abs(Pb - Po).max() <= 3e-2 * (1 + np.abs(Po).max())


@pytest.mark.gpu
def test_gpu_training_fits_a_smooth_map():
    from pdal_gb300.learn import MLP

    rng = np.random.default_rng(2)
    X = rng.uniform(-1, 1, (2048, 16)).astype(np.float32)
    W = rng.standard_normal((16, 8))
    Y = np.tanh(X @ W).astype(np.float32)
    net = MLP(16, 64, 8, seed=0)
    l0 = net.loss_grad(X, Y, grad=False)[0]
    net.set_data(X, Y)
    l1 = net.train(60, batch=128, lr=3e-3, seed=0)
    assert l1 < 0.1 * l0
    # reproducible: the same seeds give the same parameters
    net2 = MLP(16, 64, 8, seed=0)
    net2.set_data(X, Y)
    net2.train(60, batch=128, lr=3e-3, seed=0)
    assert np.array_equal(net.get_params(), net2.get_params())


@pytest.mark.gpu
def test_learned_warm_start_against_cold_start():
    """Small transportation family (12 x 12): train on 1,024 solved instances
    (one batch launch), evaluate on 64 held-out ones against the cold start.
    The solver must reach the same optimum from the learned point, the
    fallback must keep every used prediction better than the cold start by
    the point's own KKT measure, and the measured iteration ratio is reported
    (on this family the network's points are only slightly better than the
    cold start, so the gain is small)."""
    from pdal_gb300.instances import transport_family
    from pdal_gb300.learn import WarmStart, point_kkt

    S = D = 12
    base = np.random.default_rng(4000).uniform(1, 100, S * D)
    train = transport_family(S, D, range(10_000, 11_024), base)
    test = transport_family(S, D, range(900_000, 900_064), base)
    params = {"eps": 1e-6, "l_inf_ruiz_iterations": 10, "iteration_limit": 100000}
    ws = WarmStart.fit(train, S, D, params, hidden=256, epochs=100, batch=128, lr=1e-3)
    cold, _ = WarmStart.solve_family(test, params)
    xs, ys, sig, used, kkt = ws.predict(test)
    for d, x, y, u, k in zip(test, xs, ys, used, kkt):
        if u:
            assert k < point_kkt(d, np.zeros(S * D), np.zeros(S + D))
        d.primal_start, d.dual_start = x, y
    warm, _ = WarmStart.solve_family(test, params, sigma0=sig)
    assert all(r.status == "OPTIMAL" for r in cold + warm)
    ic = np.mean([r.iterations for r in cold])
    iw = np.mean([r.iterations for r in warm])
    print(f"learned warm start: {used.mean():.2f} of predictions used, iterations {iw:.0f} vs cold {ic:.0f}")
    assert iw <= 1.1 * ic
    for c, w in zip(cold, warm):  # same optimum either way
        assert abs(c.primal_objective - w.primal_objective) <= 1e-5 * (1 + abs(c.primal_objective))
