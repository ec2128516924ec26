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


def _bf16(a):
    """Round to the nearest BF16 (ties to even), as __float2bfloat16 does."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("inp,h,out,n", [(512, 256, 300, 700), (1030, 256, 2049, 130)])
def test_tensor_core_inference_matches_bf16_reference(inp, h, out, n):
    """BF16 inference on the tensor cores (aligned operands: the 16-byte copy
    path; ragged output and batch edges) against the same network evaluated
    in FP64 from BF16-rounded weights, inputs and activations: only the FP32
    accumulation order differs.  A prediction is reproducible bit for bit."""
    from pdal_gb300.learn import MLP

    rng = np.random.default_rng(5)
    net = MLP(inp, h, out, seed=7)
    p = net.get_params()
    X = rng.standard_normal((n, inp)).astype(np.float32)
    o = 0
    W1 = p[o:o + inp * h].reshape(inp, h); o += inp * h
    b1 = p[o:o + h]; o += h
    W2 = p[o:o + h * h].reshape(h, h); o += h * h
    b2 = p[o:o + h]; o += h
    W3 = p[o:o + h * out].reshape(h, out); o += h * out
    b3 = p[o:o + out]
    f64 = lambda a: np.asarray(a, dtype=np.float64)
    H1 = _bf16(np.maximum(f64(_bf16(X)) @ f64(_bf16(W1)) + b1, 0))
    H2 = _bf16(np.maximum(f64(H1) @ f64(_bf16(W2)) + b2, 0))
    ref = f64(H2) @ f64(_bf16(W3)) + b3
    got = net.predict(X, bf16=True)
    # a BF16 activation may round the other way after a different FP32 sum order
    assert np.abs(got - ref).max() <= 2e-2 * (1 + np.abs(ref).max())
    assert np.median(np.abs(got - ref)) <= 1e-4 * (1 + np.abs(ref).max())
    assert np.array_equal(got, net.predict(X, bf16=True))


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
@pytest.mark.parametrize("bf16", [True, False])
def test_device_prediction_matches_host_pipeline(bf16):
    """pdal_transport_warm_start (features, network, decoding and point KKT
    on the GPU) against the same steps on the host: numpy features and
    decoding around pdal_mlp_predict, and the numpy point_kkt."""
    from pdal_gb300.instances import transport_family
    from pdal_gb300.learn import MLP, WarmStart, decode, features, point_kkt

    S, D = 9, 14
    base = np.random.default_rng(4000).uniform(1, 100, S * D)
    items = transport_family(S, D, range(500, 530), base)
    rng = np.random.default_rng(3)
    n, m = S * D, S + D
    X = np.stack([features(d, S, D) for d in items])
    mlp = MLP(2 * n + m, 64, n + m + 1, seed=2)
    ws = WarmStart(mlp, S, D, X.mean(0), X.std(0) + 1e-6, rng.uniform(0.2, 0.6, n + m + 1),
                   rng.uniform(0.1, 0.3, n + m + 1), 0.0, 0.0)
    x, y, sig, kp, kc = ws.predict_device(items, bf16=bf16)
    T = ws.raw_predict(items, bf16=bf16)
    for i, d in enumerate(items):
        xh, yh, sh = decode(d, T[i], S, D)
        assert np.array_equal(x[i], xh) and np.array_equal(y[i], yh)
        assert abs(sig[i] - sh) <= 1e-15 * sh
        assert abs(kp[i] - point_kkt(d, xh, yh)) <= 1e-12 * (1 + kp[i])
        assert abs(kc[i] - point_kkt(d, np.zeros(n), np.zeros(m))) <= 1e-12


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
    assert iw <= ic
    for c, w in zip(cold, warm):  # same optimum either way
        assert abs(c.primal_objective - w.primal_objective) <= 1e-5 * (1 + abs(c.primal_objective))


@pytest.mark.gpu
def test_learned_warm_start_gains_on_the_40x40_family():
    """The 40 x 40 transportation family (1,600 arcs): 4,096 training optima
    solved in one batch, 100 epochs, 128 held-out instances solved to relative
    KKT 1e-6 from the learned start and initial sigma and from the cold start.
    The learned start must save at least 10% of the iterations on average,
    and every instance must reach the same optimum either way."""
    from pdal_gb300.instances import transport_family
    from pdal_gb300.learn import WarmStart

    S = D = 40
    base = np.random.default_rng(4000).uniform(1, 100, S * D)
    train = transport_family(S, D, range(10_000, 14_096), base)
    test = transport_family(S, D, range(900_000, 900_128), base)
    params = {"eps": 1e-6, "l_inf_ruiz_iterations": 10, "iteration_limit": 100_000}
    ws = WarmStart.fit(train, S, D, params, hidden=256, epochs=100, batch=128, lr=1e-3)
    cold, _ = WarmStart.solve_family(test, params)
    xs, ys, sig, used, kkt = ws.predict(test)
    for d, x, y in zip(test, xs, ys):
        d.primal_start, d.dual_start = x, y
    warm, _ = WarmStart.solve_family(test, params, sigma0=sig)
    assert all(r.status == "OPTIMAL" for r in cold + warm)
    ic = np.mean([r.iterations for r in cold])
    iw = np.mean([r.iterations for r in warm])
    print(f"40x40 learned warm start: {used.mean():.2f} used, iterations {iw:.0f} vs cold {ic:.0f} ({iw / ic:.3f})")
    assert iw <= 0.9 * ic
    for c, w in zip(cold, warm):
        assert abs(c.primal_objective - w.primal_objective) <= 1e-5 * (1 + abs(c.primal_objective))
