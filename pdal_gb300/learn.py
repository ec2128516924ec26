"""Learned warm start and initial sigma for a parametric LP family.

The family is the min-cost transportation LP on a fixed S x D bipartite graph
(pdal_gb300.instances.transport_lp): every instance perturbs the base costs
and draws new supplies, demands and capacities.  A three-layer MLP
(libpdal_learn_gb300.so, trained and run by the library's own CUDA kernels)
maps an instance's data to a predicted optimal primal/dual pair and the sigma
the solver ended with.  The solver then runs from that point to its own KKT
tolerance; when the predicted point's residual is worse than the cold start's,
the cold start is used instead.

    ws = WarmStart.fit(train_instances, S, D)     # solves them in one batch
    x0, y0, sigma0, used = ws.predict(test_instances)
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from . import lp
from .lp import LPData

_fp = C.POINTER(C.c_float)

# the reference's random-LP controller settings; the learned sigma is the
# initial sigma of this controller
SIGMA_PROTOCOL = {"sigma_mode": 1, "sigma_adaptive": 1, "sigma_init_factor": 0.5, "sigma_min_factor": 1e-4,
                  "sigma_max_factor": 100.0, "sigma_balance_gain": 0.0, "sigma_kp": 0.5, "sigma_ki": 0.0,
                  "sigma_kd": 0.0, "sigma_update_min": 1e-6, "sigma_update_max": 1e6, "lambda_factor": 2.01,
                  "al_lambda": 0.0, "restart_sufficient": 0.2, "restart_necessary": 0.8, "restart_artificial": 0.36}


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class MLP:
    """ReLU MLP in -> hidden -> hidden -> out on the GPU (include/pdal_learn.h)."""

    def __init__(self, inp: int, hidden: int, out: int, seed: int = 0, device: int = -1):
        self.lib = N.load_learn()
        self.h = self.lib.pdal_mlp_create(inp, hidden, out, seed, device)
        if not self.h:
            raise RuntimeError("pdal_mlp_create failed: " + self.lib.pdal_mlp_last_error().decode())
        self.inp, self.hidden, self.out = inp, hidden, out

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.pdal_mlp_last_error().decode())

    @property
    def num_params(self) -> int:
        return int(self.lib.pdal_mlp_num_params(self.h))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params, dtype=np.float32)
        self._check(self.lib.pdal_mlp_get_params(self.h, p.ctypes.data_as(_fp)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = _f32(p)
        assert p.size == self.num_params
        self._check(self.lib.pdal_mlp_set_params(self.h, p.ctypes.data_as(_fp)))

    def set_data(self, X: np.ndarray, Y: np.ndarray) -> None:
        X, Y = _f32(X), _f32(Y)
        self._keep = (X, Y)
        self._check(self.lib.pdal_mlp_set_data(self.h, X.shape[0], X.ctypes.data_as(_fp), Y.ctypes.data_as(_fp)))

    def train(self, epochs: int, batch: int = 256, lr: float = 1e-3, seed: int = 0) -> float:
        loss = self.lib.pdal_mlp_train(self.h, epochs, batch, lr, seed)
        if loss < 0:
            raise RuntimeError(self.lib.pdal_mlp_last_error().decode())
        return float(loss)

    def loss_grad(self, X: np.ndarray, Y: np.ndarray, grad: bool = True):
        X, Y = _f32(X), _f32(Y)
        g = np.empty(self.num_params, dtype=np.float32) if grad else None
        loss = self.lib.pdal_mlp_loss_grad(self.h, X.shape[0], X.ctypes.data_as(_fp), Y.ctypes.data_as(_fp),
                                           g.ctypes.data_as(_fp) if grad else None)
        if loss < 0:
            raise RuntimeError(self.lib.pdal_mlp_last_error().decode())
        return float(loss), g

    def predict(self, X: np.ndarray, bf16: bool = True) -> np.ndarray:
        X = _f32(X)
        Y = np.empty((X.shape[0], self.out), dtype=np.float32)
        self._check(self.lib.pdal_mlp_predict(self.h, X.shape[0], X.ctypes.data_as(_fp), Y.ctypes.data_as(_fp),
                                              1 if bf16 else 0))
        return Y

    def close(self):
        if getattr(self, "h", None):
            self.lib.pdal_mlp_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


# ---------------------------------------------------------------- the transport family

def features(d: LPData, S: int, D: int) -> np.ndarray:
    """Instance data normalised to O(1): costs / 100, capacities / 200,
    supplies and demands / 100."""
    b = np.asarray(d.con_ub, dtype=np.float64)
    return np.concatenate([np.asarray(d.c) / 100.0, np.asarray(d.var_ub) / 200.0, b[:S] / 100.0, b[S:] / 100.0])


def targets(d: LPData, x: np.ndarray, y: np.ndarray, sigma: float) -> np.ndarray:
    """Primal as a fraction of capacity, duals / 100, log sigma."""
    return np.concatenate([x / np.asarray(d.var_ub), y / 100.0, [np.log(max(sigma, 1e-12))]])


def decode(d: LPData, t: np.ndarray, S: int, D: int):
    n = S * D
    cap = np.asarray(d.var_ub)
    x = np.clip(t[:n], 0.0, 1.0) * cap
    y = t[n:n + S + D] * 100.0
    sigma = float(np.exp(t[n + S + D]))
    return x, y, sigma


def point_kkt(d: LPData, x: np.ndarray, y: np.ndarray) -> float:
    """Relative KKT error of (x, y) for min c'x, Ax = b, 0 <= x <= u (finite
    box, so every reduced cost is dual feasible): max of the primal residual
    |Ax - b| / (1 + |b|) and the relative gap between c'x and the dual
    objective b'y + sum min(c - A'y, 0) u."""
    rp, ci, v, (m, n) = d.csr()
    import scipy.sparse as sp

    A = sp.csr_matrix((v, ci, rp), shape=(m, n))
    b = np.asarray(d.con_ub)
    u = np.asarray(d.var_ub)
    x = np.clip(x, 0.0, u)
    rel_p = np.linalg.norm(A @ x - b) / (1.0 + np.linalg.norm(b))
    rc = np.asarray(d.c) - A.T @ y
    pobj = float(np.dot(d.c, x))
    dobj = float(b @ y + np.minimum(rc, 0.0) @ u)
    gap = abs(pobj - dobj) / (1.0 + abs(pobj) + abs(dobj))
    return float(max(rel_p, gap))


@dataclass
class WarmStart:
    """MLP from instance features to (primal, dual, log sigma); inputs and
    outputs are standardised with the training set's mean and deviation."""

    mlp: MLP
    S: int
    D: int
    xm: np.ndarray
    xs: np.ndarray
    ym: np.ndarray
    ys: np.ndarray
    train_loss: float
    train_sec: float

    @staticmethod
    def solve_family(items: list[LPData], params: dict, chunk: int = 2048, sigma0=None):
        """Batch solves in chunks (one persistent launch per chunk)."""
        out, stats = [], []
        for i in range(0, len(items), chunk):
            s0 = None if sigma0 is None else sigma0[i:i + chunk]
            r, st = lp.solve_batch(items[i:i + chunk], params, SIGMA_PROTOCOL, sigma0=s0)
            out += r
            stats.append(st)
        return out, stats

    @classmethod
    def fit(cls, items: list[LPData], S: int, D: int, params: dict, hidden: int = 256, epochs: int = 30,
            batch: int = 256, lr: float = 1e-3, seed: int = 0, solved=None):
        import time

        res = solved if solved is not None else cls.solve_family(items, params)[0]
        keep = [i for i, r in enumerate(res) if r.status == "OPTIMAL"]
        X = np.stack([features(items[i], S, D) for i in keep])
        Y = np.stack([targets(items[i], res[i].x, res[i].y, res[i].stats.get("sigma_best", 0.0) or 1.0)
                      for i in keep])
        xm, xs = X.mean(0), X.std(0) + 1e-6
        ym, ys = Y.mean(0), Y.std(0) + 1e-6
        mlp = MLP(X.shape[1], hidden, Y.shape[1], seed=seed)
        mlp.set_data((X - xm) / xs, (Y - ym) / ys)
        t0 = time.perf_counter()
        loss = mlp.train(epochs, batch, lr, seed)
        return cls(mlp, S, D, xm, xs, ym, ys, loss, time.perf_counter() - t0)

    def raw_predict(self, items: list[LPData], bf16: bool = True) -> np.ndarray:
        X = np.stack([features(d, self.S, self.D) for d in items])
        T = self.mlp.predict((X - self.xm) / self.xs, bf16=bf16).astype(np.float64)
        return T * self.ys + self.ym

    def predict_device(self, items: list[LPData], bf16: bool = True):
        """The whole prediction on the GPU (pdal_transport_warm_start):
        features, network, decoding and the KKT error of the predicted point
        and of the cold start.  Returns (x, y, sigma, kkt_pred, kkt_cold) as
        arrays over the instances."""
        S, D = self.S, self.D
        n, m = S * D, S + D
        k = len(items)
        c = np.ascontiguousarray(np.stack([np.asarray(d.c, dtype=np.float64) for d in items]))
        u = np.ascontiguousarray(np.stack([np.asarray(d.var_ub, dtype=np.float64) for d in items]))
        b = np.ascontiguousarray(np.stack([np.asarray(d.con_ub, dtype=np.float64) for d in items]))
        x = np.empty((k, n))
        y = np.empty((k, m))
        sig, kp, kc = np.empty(k), np.empty(k), np.empty(k)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        xm, xs, ym, ys = f64(self.xm), f64(self.xs), f64(self.ym), f64(self.ys)
        P = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        lib = self.mlp.lib
        rc = lib.pdal_transport_warm_start(self.mlp.h, S, D, k, P(c), P(u), P(b), P(xm), P(xs), P(ym), P(ys),
                                           1 if bf16 else 0, P(x), P(y), P(sig), P(kp), P(kc))
        if rc != 0:
            raise RuntimeError(lib.pdal_mlp_last_error().decode())
        return x, y, sig, kp, kc

    def predict(self, items: list[LPData], bf16: bool = True):
        """Warm starts, initial sigmas, whether each prediction was kept
        (False: its residual was worse than the cold start's) and the
        predicted points' KKT errors, all computed on the GPU."""
        x, y, sig, kp, kc = self.predict_device(items, bf16)
        used = kp < kc
        xs = [x[i] if used[i] else None for i in range(len(items))]
        ys = [y[i] if used[i] else None for i in range(len(items))]
        return xs, ys, np.where(used, sig, 0.0), used, kp
