"""The allocation-free entry point cp_al_gb300_primal_kkt_noalloc, through the
C-ABI, against what the solver's own entry point reports.

It exists for callers that cannot allocate device memory (another framework
owns the allocator, a memory pool forbids cudaMalloc, a latency-critical loop
must not synchronise): they pass device buffers and get the primal residual
norms and the objective of a candidate point, with the library's fixed scratch
array as the only working memory.  This file is collected last so that a run
that stops at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from pdal_gb300 import _native as N
from pdal_gb300 import instances as I
from pdal_gb300 import lp

pytestmark = pytest.mark.gpu

RTOL = 1e-8  # the objective tolerance of the parity tests


def _device(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def test_noalloc_matches_solver_twice_in_a_row(lp_lib):
    torch = pytest.importorskip("torch")
    d = I.random_lp(2000, 5000, 8, seed=0)
    # the existing entry point: a solve stopped after 400 iterations, so the
    # residual is large enough to compare relatively
    params = {"eps": 1e-12, "iteration_limit": 400, "l_inf_ruiz_iterations": 4}
    ref = lp.solve(d, params)
    rp, ci, v, (m, n) = d.csr()
    t = {
        "rp": _device(torch, rp, torch.int32), "ci": _device(torch, ci, torch.int32),
        "v": _device(torch, v, torch.float64), "lb": _device(torch, d.con_lb, torch.float64),
        "ub": _device(torch, d.con_ub, torch.float64), "c": _device(torch, d.c, torch.float64),
        "x": _device(torch, ref.x, torch.float64),
    }
    stream = torch.cuda.current_stream().cuda_stream
    results = []
    for _ in range(2):
        out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lp_lib.cp_al_gb300_primal_kkt_noalloc(
            m, n, t["rp"].data_ptr(), t["ci"].data_ptr(), t["v"].data_ptr(), t["lb"].data_ptr(),
            t["ub"].data_ptr(), t["c"].data_ptr(), t["x"].data_ptr(), out.data_ptr(), C.c_void_p(stream))
        assert rc == 0
        torch.cuda.synchronize()
        results.append(out.cpu().numpy())
    for r in results:
        # L2 primal residual of the solver's result equals the solver's own
        # absolute primal residual (LP/CP_AL/src/utils.cu:859-880), and c'x
        # its primal objective (no objective constant here)
        assert abs(r[0] - ref.absolute_primal_residual) <= RTOL * ref.absolute_primal_residual
        assert abs(r[2] - ref.primal_objective) <= RTOL * (1 + abs(ref.primal_objective))
        assert r[1] <= r[0] + 1e-300
    assert np.array_equal(results[0], results[1])


def test_noalloc_refuses_too_many_rows(lp_lib):
    dummy = C.c_void_p(1)
    rc = lp_lib.cp_al_gb300_primal_kkt_noalloc(524_289, 10, dummy, dummy, dummy, dummy, dummy, dummy, dummy,
                                               dummy, None)
    assert rc == -1
    # the refusal is reported through the library's error message, and checked
    # before any device pointer is touched
    assert "524288 rows" in N.last_error(lp_lib)


def test_noalloc_refuses_missing_matrix_pointers(lp_lib):
    dummy = C.c_void_p(1)
    for k in (1, 2):  # col_ind, vals
        args = [dummy] * 8
        args[k] = None
        rc = lp_lib.cp_al_gb300_primal_kkt_noalloc(10, 10, *args, dummy, None)
        assert rc == -1
        assert "missing device pointer" in N.last_error(lp_lib)


def _call(lib, torch, m, n, rp, ci, v, lb, ub, c, x):
    out = torch.full((3,), -1.0, dtype=torch.float64, device="cuda")
    rc = lib.cp_al_gb300_primal_kkt_noalloc(m, n, rp.data_ptr(), ci.data_ptr(), v.data_ptr(), lb.data_ptr(),
                                            ub.data_ptr(), c.data_ptr(), x.data_ptr(), out.data_ptr(), None)
    assert rc == 0, N.last_error(lib)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_edge_sizes_and_nan(lp_lib):
    """m = 0 (no constraints: both norms 0, out[2] = c'x), exactly the largest
    accepted row count (524,288 empty rows), and a NaN in x, which must show
    in both norms instead of being dropped by a maximum."""
    torch = pytest.importorskip("torch")
    n = 1000
    rng = np.random.default_rng(3)
    c = _device(torch, rng.standard_normal(n), torch.float64)
    x = _device(torch, rng.standard_normal(n), torch.float64)
    one_i = torch.zeros(1, dtype=torch.int32, device="cuda")
    one_d = torch.zeros(1, dtype=torch.float64, device="cuda")
    cx = float((c * x).sum().item())
    r = _call(lp_lib, torch, 0, n, one_i, one_i, one_d, one_d, one_d, c, x)
    assert r[0] == 0.0 and r[1] == 0.0 and abs(r[2] - cx) <= 1e-12 * (1 + abs(cx))
    m = 524_288
    rp = torch.zeros(m + 1, dtype=torch.int32, device="cuda")
    lb = torch.full((m,), -1.0, dtype=torch.float64, device="cuda")
    ub = torch.ones(m, dtype=torch.float64, device="cuda")
    r = _call(lp_lib, torch, m, n, rp, one_i, one_d, lb, ub, c, x)
    assert r[0] == 0.0 and r[1] == 0.0 and abs(r[2] - cx) <= 1e-12 * (1 + abs(cx))
    d = I.random_lp(200, 500, 5, seed=1)
    drp, dci, dv, (dm, dn) = d.csr()
    xn = np.linspace(0.0, 1.0, dn)
    xn[7] = np.nan
    r = _call(lp_lib, torch, dm, dn, _device(torch, drp, torch.int32), _device(torch, dci, torch.int32),
              _device(torch, dv, torch.float64), _device(torch, d.con_lb, torch.float64),
              _device(torch, d.con_ub, torch.float64), _device(torch, d.c, torch.float64),
              _device(torch, xn, torch.float64))
    assert np.isnan(r[0]) and np.isnan(r[1]) and np.isnan(r[2])
