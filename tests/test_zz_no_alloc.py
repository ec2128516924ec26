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
