"""micropp3_ell_solve_cgpd_noalloc: the stencil-ELL DPCG solve for callers that may not allocate device memory
while they run (for example a macro solver that owns the whole device through its own memory pool).  It uses
the library's fixed scratch array instead of cudaMalloc; its results must equal those of
micropp3_ell_solve_cgpd, the allocating entry point, on two calls in a row (the second call finds the first
call's data in the shared array and must not depend on it).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from test_gpu_ell import stencil_system

pytestmark = pytest.mark.gpu

TOL = 1e-10  # relative, as for solutions elsewhere in the GPU tests


def _solve(lib, name, nodes, dv, db, dx, rel_tol=1e-10):
    its = ctypes.c_int(-1)
    n3 = (ctypes.c_int * 3)(*nodes)
    rc = getattr(lib, name)(n3, dv.data_ptr(), db.data_ptr(), dx.data_ptr(), rel_tol, 1e-50, 1000,
                            ctypes.byref(its), None)
    return rc, its.value


def test_noalloc_matches_allocating_solve_twice(gpu_lib):
    import torch
    nodes = (9, 8, 7)
    vals, b, _, _ = stencil_system(nodes, seed=3)
    dv = torch.tensor(vals, dtype=torch.float64, device="cuda").contiguous()
    rhs = [torch.tensor(b, dtype=torch.float64, device="cuda"),
           torch.tensor(-2.5 * b + 0.1 * np.roll(b, 3), dtype=torch.float64, device="cuda")]
    for db in rhs:
        # interior rows only carry a right-hand side
        db.view(-1, 3)[torch.tensor(np.all(np.asarray(b).reshape(-1, 3) == 0, axis=1), device="cuda")] = 0.0
    results = []
    for call, db in enumerate(rhs):
        x_ref = torch.full_like(db, 3.0)
        rc, its_ref = _solve(gpu_lib, "micropp3_ell_solve_cgpd", nodes, dv, db, x_ref)
        assert rc == 0
        x_na = torch.full_like(db, -7.0)
        rc, its_na = _solve(gpu_lib, "micropp3_ell_solve_cgpd_noalloc", nodes, dv, db, x_na)
        torch.cuda.synchronize()
        assert rc == 0, call
        assert its_na == its_ref, call
        a, r = x_na.cpu().numpy(), x_ref.cpu().numpy()
        assert np.max(np.abs(a - r)) <= TOL * np.max(np.abs(r)), call
        results.append(a)
    assert not np.allclose(results[0], results[1])


def test_noalloc_rejects_grids_over_the_limit(gpu_lib):
    import torch
    nodes = (51, 51, 51)  # 132,651 nodes > MICROPP3_NOALLOC_MAX_NODES = 131,072
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc, _ = _solve(gpu_lib, "micropp3_ell_solve_cgpd_noalloc", nodes, d, d, d)
    assert rc == -3
