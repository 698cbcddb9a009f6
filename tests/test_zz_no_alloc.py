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


def _stencil_vals(nodes, seed):
    """The symmetric, diagonally dominant block stencil of test_gpu_ell.stencil_system, built with array
    operations so that grids at the scratch limit take a fraction of a second."""
    nx, ny, nz = nodes
    nn = nx * ny * nz
    np_ = (nn + 31) // 32 * 32
    rng = np.random.default_rng(seed)
    w_node = rng.uniform(0.5, 1.5, nn)
    idx = np.arange(nn)
    i, j, k = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    inner = idx[(i > 0) & (j > 0) & (k > 0) & (i < nx - 1) & (j < ny - 1) & (k < nz - 1)]
    vals = np.zeros((243, np_))
    diag = np.zeros(len(inner))
    for s in range(27):
        if s == 13:
            continue
        dz, dy, dx = s // 9 - 1, (s // 3) % 3 - 1, s % 3 - 1
        w = 0.5 * (w_node[inner] + w_node[inner + dz * nx * ny + dy * nx + dx])
        for d in range(3):
            vals[s * 9 + d * 3 + d, inner] = -w
        diag += w
    for d in range(3):
        vals[13 * 9 + d * 3 + d, inner] = diag + 1.0
    b = np.zeros((nn, 3))
    b[inner] = rng.standard_normal((len(inner), 3))
    return vals, b.reshape(-1)


def _solve_on(lib, name, nodes, dv, db, dx, stream):
    its = ctypes.c_int(-1)
    n3 = (ctypes.c_int * 3)(*nodes)
    rc = getattr(lib, name)(n3, dv.data_ptr(), db.data_ptr(), dx.data_ptr(), 1e-10, 1e-50, 1000,
                            ctypes.byref(its), ctypes.c_void_p(stream))
    return rc, its.value


@pytest.mark.parametrize("nodes", [(64, 64, 32), (50, 50, 50)], ids=["at_limit_131072", "50cubed"])
def test_noalloc_at_the_size_limit_on_a_stream(gpu_lib, nodes):
    """Grids at (64 x 64 x 32 = MICROPP3_NOALLOC_MAX_NODES) and just under the limit, where the scratch's
    reduction partials are sized for the largest grid, solved on a non-default stream twice in a row."""
    import torch
    vals, b = _stencil_vals(nodes, seed=11)
    dv = torch.tensor(vals, dtype=torch.float64, device="cuda")
    st = torch.cuda.Stream()
    for call, scale in enumerate((1.0, -0.5)):
        db = torch.tensor(scale * b + (0.25 * np.roll(b, 7) if call else 0.0), dtype=torch.float64,
                          device="cuda")
        db.view(-1, 3)[torch.tensor(np.all(b.reshape(-1, 3) == 0, axis=1), device="cuda")] = 0.0
        x_ref = torch.zeros_like(db)
        x_na = torch.full_like(db, 5.0)
        torch.cuda.synchronize()
        rc, its_ref = _solve_on(gpu_lib, "micropp3_ell_solve_cgpd", nodes, dv, db, x_ref, st.cuda_stream)
        assert rc == 0
        rc, its_na = _solve_on(gpu_lib, "micropp3_ell_solve_cgpd_noalloc", nodes, dv, db, x_na, st.cuda_stream)
        st.synchronize()
        assert rc == 0, call
        assert its_na == its_ref and 0 < its_na < 1000, (call, its_na, its_ref)
        a, r = x_na.cpu().numpy(), x_ref.cpu().numpy()
        assert np.max(np.abs(a - r)) <= TOL * np.max(np.abs(r)), call


def test_noalloc_rejects_grids_over_the_limit(gpu_lib):
    import torch
    nodes = (51, 51, 51)  # 132,651 nodes > MICROPP3_NOALLOC_MAX_NODES = 131,072
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc, _ = _solve(gpu_lib, "micropp3_ell_solve_cgpd_noalloc", nodes, d, d, d)
    assert rc == -3
