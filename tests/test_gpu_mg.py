"""Multigrid preconditioner of the fast form's FP32 solves (Newton corrections and the 6-RHS tangent solve).

The preconditioner changes how many CG iterations a solve takes, not what it converges to: the fast form with
multigrid (precond = MICROPP3_PRECOND_MG) must meet the same bars against the tightly converged FP64 oracle as
with Jacobi (average stress within 1e-7, ctan within 1e-5 of the oracle's central difference), with fewer CG
iterations.  Grids with an odd number of elements or different counts per axis coarsen to ceil(n / 2) per axis.
"""
import numpy as np
import pytest

import pyoracle as orc
from cases import gpu_config, oracle_config
from conftest import rel_err
from test_gpu_mixed import FAST, TIGHT, TOL_CTAN, TOL_STRESS, central_fd_ctan, damage_kw

pytestmark = pytest.mark.gpu

SPHERE_DAMAGE = dict(micro_type=1, geo=(0.2, 0, 0, 0),
                     mats=((2, 1e7, 0.25, 0, 0, 1e5), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0)),
                     coupling=[2], lin_stress=0)


@pytest.mark.parametrize("n,levels", [(5, 2), (10, 3), ((13, 6, 9), 2), (60, 5)])
def test_levels(gpu_lib, n, levels):
    import micropp_gb300 as mg
    g = mg.Micropp(gpu_config(n, precision=mg.MIXED, ctan_mode=mg.CTAN_IMPLICIT, calc_ctan_lin=0,
                              precond=mg.PRECOND_MG))
    assert g.mg_levels() == levels
    j = mg.Micropp(gpu_config(n, precision=mg.MIXED, ctan_mode=mg.CTAN_IMPLICIT, calc_ctan_lin=0))
    assert j.mg_levels() == 0  # Jacobi is the default


def test_rejected_configurations(gpu_lib):
    import micropp_gb300 as mg
    with pytest.raises(RuntimeError, match="FP32 solves"):
        mg.Micropp(gpu_config(6, precond=mg.PRECOND_MG))  # FP64 Newton and perturbation ctan: no FP32 solve
    for n in (4, (3, 8, 8)):
        with pytest.raises(RuntimeError, match="4 elements"):
            mg.Micropp(gpu_config(n, precision=mg.MIXED, precond=mg.PRECOND_MG))
    with pytest.raises(RuntimeError, match="precond"):
        mg.Micropp(gpu_config(6, precision=mg.MIXED, precond=7))


def _fast_path(n, kw, path, precond):
    """The fast form along `path` against the tight oracle; returns (CG iterations, handle)."""
    import micropp_gb300 as mg
    g = mg.Micropp(gpu_config(n, precision=mg.MIXED, ctan_mode=mg.CTAN_IMPLICIT, precond=precond, **kw, **FAST))
    o = orc.OracleRVE(oracle_config(n, **kw, **TIGHT))
    done = []
    its0 = g.total_cg_its()
    for e in path:
        for r in (g, o):
            r.set_strain(0, e)
            r.homogenize()
        assert g.has_converged(0) and o.has_converged(0)
        assert g.is_non_linear(0) == o.is_non_linear(0)
        assert rel_err(g.get_stress(0), o.get_stress(0)) < TOL_STRESS
        if g.is_non_linear(0):
            fd = central_fd_ctan(n, kw, e, done)
            assert rel_err(g.get_ctan(0), fd) < TOL_CTAN
        for r in (g, o):
            r.update_vars()
        done.append(e)
    return g.total_cg_its() - its0, g


DAMAGE_PATH = [np.array([2e-2, -6e-3, 0, 1e-2, 0, 0]) * s / 2 for s in (1, 2)]


def test_damage_layers_mg_against_jacobi(gpu_lib):
    """Layered damage RVE of 12^3: both preconditioners meet the bars, multigrid with fewer CG iterations.  The
    gap grows with the grid (Jacobi-PCG iterations grow with n, the V-cycle's stay near 10 per solve): 2x here,
    about 20x on 60^3 RVEs."""
    import micropp_gb300 as mg
    its_mg, g = _fast_path(12, damage_kw(12), DAMAGE_PATH, mg.PRECOND_MG)
    assert g.mg_levels() == 3
    its_j, _ = _fast_path(12, damage_kw(12), DAMAGE_PATH, mg.PRECOND_JACOBI)
    assert its_mg < 0.6 * its_j, (its_mg, its_j)


def test_fp16_smoothing_operator_meets_the_bars(gpu_lib):
    """MICROPP3_PRECOND_MG_HALF (the level-0 smoothing passes read an FP16 copy of the fine operator): the same
    bars against the tight oracle, with CG iterations close to the FP32 V-cycle's."""
    import micropp_gb300 as mg
    its_h, g = _fast_path(12, damage_kw(12), DAMAGE_PATH, mg.PRECOND_MG_HALF)
    assert g.mg_levels() == 3
    its_f, _ = _fast_path(12, damage_kw(12), DAMAGE_PATH, mg.PRECOND_MG)
    assert its_h <= 1.25 * its_f + 2, (its_h, its_f)


@pytest.mark.parametrize("n", [9, (13, 6, 9)])
def test_odd_and_noncubic_grids(gpu_lib, n):
    import micropp_gb300 as mg
    _, g = _fast_path(n, SPHERE_DAMAGE, [np.array([2.5e-2, -5e-3, 0, 1e-2, 0, 0])], mg.PRECOND_MG)
    assert g.mg_levels() >= 2


def test_linear_ctan_mg(gpu_lib):
    """The constructor's linear ctan through the multigrid tangent solve equals the oracle's (tight CG) and the
    Jacobi form's: the refined solve does not depend on the preconditioner (measured on a GB300: 2.3e-8 from the
    oracle with either).  On an 11^3 grid both reach only 3.2e-6, the rounding of the FP32 Jacobian."""
    import micropp_gb300 as mg
    kw = dict(micro_type=1, geo=(0.2, 0, 0, 0),
              mats=((0, 1e7, 0.25, 0, 0, 0), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0)), coupling=[2])
    g = mg.Micropp(gpu_config(10, precision=mg.MIXED, ctan_mode=mg.CTAN_IMPLICIT, precond=mg.PRECOND_MG, **kw))
    j = mg.Micropp(gpu_config(10, precision=mg.MIXED, ctan_mode=mg.CTAN_IMPLICIT, **kw))
    o = orc.OracleRVE(oracle_config(10, cg_rel_tol=1e-13, **kw))
    assert g.mg_levels() == 3
    assert rel_err(g.ctan_lin(), o.ctan_lin()) < 1e-6
    assert rel_err(g.ctan_lin(), j.ctan_lin()) < 1e-7


@pytest.mark.parametrize("precond", [1, 2], ids=["fp32", "fp16_smoothing"])
def test_batched_mg_uneven_points(gpu_lib, precond):
    """Four points of one handle, different strains (one stays linear), multigrid batch of uneven solves."""
    import micropp_gb300 as mg
    n = 10
    kw = damage_kw(n)
    kw["coupling"] = [2] * 4
    g = mg.Micropp(gpu_config(n, ngp=4, precision=mg.MIXED, ctan_mode=mg.CTAN_IMPLICIT, precond=precond,
                              **kw, **FAST))
    o = orc.OracleRVE(oracle_config(n, ngp=4, **kw, **TIGHT))
    assert g.mg_levels() == 3
    strains = [DAMAGE_PATH[1], 0.1 * DAMAGE_PATH[1], -DAMAGE_PATH[1], DAMAGE_PATH[0]]
    for r in (g, o):
        for gp, e in enumerate(strains):
            r.set_strain(gp, e)
        r.homogenize()
    for gp in range(4):
        assert g.has_converged(gp)
        assert g.is_non_linear(gp) == o.is_non_linear(gp)
        assert rel_err(g.get_stress(gp), o.get_stress(gp)) < TOL_STRESS
        if g.is_non_linear(gp):
            assert rel_err(g.get_ctan(gp), o.get_ctan(gp)) < 1e-4


@pytest.mark.parametrize("precond", [1, 2], ids=["fp32", "fp16_smoothing"])
def test_damage_path_20_converges_with_mg(gpu_lib, precond):
    """The 20^3 layered damage step whose first Jacobian (uniform strain (1e-2, -3e-3, 0, 5e-3, 0, 0), loading
    with q/r = 1.67) is strongly anisotropic: lambda_max(D^-1 A) = 4.15 > 2 / 0.6, where a plain damped-Jacobi
    V-cycle stops being positive definite and its CG stalled at the iteration cap in every Newton iteration.
    With the safeguarded smoother diagonal it converges; the results meet the parity bars."""
    import micropp_gb300 as mg
    its_mg, g = _fast_path(20, damage_kw(20), DAMAGE_PATH, precond)
    its_j, _ = _fast_path(20, damage_kw(20), DAMAGE_PATH, mg.PRECOND_JACOBI)
    assert its_mg < its_j, (its_mg, its_j)


def test_newton_iteration_graphs_match_unfused(gpu_lib):
    """With CUDA graphs on and kernel timers off, a Newton iteration of the mixed multigrid form runs as one
    graph (assembly, CG start, a WHILE node over the CG chunks, u += du, residual).  Its kernels and their order
    are those of the unfused iteration, so stress, ctan and the iteration counts are bitwise the same."""
    import micropp_gb300 as mg
    n = 12
    kw = damage_kw(n)
    kw["coupling"] = [2] * 3
    handles = []
    for graphs in (True, False):
        g = mg.Micropp(gpu_config(n, ngp=3, precision=mg.MIXED, ctan_mode=mg.CTAN_IMPLICIT, precond=mg.PRECOND_MG,
                                  **kw, **FAST))
        g.set_kernel_timing(False)
        g.set_cuda_graphs(graphs)
        handles.append(g)
    strains = [DAMAGE_PATH[1], 0.5 * DAMAGE_PATH[1], -DAMAGE_PATH[0]]
    for step in range(3):
        for g in handles:
            for gp, e in enumerate(strains):
                g.set_strain(gp, e * (1 + 0.2 * step))
            g.homogenize()
        a, b = handles
        for gp in range(3):
            assert np.array_equal(a.get_stress(gp), b.get_stress(gp)), (step, gp)
            assert np.array_equal(a.get_ctan(gp), b.get_ctan(gp)), (step, gp)
            assert a.newton(gp) == b.newton(gp)
            assert a.status(gp) == b.status(gp) == mg.STATUS_OK
        for g in handles:
            g.update_vars()
    assert handles[0].total_cg_its() == handles[1].total_cg_its()
