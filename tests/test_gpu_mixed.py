"""The fast form: FP32 Jacobian/CG inside FP64 refinement, and ctan by implicit differentiation.

It is judged against the FP64 oracle converged tightly (CG relative tolerance 1e-12, Newton relative 1e-11):
average stress within 1e-7 and ctan within 1e-5, relative to the largest entry.  The reference ctan for the
tolerance is the oracle's central difference of the converged average stress with h = 1e-7 (its truncation
and rounding errors are ~1e-7); the oracle's own forward-difference ctan is also compared, at 1e-4, since
its step 1e-8 leaves an error near 1e-5 even with tight solves.
"""
import numpy as np
import pytest

import pyoracle as orc
from cases import gpu_config, oracle_config
from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL_STRESS = 1e-7
TOL_CTAN = 1e-5

TIGHT = dict(cg_rel_tol=1e-12, nr_rel_tol=1e-11, nr_max_tol=1e-30, nr_max_its=40)
FAST = dict(cg_rel_tol=1e-5, nr_rel_tol=1e-10, nr_max_tol=1e-30, nr_max_its=40)


def central_fd_ctan(n, kw, strain, vars_setup_steps, h=1e-7):
    """d(sigma)/d(eps) by central differences of tightly converged oracle solves (FE_ONE_WAY: no ctan work),
    starting from the state left by `vars_setup_steps` (strains accepted with update_vars)."""
    kw = dict(kw)
    kw["coupling"] = [1]
    kw["ngp"] = 1
    o = orc.OracleRVE(oracle_config(n, **kw, **TIGHT))
    for e in vars_setup_steps:
        o.set_strain(0, e)
        o.homogenize()
        o.update_vars()
    C = np.zeros((6, 6))
    for i in range(6):
        ep, em = strain.copy(), strain.copy()
        ep[i] += h
        em[i] -= h
        o.set_strain(0, ep)
        o.homogenize()
        sp = o.get_stress(0)
        o.set_strain(0, em)
        o.homogenize()
        sm = o.get_stress(0)
        C[:, i] = (sp - sm) / (2 * h)
    return C


def run_fast_vs_oracle(n, kw, path, precision, ctan_mode=1):
    import micropp_gb300 as mg
    g = mg.Micropp(gpu_config(n, precision=precision, ctan_mode=ctan_mode, **kw, **FAST))
    o = orc.OracleRVE(oracle_config(n, **kw, **TIGHT))
    done = []
    for e in path:
        g.set_strain(0, e)
        o.set_strain(0, e)
        g.homogenize()
        o.homogenize()
        assert g.has_converged(0) and o.has_converged(0)
        assert g.is_non_linear(0) == o.is_non_linear(0)
        es = rel_err(g.get_stress(0), o.get_stress(0))
        assert es < TOL_STRESS, es
        if g.is_non_linear(0):
            fd = central_fd_ctan(n, kw, e, done)
            ec = rel_err(g.get_ctan(0), fd)
            assert ec < TOL_CTAN, ec
            assert rel_err(o.get_ctan(0), fd) < 1e-4
        g.update_vars()
        o.update_vars()
        done.append(e)
    return g, o


def damage_kw(n):
    from micropp_gb300 import workloads as wl
    return dict(elem_type=wl.layers_z(n),
                mats=((2, 1e7, 0.25, 0, 0, 1e5), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0)),
                coupling=[2], lin_stress=0)


DAMAGE_PATH = [np.array([2e-2, -6e-3, 0, 1e-2, 0, 0]) * s / 2 for s in (1, 2)]


@pytest.mark.parametrize("precision", [1, 0])
def test_implicit_ctan_damage_layers(gpu_lib, precision):
    run_fast_vs_oracle(8, damage_kw(8), DAMAGE_PATH, precision)


def test_implicit_ctan_j2_sphere(gpu_lib):
    kw = dict(micro_type=1, geo=(0.2, 0, 0, 0),
              mats=((1, 1e7, 0.3, 1e5, 1e4, 0), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0)), coupling=[2],
              lin_stress=0)
    run_fast_vs_oracle(6, kw, [np.array([1e-2, 0, 0, 0, 0, 0]) * s / 2 for s in (1, 2)], 1)


def test_implicit_linear_ctan(gpu_lib):
    """The constructor's linear ctan by one tangent solve equals the oracle's six linear solves (tight CG)."""
    import micropp_gb300 as mg
    kw = dict(micro_type=1, geo=(0.2, 0, 0, 0),
              mats=((0, 1e7, 0.25, 0, 0, 0), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0)), coupling=[2])
    g = mg.Micropp(gpu_config(10, precision=1, ctan_mode=1, **kw))
    o = orc.OracleRVE(oracle_config(10, cg_rel_tol=1e-13, **kw))
    assert rel_err(g.ctan_lin(), o.ctan_lin()) < 1e-6


def test_mixed_newton_perturbation_ctan_runs(gpu_lib):
    """MIXED precision with the reference's perturbation ctan: stress as accurate as the tight oracle."""
    n, kw = 6, damage_kw(6)
    import micropp_gb300 as mg
    g = mg.Micropp(gpu_config(n, precision=1, ctan_mode=0, **kw, **FAST))
    o = orc.OracleRVE(oracle_config(n, **kw, **TIGHT))
    for r in (g, o):
        r.set_strain(0, DAMAGE_PATH[1])
        r.homogenize()
    assert rel_err(g.get_stress(0), o.get_stress(0)) < TOL_STRESS
    assert np.isfinite(g.get_ctan(0)).all()


def test_batched_fast_form_uneven_points(gpu_lib):
    """Several points of one handle in the fast form, with different strains (some stay linear)."""
    import micropp_gb300 as mg
    n = 6
    kw = damage_kw(n)
    kw["coupling"] = [2] * 4
    g = mg.Micropp(gpu_config(n, ngp=4, precision=1, ctan_mode=1, **kw, **FAST))
    o = orc.OracleRVE(oracle_config(n, ngp=4, **kw, **TIGHT))
    strains = [DAMAGE_PATH[1], 0.1 * DAMAGE_PATH[1], -DAMAGE_PATH[1], DAMAGE_PATH[0]]
    for r in (g, o):
        for gp, e in enumerate(strains):
            r.set_strain(gp, e)
        r.homogenize()
    for gp in range(4):
        assert g.is_non_linear(gp) == o.is_non_linear(gp)
        assert rel_err(g.get_stress(gp), o.get_stress(gp)) < TOL_STRESS
        if g.is_non_linear(gp):
            assert rel_err(g.get_ctan(gp), o.get_ctan(gp)) < 1e-4
