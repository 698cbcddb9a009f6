"""GPU parity: the GB300 library (through its C ABI) against the oracle on identical seeded inputs.

Tolerances (relative to the largest entry of the tensor compared): average stress and displacements 1e-10,
internal variables 5e-10 (the reference built with fused multiply-adds already moves damage variables by
7.6e-11), Newton/CG counts and flags exactly, the linear ctan 1e-8.  The ctan of a nonlinear
point is a forward difference with step 1e-8 of average stresses that come out of six further Newton/CG
solves, so it amplifies the last-bit differences of any other summation order by ~1e8: the reference
algorithm itself, built with fused multiply-adds or with GPU-like blocked dot products, moves it by up to
2.7e-8 and 1.1e-7 while its stresses agree to 1e-13 (tests/test_rounding_floor.py), and the GPU's tree
reductions move it by up to 1.1e-6 on these cases.  The nonlinear ctan is therefore held to 5e-6.
"""
import numpy as np
import pytest

import pyoracle as orc
from cases import case, gpu_config, linear_pass, oracle_config, split_kw
from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL_STRESS = 1e-10
TOL_CTAN_LIN = 1e-8
TOL_CTAN = 5e-6
TOL_VARS = 5e-10


def run_pair(name, gpu_lib, check_vars=True, cost_exact=True, tol_ctan=TOL_CTAN):
    import micropp_gb300 as mg
    kw, steps = case(name)
    n, kw2 = split_kw(kw)
    o = orc.OracleRVE(oracle_config(n, **kw2))
    g = mg.Micropp(gpu_config(n, **kw2))
    assert rel_err(g.ctan_lin(), o.ctan_lin()) < TOL_CTAN_LIN
    assert np.array_equal(g.elem_type(), o.elem_type())
    for st in steps:
        for gp, e in enumerate(st):
            o.set_strain(gp, e)
            g.set_strain(gp, e)
        o.homogenize()
        g.homogenize()
        for gp in range(len(st)):
            assert g.has_converged(gp) == o.has_converged(gp)
            assert g.is_non_linear(gp) == o.is_non_linear(gp)
            assert g.has_subiterated(gp) == o.has_subiterated(gp)
            es = rel_err(g.get_stress(gp), o.get_stress(gp))
            ec = rel_err(g.get_ctan(gp), o.get_ctan(gp))
            assert es < TOL_STRESS, (name, gp, es)
            assert ec < tol_ctan, (name, gp, ec)
            assert rel_err(g.u(gp, 1), o.u(gp, 1)) < 1e-10
            if check_vars:
                assert rel_err(g.vars(gp, 1), o.vars(gp, 1)) < TOL_VARS
            if cost_exact:
                assert g.get_cost(gp) == o.get_cost(gp)
                assert g.newton(gp) == o.newton(gp)
        o.update_vars()
        g.update_vars()
    assert g.get_non_linear_gps() == o.get_non_linear_gps()
    return g, o


def test_c1_sphere_elastic(gpu_lib):
    run_pair("c1_sphere_elastic", gpu_lib)


def test_c1_sphere_elastic_cg_tol_1e8(gpu_lib):
    """C1 at its stated CG tolerance 1e-8 (cg_rel_tol), against the oracle and the fixture of the reference
    compiled with CG_REL_TOL = 1e-8 (ell.hpp:35)."""
    import os
    g, _ = run_pair("c1_sphere_elastic_cg1e8", gpu_lib)
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_c1_sphere_elastic_cg1e8.npz"))
    assert rel_err(g.get_stress(0), ref["stress"][-1][0]) < TOL_STRESS
    assert g.get_cost(0) == ref["cost"][-1][0] == 32
    assert rel_err(g.ctan_lin(), ref["ctan_lin"]) < TOL_CTAN_LIN


def test_fe_linear_next_to_fe_full_and_homogenize_linear(gpu_lib):
    """FE_LINEAR points (stress = ctan_lin strain, no FE solve, cost 0) beside an FE_FULL damage point
    (homogenize.cpp:68-99), then micropp3_homogenize_linear over all points (homogenize.cpp:51-66): against
    the oracle and the compiled reference's fixture."""
    import os
    g, o = run_pair("linear_full", gpu_lib)
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_linear_full.npz"))
    assert [g.get_cost(gp) for gp in range(3)] == [0, ref["cost"][-1][1], 0]
    lin = linear_pass("linear_full")
    for gp, e in enumerate(lin):
        g.set_strain(gp, e)
        o.set_strain(gp, e)
    g.homogenize_linear()
    o.homogenize_linear()
    for gp in range(3):
        # stress = ctan strain: held to the tolerance of the point's ctan (a nonlinear point's is a forward
        # difference, see the module docstring); the linear pass leaves ctan as it was
        tol = TOL_CTAN if o.is_non_linear(gp) else TOL_CTAN_LIN
        assert rel_err(g.get_stress(gp), o.get_stress(gp)) < tol
        assert rel_err(g.get_stress(gp), ref["stress_linear"][gp]) < tol
        assert rel_err(g.get_ctan(gp), o.get_ctan(gp)) < tol


def test_damage_layers_two_points(gpu_lib):
    run_pair("damage_layers", gpu_lib)


def test_plastic_sphere(gpu_lib):
    run_pair("plastic_sphere", gpu_lib)


@pytest.mark.parametrize("law", [0, 1, 2])
def test_reference_golden_tables(gpu_lib, law):
    """benchmark-{elastic,plastic,damage}.cpp: one element (n=2 nodes), 10 steps of eps_xx = 0.1 t."""
    import json
    import os

    import micropp_gb300 as mg
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "benchmark_tables.json")))
    key = ["elastic", "plastic", "damage"][law]
    table = np.array(gold[key]["sig"])
    tol = gold[key]["tol"]
    mats = [mg.material(*gold[key]["material"]), mg.material(0, 3e7, 0.25), mg.material(0, 3e7, 0.25)]
    g = mg.Micropp(mg.config(1, mats=mats, lin_stress=0))
    t = 0.0
    for s in range(10):
        eps = np.zeros(6)
        eps[0] = 0.1 * t
        g.set_strain(0, eps)
        g.homogenize()
        assert np.max(np.abs(g.get_stress(0) - table[s])) < tol
        g.update_vars()
        t += 0.015


def _compare_steps(g, o, strains_per_step, tol_ctan=TOL_CTAN, check_cost=True):
    for st in strains_per_step:
        for gp, e in enumerate(st):
            o.set_strain(gp, e)
            g.set_strain(gp, e)
        o.homogenize()
        g.homogenize()
        for gp in range(len(st)):
            assert rel_err(g.get_stress(gp), o.get_stress(gp)) < TOL_STRESS
            assert rel_err(g.get_ctan(gp), o.get_ctan(gp)) < tol_ctan
            assert g.has_converged(gp) == o.has_converged(gp)
            assert g.has_subiterated(gp) == o.has_subiterated(gp)
            assert g.is_non_linear(gp) == o.is_non_linear(gp)
            if check_cost:
                assert g.get_cost(gp) == o.get_cost(gp)
        o.update_vars()
        g.update_vars()


def test_non_cubic_mesh(gpu_lib):
    """5 x 7 x 4 elements, a z-fibre (MIC_CILI_FIB_Z), damage matrix."""
    mats = ((2, 1e7, 0.25, 0, 0, 1e5), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0))
    kw = dict(micro_type=4, geo=(0.25, 0, 0, 0), mats=mats, coupling=[2], lin_stress=0, nr_max_its=12)
    o = orc.OracleRVE(oracle_config((5, 7, 4), **kw))
    g = __import__("micropp_gb300").Micropp(gpu_config((5, 7, 4), **kw))
    assert np.array_equal(g.elem_type(), o.elem_type())
    base = np.array([1e-2, 2e-2, -5e-3, 4e-3, -2e-3, 6e-3])
    _compare_steps(g, o, [[base * s / 2] for s in (1, 2)])


@pytest.mark.parametrize("seed", [1, 2])
def test_subiterations_mixture_rule_one_way(gpu_lib, seed):
    """Three points: FE_FULL, FE_ONE_WAY and MIX_RULE_CHAMIS, nr_max_its = 2 to force sub-iterations."""
    import micropp_gb300 as mg
    rng = np.random.default_rng(seed)
    law = [(2, 1e7, 0.25, 0, 0, 1e5), (1, 1e7, 0.3, 1e5, 1e4, 0)][seed % 2]
    mats = (law, (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0))
    kw = dict(ngp=3, micro_type=1, geo=(0.25, 0, 0, 0), mats=mats, coupling=[2, 1, 3], lin_stress=0, nr_max_its=2,
              subiterations=1, nsubiterations=3)
    o = orc.OracleRVE(oracle_config(5, **kw))
    g = mg.Micropp(gpu_config(5, **kw))
    steps = [[rng.uniform(-1.5e-2, 1.5e-2, 6) for _ in range(3)] for _ in range(3)]
    _compare_steps(g, o, steps)


@pytest.mark.parametrize("law,its_with_A0", [(0, 1), (1, 2)])
def test_use_A0(gpu_lib, law, its_with_A0):
    """use_A0: the first its_with_A0 Newton iterations (also of the linear-ctan and the perturbed solves) solve
    with the Jacobian at u = 0 (micropp.cpp:128-143, solve.cpp:55-66); same costs as the oracle, which is
    pinned to the compiled reference on this option."""
    import micropp_gb300 as mg
    lawp = [(2, 1e7, 0.25, 0, 0, 1e5), (1, 1e7, 0.3, 1e5, 1e4, 0)][law]
    mats = (lawp, (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0))
    kw = dict(ngp=2, micro_type=1, geo=(0.25, 0, 0, 0), mats=mats, coupling=[2, 1], lin_stress=0, nr_max_its=8,
              use_A0=1, its_with_A0=its_with_A0)
    o = orc.OracleRVE(oracle_config(5, **kw))
    g = mg.Micropp(gpu_config(5, **kw))
    assert rel_err(g.ctan_lin(), o.ctan_lin()) < TOL_CTAN_LIN
    rng = np.random.default_rng(law)
    _compare_steps(g, o, [[rng.uniform(-2e-2, 2e-2, 6) for _ in range(2)] for _ in range(3)])


def test_restart_roundtrip(gpu_lib, tmp_path, monkeypatch):
    """write_restart produces the reference's bytes; read_restart into a new handle continues identically."""
    import micropp_gb300 as mg
    monkeypatch.chdir(tmp_path)
    mats = ((2, 1e7, 0.25, 0, 0, 1e5), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0))
    kw = dict(ngp=2, micro_type=1, geo=(0.25, 0, 0, 0), mats=mats, coupling=[2, 2], lin_stress=0, nr_max_its=12)
    o = orc.OracleRVE(oracle_config(4, **kw))
    g = mg.Micropp(gpu_config(4, **kw))
    e1 = [np.array([3e-2, 0, 0, 0, 0, 0]), np.array([1e-4, 0, 0, 0, 0, 0])]
    _compare_steps(g, o, [e1])
    g.write_restart(3)
    o.write_restart(str(tmp_path / "oracle.bin"))
    a = (tmp_path / "micropp-restart-0-3.bin").read_bytes()
    b = (tmp_path / "oracle.bin").read_bytes()
    assert len(a) == len(b) and a[0] == b[0]
    va = np.frombuffer(a[1:1 + 8 * g.nelem * 56], dtype=np.float64)
    vb = np.frombuffer(b[1:1 + 8 * g.nelem * 56], dtype=np.float64)
    assert rel_err(va, vb) < TOL_VARS
    g2 = mg.Micropp(gpu_config(4, **kw))
    g2.read_restart(3)
    e2 = [np.array([4e-2, 1e-3, 0, 0, 0, 0]), np.array([2e-4, 0, 0, 0, 0, 0])]
    for r in (g, g2):
        for gp in range(2):
            r.set_strain(gp, e2[gp])
    g.homogenize()
    g2.homogenize()
    # Point 0 is nonlinear, so its restart record holds vars_n and u_n and the continuation is identical.
    # Point 1 is still linear: the reference's format keeps no u_n for it (gp.hpp:107-113), its Newton
    # solve restarts from u = 0 and agrees within the Newton tolerance only.
    assert g.is_non_linear(0) and not g.is_non_linear(1)
    assert rel_err(g2.get_stress(0), g.get_stress(0)) < 1e-14
    assert rel_err(g2.get_stress(1), g.get_stress(1)) < 1e-3
    for gp in range(2):
        assert g2.is_non_linear(gp) == g.is_non_linear(gp)


def test_reference_constructor_signature(gpu_lib):
    """micropp3_new as the reference wrapper: sub-iterations forced on, lin_stress default (true)."""
    import ctypes

    import micropp_gb300 as mg
    L = gpu_lib
    h = mg.Handle()
    size = (ctypes.c_int * 3)(7, 7, 7)
    geo = (ctypes.c_double * 4)(0.2, 0.2, 0.2, 0.2)
    specs = [(2, 1e7, 0.25, 0, 0, 1e5), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0)]
    mats = (mg.MaterialBase * 3)(*[mg.material(*m) for m in specs])
    coup = (ctypes.c_int * 2)(2, 2)
    L.micropp3_new(ctypes.byref(h), 2, size, 1, geo, mats, coup, 4, 0)
    assert h.ptr
    o = orc.OracleRVE(oracle_config(6, ngp=2, micro_type=1, geo=(0.2, 0.2, 0.2, 0.2), mats=specs, coupling=[2, 2],
                                    subiterations=1, nsubiterations=4))
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    for step in range(3):
        for gp in range(2):
            e = np.array([1.2e-2, -3e-3, 0, 4e-3, 0, 0]) * (step + 1) * (gp + 1) / 2
            L.micropp3_set_strain(ctypes.byref(h), gp, dp(e))
            o.set_strain(gp, e)
        L.micropp3_homogenize(ctypes.byref(h))
        o.homogenize()
        for gp in range(2):
            s, c = np.zeros(6), np.zeros(36)
            L.micropp3_get_stress(ctypes.byref(h), gp, dp(s))
            L.micropp3_get_ctan(ctypes.byref(h), gp, dp(c))
            assert rel_err(s, o.get_stress(gp)) < TOL_STRESS
            tol = TOL_CTAN if o.is_non_linear(gp) else TOL_CTAN_LIN
            assert rel_err(c.reshape(6, 6), o.get_ctan(gp)) < tol
            assert L.micropp3_get_cost(ctypes.byref(h), gp) == o.get_cost(gp)
            assert L.micropp3_has_subiterated(ctypes.byref(h), gp) == o.has_subiterated(gp)
            assert L.micropp3_is_non_linear(ctypes.byref(h), gp) == o.is_non_linear(gp)
        L.micropp3_update_vars(ctypes.byref(h))
        o.update_vars()
    assert L.micropp3_get_non_linear_gps(ctypes.byref(h)) == o.get_non_linear_gps()
    L.micropp3_free(ctypes.byref(h))


def test_nonfinite_and_caps_report_status(gpu_lib):
    """A NaN strain, a damage threshold that fully damages points (the literal r0 ~ 2e3, for which the
    reference returns NaN), a CG capped at 5 iterations and Newton capped at 1: statuses, no hang."""
    import micropp_gb300 as mg
    mats = ((2, 1e7, 0.25, 0, 0, 2e3), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0))
    kw = dict(ngp=4, micro_type=1, geo=(0.2, 0, 0, 0), mats=mats, coupling=[2, 2, 2, 2], lin_stress=0,
              nr_max_its=12)
    g = mg.Micropp(gpu_config(6, **kw))
    o = orc.OracleRVE(oracle_config(6, **kw))
    strains = [np.full(6, np.nan), np.array([2e-2, 0, 0, 0, 0, 0]), np.array([1e-5, 0, 0, 0, 0, 0]),
               np.array([1e-6, 0, 0, 0, 0, 0])]
    for r in (g, o):
        for gp, e in enumerate(strains):
            r.set_strain(gp, e)
        r.homogenize()
    assert g.status(0) & mg.STATUS_NONFINITE
    assert np.isnan(g.get_stress(0)).all() and np.isnan(o.get_stress(0)).all()
    assert np.isnan(g.get_stress(1)).any() == np.isnan(o.get_stress(1)).any()
    for gp in (2, 3):
        assert g.status(gp) == mg.STATUS_OK
        assert rel_err(g.get_stress(gp), o.get_stress(gp)) < TOL_STRESS
    kw2 = dict(micro_type=1, geo=(0.2, 0, 0, 0), mats=((0, 1e7, 0.25, 0, 0, 0), (0, 1e8, 0.25, 0, 0, 0),
                                                       (0, 1e7, 0.25, 0, 0, 0)),
               coupling=[2], lin_stress=0, cg_max_its=5, nr_max_its=1, calc_ctan_lin=0)
    g2 = mg.Micropp(gpu_config(8, **kw2))
    o2 = orc.OracleRVE(oracle_config(8, **kw2))
    for r in (g2, o2):
        r.set_strain(0, np.array([1e-3, 0, 0, 0, 0, 0]))
        r.homogenize()
    assert g2.status(0) == (mg.STATUS_NEWTON_MAX_ITS | mg.STATUS_CG_MAX_ITS)
    assert not g2.has_converged(0) and not o2.has_converged(0)
    assert g2.get_cost(0) == o2.get_cost(0) == 5
    assert rel_err(g2.get_stress(0), o2.get_stress(0)) < TOL_STRESS


def test_batched_points_equal_single_runs(gpu_lib):
    """Five FE_FULL points of one handle, solved in one batch, each equal to its oracle run."""
    import micropp_gb300 as mg
    mats = ((2, 1e7, 0.25, 0, 0, 1e5), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0))
    n = 6
    kw = dict(ngp=5, elem_type=__import__("micropp_gb300.workloads", fromlist=["x"]).layers_z(n), mats=mats,
              coupling=[2] * 5, lin_stress=0, nr_max_its=12)
    g = mg.Micropp(gpu_config(n, **kw))
    o = orc.OracleRVE(oracle_config(n, **kw))
    rng = np.random.default_rng(7)
    steps = [[rng.uniform(-2.5e-2, 2.5e-2, 6) * s / 2 for _ in range(5)] for s in (1, 2)]
    _compare_steps(g, o, steps)
