"""The rounding floor of the parity tolerances.

Two valid FP64 builds of the same algorithm -- the oracle with every multiply and add rounded separately
(as the reference's x86-64 build), and the oracle with fused multiply-add contraction -- are compared on the
parity cases.  Their spread is the accuracy to which any other FP64 implementation (the GPU path sums in a
different order and contracts to FMA) can be expected to reproduce the reference.  The GPU parity tests use
1e-10 for stress and internal variables and 1e-8 for ctan except where this floor is above 1e-8 (J2).
"""
import ctypes
import os
import platform
import subprocess

import numpy as np
import pytest

import pyoracle as orc
from cases import case, oracle_config, split_kw
from conftest import rel_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _variant(tmp_path_factory, name, flags):
    out = tmp_path_factory.mktemp(name) / f"liboracle_{name}.so"
    subprocess.run(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp", *flags, "-o", str(out),
                    os.path.join(ROOT, "oracle", "micropp_oracle.c"), "-lm"], check=True)
    return str(out)


@pytest.fixture(scope="module")
def fma_oracle(tmp_path_factory):
    flags = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    return _variant(tmp_path_factory, "fma", ["-ffp-contract=fast", *flags])


@pytest.fixture(scope="module")
def blocked_oracle(tmp_path_factory):
    return _variant(tmp_path_factory, "blocked", ["-ffp-contract=off", "-DORC_BLOCKED_DOTS"])


def _pair(fma_path, cfg):
    class FmaRVE(orc.OracleRVE):
        pass
    FmaRVE.lib = ctypes.CDLL(fma_path)
    r = FmaRVE.__new__(FmaRVE)
    r._setup()
    orc._Base.__init__(r, cfg)
    return orc.OracleRVE(cfg), r


def spread(fma_path, name):
    kw, steps = case(name)
    n, kw2 = split_kw(kw)
    a, b = _pair(fma_path, oracle_config(n, **kw2))
    worst = {"stress": 0.0, "ctan": 0.0, "vars": 0.0}
    for st in steps:
        for gp, e in enumerate(st):
            a.set_strain(gp, e)
            b.set_strain(gp, e)
        a.homogenize()
        b.homogenize()
        for gp in range(len(st)):
            worst["stress"] = max(worst["stress"], rel_err(b.get_stress(gp), a.get_stress(gp)))
            worst["ctan"] = max(worst["ctan"], rel_err(b.get_ctan(gp), a.get_ctan(gp)))
            worst["vars"] = max(worst["vars"], rel_err(b.vars(gp, 1), a.vars(gp, 1)))
            assert a.get_cost(gp) == b.get_cost(gp)
        a.update_vars()
        b.update_vars()
    return worst


def test_floor_elastic_and_damage_within_tolerances(fma_oracle):
    for name in ("c1_sphere_elastic", "damage_layers"):
        w = spread(fma_oracle, name)
        assert w["stress"] < 1e-13 and w["ctan"] < 1e-8 and w["vars"] < 1e-10, (name, w)


@pytest.mark.parametrize("name", ["damage_layers", "plastic_sphere"])
def test_floor_blocked_summation(blocked_oracle, name):
    """The reference algorithm with GPU-like blocked dot products: stress agrees to ~1e-13, while the
    forward-difference ctan (step 1e-8) moves by up to ~1e-7 -- the level the GPU parity tests allow."""
    w = spread(blocked_oracle, name)
    assert w["stress"] < 1e-12, w
    assert w["ctan"] < 1e-6, w
    print(name, w)


def test_floor_j2_ctan_above_1e8(fma_oracle):
    """On the J2 case the spread of ctan between the two reference builds exceeds 1e-8 (measured 2.7e-8 on
    x86-64), which is why the GPU parity test of that case allows 1e-7."""
    w = spread(fma_oracle, "plastic_sphere")
    assert w["stress"] < 1e-12
    assert 1e-9 < w["ctan"] < 1e-7, w


@pytest.fixture(scope="module")
def gpuorder_oracle(tmp_path_factory):
    return _variant(tmp_path_factory, "gpuorder", ["-ffp-contract=off", "-DORC_GPU_ORDER"])


@pytest.mark.parametrize("name", ["damage_layers", "plastic_sphere"])
def test_floor_gpu_reduction_order(gpuorder_oracle, name):
    """The reference algorithm with the GPU library's CG reduction tree and colour-ordered assembly: the same
    costs, stress to ~1e-13, and the forward-difference ctan moved by up to ~1e-7 -- the floor against which
    the GPU's nonlinear ctan is held (tests/test_gpu_rounding_floor.py)."""
    w = spread(gpuorder_oracle, name)
    assert w["stress"] < 1e-12, w
    assert w["ctan"] < 1e-6, w
