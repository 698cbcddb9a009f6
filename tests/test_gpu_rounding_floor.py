"""The FP64 form's nonlinear ctan against the rounding floor measured on the same case.

The ctan of a nonlinear point is a forward difference (step 1e-8) of average stresses that come out of Newton/CG
solves stopped at the reference's tolerances, so any valid FP64 implementation that sums in another order moves
it far more than the stress.  The floor of a case is measured here, on the machine that runs the test, as the
largest deviation from the oracle's stock build among four other valid FP64 builds of the same restatement:
  fma           every multiply-add contracted;
  blocked       dot products summed in blocks of 768 terms;
  gpuorder      the CG's dot products in the GPU library's reduction tree and the Jacobian assembled in its
                8-colour order;
  gpuorder_fma  gpuorder with contraction.
The GPU's deviation from the stock oracle is held to twice that floor at every nonlinear point.
"""
import platform

import numpy as np
import pytest

from cases import case, gpu_config, oracle_config, split_kw
from conftest import rel_err
from test_rounding_floor import _pair, _variant

pytestmark = pytest.mark.gpu

FMA = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
VARIANTS = {"fma": ["-ffp-contract=fast", *FMA], "blocked": ["-ffp-contract=off", "-DORC_BLOCKED_DOTS"],
            "gpuorder": ["-ffp-contract=off", "-DORC_GPU_ORDER"],
            "gpuorder_fma": ["-ffp-contract=fast", *FMA, "-DORC_GPU_ORDER"]}


@pytest.fixture(scope="module")
def variant_libs(tmp_path_factory):
    return {k: _variant(tmp_path_factory, k, f) for k, f in VARIANTS.items()}


@pytest.mark.parametrize("name", ["damage_layers", "plastic_sphere", "linear_full"])
def test_nonlinear_ctan_within_twice_the_rounding_floor(gpu_lib, variant_libs, name):
    import micropp_gb300 as mg
    kw, steps = case(name)
    n, kw2 = split_kw(kw)
    g = mg.Micropp(gpu_config(n, **kw2))
    ref = None
    others = {}
    for k, path in variant_libs.items():
        a, b = _pair(path, oracle_config(n, **kw2))
        ref = ref or a
        others[k] = b
    checked = 0
    for s, st in enumerate(steps):
        rs = [ref, g, *others.values()]
        for r in rs:
            for gp, e in enumerate(st):
                r.set_strain(gp, e)
            r.homogenize()
        for gp in range(len(st)):
            if not ref.is_non_linear(gp):
                continue
            c0 = ref.get_ctan(gp)
            floor = max(rel_err(b.get_ctan(gp), c0) for b in others.values())
            dev = rel_err(g.get_ctan(gp), c0)
            print(f"{name} step {s} point {gp}: GPU {dev:.2e}  floor {floor:.2e}")
            assert dev <= 2 * floor + 1e-13, (name, s, gp, dev, floor)
            checked += 1
        for r in rs:
            r.update_vars()
    assert checked > 0
