"""micropp3_homogenize_many: handles of different sizes and laws homogenized concurrently give exactly what
homogenizing them one by one gives (each handle has its own stream and workspace; every reduction has a
fixed order)."""
import ctypes

import numpy as np
import pytest

import micropp_gb300 as mg
from micropp_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _handles(precision):
    out = []
    for n, law in ((6, 1), (8, 2), (5, 0)):
        mats = [{0: mg.material(0, 1e7, 0.25), 1: mg.material(1, 1e7, 0.3, 1e5, 1e4),
                 2: mg.material(2, 1e7, 0.25, 0, 0, 1e5)}[law], mg.material(0, 1e8, 0.25), mg.material(0, 1e7, 0.25)]
        out.append(mg.Micropp(mg.config(n, ngp=2, mats=mats, coupling=[2, 2], elem_type=wl.layers_z(n), lin_stress=0,
                                        nr_max_its=12, nr_max_tol=1e-9, precision=precision,
                                        ctan_mode=precision)))
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_many_equals_one_by_one(gpu_lib, precision):
    L = mg.load()
    strains = [np.array([2e-2, -5e-3, 1e-3, 4e-3, 0, 1e-3]), np.array([-1e-2, 8e-3, 0, 0, 2e-3, 0])]
    results = []
    for concurrent in (False, True):
        hs = _handles(precision)
        for h in hs:
            for gp in range(2):
                h.set_strain(gp, strains[gp])
        if concurrent:
            arr = (ctypes.POINTER(mg.Handle) * len(hs))(*[ctypes.pointer(h.h) for h in hs])
            L.micropp3_homogenize_many(arr, len(hs))
            assert not L.micropp3_last_error()
        else:
            for h in hs:
                h.homogenize()
        results.append([(h.get_stress(gp), h.get_ctan(gp)) for h in hs for gp in range(2)])
        for h in hs:
            h.close()
    for (s0, c0), (s1, c1) in zip(*results):
        assert np.array_equal(s0, s1) and np.array_equal(c0, c1)
