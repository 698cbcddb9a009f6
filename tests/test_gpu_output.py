"""VTU field output (micropp3_output, output.cpp:29-214) against the compiled reference's files.

The fixtures tests/golden/ref_output_{damage,j2}.vtu were written by the reference's micropp<3>::output for a
3^3 RVE (tests/golden/make_golden.py, vtu_cases).  Structure and integers must be identical; floating-point
fields, printed with 7 significant digits, must agree to 1e-6 of the largest magnitude of their array.
"""
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")

CASES = {
    "damage": ([(2, 1e7, 0.25, 0, 0, 1e5), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0)],
               [np.array([3e-2, -1e-2, 0, 1e-2, 0, 0])]),
    "j2": ([(1, 1e7, 0.3, 1e5, 1e4, 0), (0, 1e8, 0.25, 0, 0, 0), (0, 1e7, 0.25, 0, 0, 0)],
           [np.array([1e-2, 0, 0, 2e-3, 0, 0]) * s for s in (1, 2)]),
}


def parse(path):
    """Split a VTU file into (tag lines, arrays of numbers between them)."""
    text = open(path).read()
    parts = re.split(r"(<[^>]*>)", text)
    tags, arrays = [], []
    for p in parts:
        if p.startswith("<"):
            tags.append(p)
        elif p.strip():
            arrays.append(np.array([float(x) for x in p.split()]))
    return tags, arrays


@pytest.mark.parametrize("tag", ["damage", "j2"])
def test_vtu_matches_reference(gpu_lib, tmp_path, tag):
    import micropp_gb300 as mg
    specs, path = CASES[tag]
    cfg = mg.config(3, micro_type=1, geo=(0.3, 0, 0, 0), mats=[mg.material(*m) for m in specs], coupling=[2],
                    lin_stress=0, nr_max_its=12, nr_max_tol=1e-5)
    g = mg.Micropp(cfg)
    for e in path:
        g.set_strain(0, e)
        g.homogenize()
        g.update_vars()
    g.set_strain(0, path[-1] * 1.2)
    g.homogenize()
    out = str(tmp_path / f"gpu_{tag}")
    g._call("micropp3_output", 0, out.encode())
    t_ref, a_ref = parse(os.path.join(GOLD, f"ref_output_{tag}.vtu"))
    t_gpu, a_gpu = parse(out + ".vtu")
    assert t_ref == t_gpu
    assert len(a_ref) == len(a_gpu)
    for x, y in zip(a_gpu, a_ref):
        assert x.shape == y.shape
        scale = max(np.max(np.abs(y)), 1e-300)
        assert np.max(np.abs(x - y)) <= 1e-6 * scale
