"""The sum-factorised strain and element residual of the trilinear hexahedron (micropp_gb300/csrc/hex_sumfact.h)
equal the B-matrix products of calc_bmat's gradients to rounding, on random displacements and stresses of a
non-cubic element.  Built with the host compiler; no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sum_factorisation_matches_b_matrix_products(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "sumfact_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "micropp_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "sumfact_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, check=True)
    errs = dict(line.split() for line in r.stdout.splitlines())
    assert set(errs) == {"strain", "residual"}
    for name, err in errs.items():
        assert float(err) < 1e-14, (name, err)
