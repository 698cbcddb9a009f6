"""The forward-mode derivatives of the Gauss-point laws used by the adjoint (micropp_gb300/csrc/adjoint_laws.h)
against central differences of the same laws, on every branch of the three laws.  Built with the host
compiler; no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dual_derivatives_match_central_differences(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "adjoint_law_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "micropp_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "adjoint_law_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    lines = [l.split() for l in r.stdout.splitlines()]
    assert len(lines) == 30, r.stdout
    for name, _, err in lines:
        assert float(err) < 1e-5, (name, err)
    assert r.returncode == 0
    # every branch exercised: the plastic and the loading cases have nonzero history derivatives
    assert {l[0] for l in lines} == {"elastic", "j2-elastic", "j2-plastic", "damage-below", "damage-unload",
                                      "damage-loading"}
