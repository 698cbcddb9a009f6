"""The C-ABI library: it builds, loads without a GPU, exports every declared entry point, serves the C and
C++ headers as a drop-in, and fails loudly (never falls back to the CPU) when no GPU is present."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import micropp_gb300
    from micropp_gb300 import build
    build.build()
    return micropp_gb300.load()


def test_exports_every_declared_symbol(lib):
    import micropp_gb300
    names = micropp_gb300.declared_symbols()
    # every entry point of the reference's micropp_c.h and material_base.h is among them
    for must in ("micropp3_new", "micropp3_free", "micropp3_set_strain", "micropp3_get_stress", "micropp3_get_ctan",
                 "micropp3_homogenize", "micropp3_homogenize_linear", "micropp3_update_vars",
                 "micropp3_is_non_linear", "micropp3_get_cost", "micropp3_has_converged", "micropp3_has_subiterated",
                 "micropp3_output", "micropp3_output2", "micropp3_print_info", "micropp3_get_non_linear_gps",
                 "micropp3_write_restart", "micropp3_read_restart", "material_set", "material_print"):
        assert must in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_material_set_matches_reference_formulas(lib):
    import micropp_gb300 as mg
    m = mg.material(2, 3e7, 0.25, 1.0, 2.0, 1e5)
    assert (m.E, m.nu, m.Ka, m.Sy, m.Xt, m.type) == (3e7, 0.25, 1.0, 2.0, 1e5, 2)
    assert m.k == 3e7 / (3. * (1. - 2. * 0.25))
    assert m.mu == 3e7 / (2. * (1. + 0.25))
    assert m.lam == 0.25 * 3e7 / ((1. + 0.25) * (1. - 2. * 0.25))


def _cuda_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_cuda_present(), reason="checks the no-GPU failure path")
def test_no_gpu_fails_loudly(lib):
    import micropp_gb300 as mg
    with pytest.raises(RuntimeError, match="CUDA|device"):
        mg.Micropp(mg.config(2))
    # the reference constructor signature leaves a NULL handle and an error message
    h = mg.Handle()
    size = (ctypes.c_int * 3)(3, 3, 3)
    geo = (ctypes.c_double * 4)(0.1, 0.1, 0.1, 0.1)
    mats = (mg.MaterialBase * 3)(mg.material(0, 1e7, 0.25), mg.material(0, 1e7, 0.25), mg.material(0, 1e7, 0.25))
    coup = (ctypes.c_int * 1)(2)
    lib.micropp3_new(ctypes.byref(h), 1, size, 0, geo, mats, coup, 10, 0)
    assert not h.ptr
    assert lib.micropp3_last_error()


DROPIN_C = r"""
#include <stdio.h>
#include "micropp_c.h"
int main(void) {
  struct micropp3 m;
  struct material_base mats[3];
  int size[3] = {6, 6, 6}, coupling[2] = {FE_FULL_, FE_FULL_};
  double geo[4] = {0.2, 0.2, 0.2, 0.2}, eps[6] = {1e-3, 0, 0, 0, 0, 0}, sig[6], ctan[36];
  material_set(&mats[0], 0, 1e7, 0.25, 0, 0, 0);
  material_set(&mats[1], 0, 1e8, 0.25, 0, 0, 0);
  material_set(&mats[2], 0, 1e7, 0.25, 0, 0, 0);
  micropp3_new(&m, 2, size, 1, geo, mats, coupling, 10, 0);
  micropp3_set_strain(&m, 0, eps);
  micropp3_homogenize(&m);
  micropp3_get_stress(&m, 0, sig);
  micropp3_get_ctan(&m, 0, ctan);
  micropp3_update_vars(&m);
  printf("%d %d %d\n", micropp3_is_non_linear(&m, 0), micropp3_get_cost(&m, 0), micropp3_has_converged(&m, 0));
  micropp3_free(&m);
  return 0;
}
""".replace("FE_FULL_", "2")

DROPIN_CXX = r"""
#include <iostream>
#include "micropp.hpp"
int main() {
  micropp_params_t p;
  p.ngp = 1;
  p.size[0] = p.size[1] = p.size[2] = 6;
  p.type = MIC_SPHERE;
  p.geo_params[0] = 0.2;
  material_set(&p.materials[0], 2, 1e7, 0.25, 0, 0, 1e5);
  material_set(&p.materials[1], 0, 1e8, 0.25, 0, 0, 0);
  material_set(&p.materials[2], 0, 1e7, 0.25, 0, 0, 0);
  int coupling[1] = {FE_FULL};
  p.coupling = coupling;
  p.lin_stress = false;
  micropp<3> micro(p);
  double eps[6] = {1e-2, 0, 0, 0, 0, 0}, sig[6], ctan[36];
  micro.set_strain(0, eps);
  micro.homogenize();
  micro.get_stress(0, sig);
  micro.get_ctan(0, ctan);
  micro.update_vars();
  std::cout << micro.is_non_linear(0) << " " << micro.get_cost(0) << " " << micro.has_converged(0) << "\n";
  return 0;
}
"""


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_dropin_headers_compile_and_link(lib, tmp_path, lang):
    """A macro-scale driver written against the reference's C / C++ API compiles and links unchanged."""
    src = tmp_path / ("drv.c" if lang == "c" else "drv.cpp")
    src.write_text(DROPIN_C if lang == "c" else DROPIN_CXX)
    cc = "gcc" if lang == "c" else "g++"
    libdir = os.path.join(ROOT, "micropp_gb300")
    r = subprocess.run([cc, str(src), "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lmicropp_gb300",
                        f"-Wl,-rpath,{libdir}", "-o", str(tmp_path / "drv")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_product_never_reaches_the_oracle():
    """The package and its sources do not import, load or link anything under oracle/."""
    pat = re.compile(r"pyoracle|liboracle|micropp_oracle|oracle/")
    for d in ("micropp_gb300", "micropp_gb300/csrc", "include"):
        for f in os.listdir(os.path.join(ROOT, d)):
            p = os.path.join(ROOT, d, f)
            if os.path.isfile(p) and f.endswith((".py", ".cu", ".cuh", ".cpp", ".hpp", ".h", ".c")):
                assert not pat.search(open(p).read()), p


def test_ctypes_mirror_matches_c_layout(tmp_path):
    """The Python ctypes structs used by the tests and the bench have the C headers' field offsets and sizes
    (compiled with the host C compiler from include/)."""
    import micropp_gb300 as mg
    structs = [("struct micropp3_config", mg.Config, {}), ("struct material_base", mg.MaterialBase, {"lam": "lambda"})]
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "micropp_gb300.h"', "int main(void) {"]
    for cname, py, rename in structs:
        lines.append(f'  printf("{cname}:sizeof %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname}:{f} %zu\\n", offsetof({cname}, {rename.get(f, f)}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                                check=True).stdout.splitlines())
    for cname, py, _ in structs:
        assert int(out[f"{cname}:sizeof"]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out[f"{cname}:{f}"]) == getattr(py, f).offset, (cname, f)
