"""Generate the golden fixtures of tests/golden/ from the reference (run where the reference tree exists).

1. benchmark_tables.json -- the known-answer tables of the reference's own tests
   test/benchmark-{elastic,plastic,damage}.cpp (sig_sol[10][6], tolerance, material), parsed from those
   files, together with the outputs of the compiled reference (oracle/_ref) on the same 10-step paths.
2. ref_<case>.npz -- outputs of the compiled reference on the seeded parity cases of tests/cases.py:
   per step and Gauss point the average stress, ctan, cost, flags, and the internal variables and the
   displacement of the last step; for cases with a final homogenize_linear pass, its stresses.  The case
   c1_sphere_elastic_cg1e8 comes from the reference built with CG_REL_TOL = 1e-8 (libref_cg1e8).
3. ref_output_damage.vtu -- the reference's VTU field output (micropp<3>::output) of a 3^3 damage RVE after
   one nonlinear step, and ref_output_j2.vtu for a J2 matrix.

Usage: python tests/golden/make_golden.py REFERENCE_ROOT   (or MICROPP_REFERENCE; needs oracle/build_ref.sh)
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import pyoracle as orc  # noqa: E402


def parse_table(path):
    text = open(path).read()
    body = re.search(r"sig_sol\[time_steps\]\[6\]\s*=\s*\{(.*?)\};", text, flags=re.S).group(1)
    rows = re.findall(r"\{([^{}]*)\}", body)
    sig = [[float(x) for x in r.split(",")] for r in rows]
    tol = float(re.search(r"fabs\(sig_sol\[t\]\[i\] - sig\[i\]\) < ([0-9.eE+-]+)\)", text).group(1))
    m = re.search(r"material_set\(&mic_params\.materials\[0\],\s*([^)]*)\)", text).group(1)
    vals = [float(x) for x in m.split(",")]
    material = [int(vals[0])] + vals[1:]
    return sig, tol, material


def run_table_case(material):
    cfg = orc.make_config(1, mats=[orc.material(*material), orc.material(0, 3e7, 0.25), orc.material(0, 3e7, 0.25)],
                          lin_stress=0)
    r = orc.RefRVE(cfg)
    out = []
    t = 0.0
    for _ in range(10):
        eps = np.zeros(6)
        eps[0] = 0.1 * t
        r.set_strain(0, eps)
        r.homogenize()
        out.append(r.get_stress(0).tolist())
        r.update_vars()
        t += 0.015
    r.close()
    return out


def run_case(name):
    from cases import REF_VARIANT, case, linear_pass, oracle_config, split_kw
    kw, steps = case(name)
    n, kw2 = split_kw(kw)
    r = orc.RefRVE(oracle_config(n, **kw2), variant=REF_VARIANT.get(name, "stock"))
    rec = {"stress": [], "ctan": [], "cost": [], "converged": [], "nonlinear": []}
    for st in steps:
        for gp, e in enumerate(st):
            r.set_strain(gp, e)
        r.homogenize()
        ng = len(st)
        rec["stress"].append([r.get_stress(g) for g in range(ng)])
        rec["ctan"].append([r.get_ctan(g) for g in range(ng)])
        rec["cost"].append([r.get_cost(g) for g in range(ng)])
        rec["converged"].append([r.has_converged(g) for g in range(ng)])
        rec["nonlinear"].append([r.is_non_linear(g) for g in range(ng)])
        last_vars = [r.vars(g, 1) for g in range(ng)]
        last_u = [r.u(g, 1) for g in range(ng)]
        r.update_vars()
    arrays = {k: np.array(v) for k, v in rec.items()}
    arrays["vars_k_last"] = np.array(last_vars)
    arrays["u_k_last"] = np.array(last_u)
    arrays["ctan_lin"] = r.ctan_lin()
    lin = linear_pass(name)
    if lin is not None:
        for gp, e in enumerate(lin):
            r.set_strain(gp, e)
        r.homogenize_linear()
        arrays["stress_linear"] = np.array([r.get_stress(g) for g in range(len(lin))])
    r.close()
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **arrays)


def vtu_cases():
    """(tag, config keywords, strain path) of the VTU fixtures (shared with tests/test_gpu_output.py)."""
    import numpy as np
    dmg = [orc.material(2, 1e7, 0.25, 0, 0, 1e5), orc.material(0, 1e8, 0.25), orc.material(0, 1e7, 0.25)]
    j2 = [orc.material(1, 1e7, 0.3, 1e5, 1e4), orc.material(0, 1e8, 0.25), orc.material(0, 1e7, 0.25)]
    common = dict(micro_type=1, geo=(0.3, 0, 0, 0), coupling=[2], lin_stress=0, nr_max_its=12, nr_max_tol=1e-5)
    return [("damage", dict(mats=dmg, **common), [np.array([3e-2, -1e-2, 0, 1e-2, 0, 0])]),
            ("j2", dict(mats=j2, **common), [np.array([1e-2, 0, 0, 2e-3, 0, 0]) * s for s in (1, 2)])]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MICROPP_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py REFERENCE_ROOT  (or set MICROPP_REFERENCE)")
    tables = {}
    for key in ("elastic", "plastic", "damage"):
        sig, tol, material = parse_table(os.path.join(ref, "test", f"benchmark-{key}.cpp"))
        tables[key] = {"source": f"test/benchmark-{key}.cpp", "sig": sig, "tol": tol, "material": material,
                       "ref_output": run_table_case(material)}
    with open(os.path.join(HERE, "benchmark_tables.json"), "w") as f:
        json.dump(tables, f, indent=1)
    for name in ("c1_sphere_elastic", "damage_layers", "plastic_sphere", "c1_sphere_elastic_cg1e8",
                 "linear_full"):
        run_case(name)
    for tag, cfg_kw, eps in vtu_cases():
        r = orc.RefRVE(orc.make_config(3, **cfg_kw))
        for e in eps:
            r.set_strain(0, e)
            r.homogenize()
            r.update_vars()
        r.set_strain(0, eps[-1] * 1.2)
        r.homogenize()
        r.output(0, os.path.join(HERE, f"ref_output_{tag}"))
        r.close()
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
