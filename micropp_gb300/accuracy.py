"""Error of the fast form against a tightly converged FP64 solution, measured with the library itself.

The FP64 solution is the plain form (the reference algorithm in FP64: Newton with the forward-difference
law tangent and Jacobi-preconditioned CG, homogenize.cpp:188-282, solve.cpp:28-82, ell.cpp:66-122) run far
below the reference's tolerances: CG to 1e-12 and Newton to 1e-11 of their initial residuals, with the
absolute Newton stop switched off.  Its ctan is a central difference of that stress,
ctan[:, j] = (sigma(eps + h e_j) - sigma(eps - h e_j)) / 2h with h = 1e-7.  The thirteen solves (eps and
eps +- h e_j) are thirteen FE_ONE_WAY points of one handle (stress only, homogenize.cpp:215-232), so they run
as one batch and share the accepted history of the previous macro step.

Errors are relative to the largest entry of the FP64 tensor: max |a - b| / max |b|.
"""
import numpy as np

# Tolerances of the FP64 solution.
TIGHT = dict(precision=0, ctan_mode=0, cg_rel_tol=1e-12, cg_abs_tol=1e-300, cg_max_its=20000, nr_rel_tol=1e-11,
             nr_max_tol=1e-30, nr_max_its=30, calc_ctan_lin=0, lin_stress=0)
H = 1e-7


def rel_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / s if s > 0 else float(np.max(np.abs(a)))


def fp64_solution(n, mats, elem_type, history_strain, strain, h=H, **over):
    """Stress and central-difference ctan at `strain` of an RVE whose history is that of `history_strain`,
    accepted.  Returns (stress (6,), ctan (6, 6), statuses of the 13 solves, Newton iterations of the eps
    solve)."""
    import micropp_gb300 as mg
    cfg = dict(TIGHT, **over)
    r = mg.Micropp(mg.config(n, ngp=13, mats=mats, coupling=[mg.FE_ONE_WAY] * 13, elem_type=elem_type, **cfg))
    try:
        if history_strain is not None:
            for gp in range(13):
                r.set_strain(gp, history_strain)
            r.homogenize()
            r.update_vars()
        eps = np.asarray(strain, dtype=np.float64)
        r.set_strain(0, eps)
        for j in range(6):
            d = np.zeros(6)
            d[j] = h
            r.set_strain(1 + 2 * j, eps + d)
            r.set_strain(2 + 2 * j, eps - d)
        r.homogenize()
        stress = r.get_stress(0)
        ctan = np.zeros((6, 6))
        for j in range(6):
            ctan[:, j] = (r.get_stress(1 + 2 * j) - r.get_stress(2 + 2 * j)) / (2 * h)
        status = [r.status(gp) for gp in range(13)]
        newton = r.newton(0)
    finally:
        r.close()
    return stress, ctan, status, newton


def fast_solution(n, mats, elem_type, history_strains, strains, fast_cfg):
    """The RVEs (one per entry of `strains`) through the fast form as Gauss points of one handle: the previous
    step at history_strains[i] accepted, then stress + ctan at strains[i].  Returns [(stress, ctan, status)]."""
    import micropp_gb300 as mg
    k = len(strains)
    f = mg.Micropp(mg.config(n, ngp=k, mats=mats, coupling=[mg.FE_FULL] * k, elem_type=elem_type,
                             lin_stress=0, calc_ctan_lin=0, **fast_cfg))
    try:
        for i in range(k):
            f.set_strain(i, history_strains[i])
        f.homogenize()
        f.update_vars()
        for i in range(k):
            f.set_strain(i, strains[i])
        f.homogenize()
        return [(f.get_stress(i), f.get_ctan(i), f.status(i)) for i in range(k)]
    finally:
        f.close()


def compare(fast, fp64):
    """Largest stress and ctan errors of fast_solution's results against fp64_solution's, with per-RVE
    detail."""
    per = []
    for (sf, cf, stf), (s64, c64, st64, nw) in zip(fast, fp64):
        per.append(dict(stress=rel_err(sf, s64), ctan=rel_err(cf, c64), fast_status=stf, fp64_status=max(st64),
                        fp64_newton_its=nw[0]))
    return dict(stress=max(p["stress"] for p in per), ctan=max(p["ctan"] for p in per), rves=per,
                reference=f"plain FP64 form, CG 1e-12, Newton 1e-11; ctan by central differences, h = {H:g}")


def fast_vs_fp64(n, mats, elem_type, history_strains, strains, fast_cfg):
    """fast_solution against fp64_solution on the same RVEs; returns compare()'s record."""
    fast = fast_solution(n, mats, elem_type, history_strains, strains, fast_cfg)
    fp64 = [fp64_solution(n, mats, elem_type, h, e) for h, e in zip(history_strains, strains)]
    return compare(fast, fp64)
