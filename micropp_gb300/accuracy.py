"""Error of the fast form against a tightly converged FP64 solution, measured with the library itself.

The FP64 solution comes from the library's FP64 load-path solver (micropp3_path_forward): FP64 Newton with
the exact consistent tangent of the laws (forward-mode dual numbers), BiCGSTAB corrections to 1e-12 and the
Newton residual to 1e-11 of its initial value, absolute stop off -- a solver that shares no code with the fast
form's FP32 Jacobian, FP32 CG, double-float residual and implicit ctan beyond the laws.  The path takes the
previous macro step (history strain) and accepts it, then the step to the strain checked.  Its ctan is exact
in FP64 too: for L = sigma_k of the last step, the reverse-mode pass (micropp3_path_vjp) gives
dL/d(strain of the last step) = row k of ctan, since that strain reaches sigma only through the last step's
solve.  (A central difference of the stress is no good reference here: with a damage matrix, a step of
h = 1e-7 in the strain moves some Gauss points across the loading/unloading switch or a kink of the softening
curve, and on 60^3 RVEs that alone moved the difference by 1.2e-5 -- for every preconditioner alike.)

Errors are relative to the largest entry of the FP64 tensor: max |a - b| / max |b|.
"""
import numpy as np

# Tolerances of the FP64 solution (the path solver's BiCGSTAB stops at max(cg_rel_tol, 1e-14) of ||b||).
TIGHT = dict(precision=0, ctan_mode=0, cg_rel_tol=1e-12, cg_abs_tol=1e-300, cg_max_its=20000, nr_rel_tol=1e-11,
             nr_max_tol=1e-30, nr_max_its=30, calc_ctan_lin=0, lin_stress=0)
H = 1e-7  # strain step of the central differences of the precision workload


def rel_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / s if s > 0 else float(np.max(np.abs(a)))


def fp64_solution(n, mats, elem_type, history_strain, strain, **over):
    """FP64 stress and ctan at `strain` of an RVE whose previous step, to `history_strain`, was accepted (None:
    no previous step), by the FP64 path solver and its reverse-mode pass.  Returns (stress (6,), ctan (6, 6),
    status bits of the path's steps, Newton iterations of the last step)."""
    import micropp_gb300 as mg
    cfg = dict(TIGHT, **over)
    strains = [strain] if history_strain is None else [history_strain, strain]
    e = np.asarray(strains, dtype=np.float64).reshape(-1, 6)
    ns = e.shape[0]
    params = np.array([[m.E, m.nu, m.Xt, m.Sy, m.Ka] for m in mats])
    r = mg.Micropp(mg.config(n, mats=mats, coupling=[mg.FE_FULL], elem_type=elem_type, **cfg))
    try:
        sig, rc = r.path_forward(e, params, checkpoint_every=ns)
        if rc != 0:
            raise RuntimeError(f"FP64 path solver returned {rc}")
        newton = [r.path_newton(k) for k in range(ns)]
        ctan = np.zeros((6, 6))
        for k in range(6):
            g = np.zeros((ns, 6))
            g[-1, k] = 1.0
            _, gs, rc = r.path_vjp(g)
            if rc != 0:
                raise RuntimeError(f"FP64 reverse pass returned {rc}")
            ctan[k, :] = gs[-1]
    finally:
        r.close()
    # the path reports converged + 2 x (a linear solve stopped at its cap); as the library's status bits:
    status = [(0 if nw[2] & 1 else mg.STATUS_NEWTON_MAX_ITS) | (mg.STATUS_CG_MAX_ITS if nw[2] & 2 else 0)
              for nw in newton]
    return sig[-1].copy(), ctan, status, newton[-1]


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
                        fp64_newton_its=nw[0], fp64_rel_residual=nw[3]))
    return dict(stress=max(p["stress"] for p in per), ctan=max(p["ctan"] for p in per), rves=per,
                reference="FP64 path solver (exact tangent, BiCGSTAB 1e-12, Newton 1e-11); ctan by its reverse "
                          "pass")


def fast_vs_fp64(n, mats, elem_type, history_strains, strains, fast_cfg):
    """fast_solution against fp64_solution on the same RVEs; returns compare()'s record."""
    fast = fast_solution(n, mats, elem_type, history_strains, strains, fast_cfg)
    fp64 = [fp64_solution(n, mats, elem_type, h, e) for h, e in zip(history_strains, strains)]
    return compare(fast, fp64)
