"""The fast form's error against a tightly converged FP64 solution at the headline size, 60^3 elements.

Three RVEs of the headline workload (4 stiff layers normal to z in a damage matrix, the bench's seeded
strain targets): the previous step at half the target accepted, then stress + ctan at the target.  The fast
form (FP32 Jacobian and CG in FP64 refinement, implicit ctan), with the multigrid (FP32 or FP16 smoothing
operator) and with the Jacobi preconditioner, is held to the bars the fast form states: average stress
within 1e-7 and ctan within 1e-5 (relative to the largest entry) of the FP64 solution: the library's FP64
path solver (exact tangent, BiCGSTAB, Newton to 1e-11) and the exact FP64 ctan of its reverse-mode pass
(micropp_gb300.accuracy).
"""
import pytest

pytestmark = pytest.mark.gpu

TOL_STRESS = 1e-7
TOL_CTAN = 1e-5
N = 60
PICK = (0, 1, 2)


@pytest.fixture(scope="module")
def rves(gpu_lib):
    import micropp_gb300 as mg
    from micropp_gb300 import accuracy, workloads as wl
    et, xts, targets = wl.damage_layers_rves(N, 32, 2024)
    mats = wl.damage_layers_materials(mg, xts[0])
    hist = [0.5 * targets[i] for i in PICK]
    eps = [targets[i] for i in PICK]
    fp64 = [accuracy.fp64_solution(N, mats, et, h, e) for h, e in zip(hist, eps)]
    return dict(et=et, mats=mats, hist=hist, eps=eps, fp64=fp64)


@pytest.mark.parametrize("precond", [1, 2, 0], ids=["multigrid", "multigrid_fp16_smoothing", "jacobi"])
def test_fast_form_error_vs_fp64_at_60cubed(rves, precond):
    import micropp_gb300 as mg
    from micropp_gb300 import accuracy, workloads as wl
    cfg = dict(wl.FAST_FORM, precond=precond)
    fast = accuracy.fast_solution(N, rves["mats"], rves["et"], rves["hist"], rves["eps"], cfg)
    res = accuracy.compare(fast, rves["fp64"])
    for i, r in zip(PICK, res["rves"]):
        print(f"RVE {i}: stress {r['stress']:.2e}  ctan {r['ctan']:.2e}  fast status {r['fast_status']}  "
              f"fp64 status {r['fp64_status']}  fp64 Newton its {r['fp64_newton_its']}")
        assert r["fast_status"] == mg.STATUS_OK and r["fp64_status"] == mg.STATUS_OK, r
    assert res["stress"] <= TOL_STRESS, res
    assert res["ctan"] <= TOL_CTAN, res
