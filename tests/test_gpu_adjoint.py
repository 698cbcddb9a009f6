"""Reverse-mode gradients of a load path (micropp3_path_forward / micropp3_path_vjp).

L = sum_n |sigma_n - sigma*_n|^2 over a cyclic macro strain path, sigma* from the same solver at parameters
+5%.  The adjoint gradients with respect to the per-phase parameters (E, nu, Xt, Sy, Ka) and to the macro
strains are checked against central differences of L, the checkpoint interval must not change them, a
one-step path from the undeformed state must give ctan^T g with the plain form's ctan, and a
torch.autograd.Function around the two entries (the gradient-check harness) must reproduce them.
"""
import numpy as np
import pytest

import micropp_gb300 as mg
from micropp_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL_GRAD = 2e-4  # relative to the largest gradient entry: the central differences carry Newton's 1e-12 noise


def _handle(kind, n):
    tight = dict(lin_stress=0, calc_ctan_lin=0, nr_max_its=30, nr_max_tol=1e-30, nr_rel_tol=1e-13,
                 cg_rel_tol=1e-13, cg_max_its=5000)
    if kind == "j2":
        mats = [mg.material(1, 1e7, 0.3, 1e5, 1e4), mg.material(0, 1e8, 0.25), mg.material(0, 1e7, 0.25)]
        return mg.Micropp(mg.config(n, micro_type=mg.MIC_SPHERE, geo=(0.2, 0.1, 0.1, 0.1), mats=mats,
                                    coupling=[mg.FE_FULL], **tight))
    mats = [mg.material(2, 1e7, 0.25, 0, 0, 1e5), mg.material(0, 1e8, 0.25), mg.material(0, 1e7, 0.25)]
    return mg.Micropp(mg.config(n, mats=mats, coupling=[mg.FE_FULL], elem_type=wl.layers_z(n), **tight))


def _params(kind):
    if kind == "j2":
        return np.array([[1e7, 0.3, 0.0, 1e4, 1e5], [1e8, 0.25, 0.0, 0.0, 0.0], [1e7, 0.25, 0.0, 0.0, 0.0]])
    return np.array([[1e7, 0.25, 1e5, 0.0, 0.0], [1e8, 0.25, 0.0, 0.0, 0.0], [1e7, 0.25, 0.0, 0.0, 0.0]])


def _path(kind, nsteps):
    k = np.arange(1, nsteps + 1)
    if kind == "j2":  # cyclic, amplitude 8e-3, mixed normal and shear
        a = 8e-3 * np.sin(2 * np.pi * k / nsteps)
        d = np.array([1.0, -0.3, -0.3, 0.5, 0.0, 0.2])
    else:  # monotone loading into the damaged range
        a = 2.5e-2 * k / nsteps
        d = np.array([1.0, -0.2, 0.1, 0.3, 0.0, 0.0])
    return np.outer(a, d)


def _loss(h, strains, params, target, every=2):
    sig, rc = h.path_forward(strains, params, every)
    assert rc == 0
    return float(np.sum((sig - target) ** 2)), sig


# (phase, parameter index) pairs each law uses: E, nu of every phase in use; Sy, Ka of J2; Xt of damage
USED = {"j2": [(0, 0), (0, 1), (0, 3), (0, 4), (1, 0), (1, 1)],
        "damage": [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1)]}


@pytest.mark.parametrize("kind,n,nsteps,every", [("j2", 6, 6, 2), ("damage", 6, 4, 3)])
def test_parameter_and_strain_gradients_match_central_differences(gpu_lib, kind, n, nsteps, every):
    h = _handle(kind, n)
    p0, eps = _params(kind), _path(kind, nsteps)
    target, rc = h.path_forward(eps, p0 * 1.05, every)
    assert rc == 0
    L0, sig = _loss(h, eps, p0, target, every)
    assert L0 > 0
    gp, gs, rc = h.path_vjp(2 * (sig - target))
    assert rc == 0
    fd = np.zeros_like(gp)
    for ph, q in USED[kind]:
        step = 1e-5 * p0[ph, q]
        pp, pm = p0.copy(), p0.copy()
        pp[ph, q] += step
        pm[ph, q] -= step
        fd[ph, q] = (_loss(h, eps, pp, target, every)[0] - _loss(h, eps, pm, target, every)[0]) / (2 * step)
    # compare relative to each parameter's scale (dL/dlog p), against the largest of them
    scale = np.abs(p0)
    ref = np.max(np.abs(fd * scale))
    assert ref > 0
    for ph, q in USED[kind]:
        assert abs(gp[ph, q] - fd[ph, q]) * scale[ph, q] <= TOL_GRAD * ref, (kind, ph, q, gp[ph, q], fd[ph, q])
    # strain gradients of two steps
    for nstep, comp in [(nsteps - 1, 0), (nsteps // 2, 3)]:
        step = 1e-6
        ep, em = eps.copy(), eps.copy()
        ep[nstep, comp] += step
        em[nstep, comp] -= step
        fds = (_loss(h, ep, p0, target, every)[0] - _loss(h, em, p0, target, every)[0]) / (2 * step)
        assert abs(gs[nstep, comp] - fds) <= TOL_GRAD * max(np.max(np.abs(gs)), 1e-300), (nstep, comp, gs[nstep, comp], fds)
    h.close()


def test_checkpoint_interval_does_not_change_gradients(gpu_lib):
    h = _handle("j2", 5)
    p0, eps = _params("j2"), _path("j2", 6)
    target = h.path_forward(eps, p0 * 1.05, 6)[0]
    grads = []
    for every in (1, 2, 4, 6):
        sig, rc = h.path_forward(eps, p0, every)
        assert rc == 0
        gp, gs, rc = h.path_vjp(2 * (sig - target))
        assert rc == 0
        grads.append((gp, gs))
    for gp, gs in grads[1:]:
        np.testing.assert_allclose(gp, grads[0][0], rtol=1e-12, atol=0)
        np.testing.assert_allclose(gs, grads[0][1], rtol=1e-12, atol=0)
    h.close()


def test_one_step_strain_gradient_is_ctan_transpose_g(gpu_lib):
    """From the undeformed state, dL/deps of a one-step path with L = g . sigma is ctan^T g; ctan from the plain
    form's six perturbed solves (forward differences with step 1e-8: agreement to their own noise)."""
    h = _handle("j2", 6)
    p0 = _params("j2")
    eps = np.array([[6e-3, -1e-3, 0.0, 4e-3, 0.0, 1e-3]])
    g = np.array([[1.0, -0.5, 0.25, 2.0, 0.0, -1.0]])
    sig, rc = h.path_forward(eps, p0, 1)
    assert rc == 0
    _, gs, rc = h.path_vjp(g)
    assert rc == 0
    h.set_strain(0, eps[0])
    h.homogenize()
    assert h.is_non_linear(0)
    np.testing.assert_allclose(h.get_stress(0), sig[0], rtol=0, atol=1e-9 * np.max(np.abs(sig)))
    ctan = h.get_ctan(0).reshape(6, 6)
    want = ctan.T @ g[0]
    assert np.max(np.abs(gs[0] - want)) <= 1e-5 * np.max(np.abs(want)), (gs[0], want)
    h.close()


def test_torch_autograd_harness(gpu_lib):
    """The gradient-check harness: a torch.autograd.Function over the two C-ABI entries."""
    torch = pytest.importorskip("torch")
    h = _handle("j2", 5)
    p0, eps = _params("j2"), _path("j2", 4)
    target = h.path_forward(eps, p0 * 1.05, 2)[0]

    class RVEPath(torch.autograd.Function):
        @staticmethod
        def forward(ctx, params, strains):
            sig, rc = h.path_forward(strains.detach().cpu().numpy(), params.detach().cpu().numpy(), 2)
            assert rc == 0
            return torch.from_numpy(sig)

        @staticmethod
        def backward(ctx, gsig):
            gp, gs, rc = h.path_vjp(gsig.detach().cpu().numpy())
            assert rc == 0
            return torch.from_numpy(gp), torch.from_numpy(gs)

    params = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    strains = torch.tensor(eps, dtype=torch.float64, requires_grad=True)
    sig = RVEPath.apply(params, strains)
    loss = ((sig - torch.from_numpy(target)) ** 2).sum()
    loss.backward()
    # the same gradient through the C ABI directly
    s2, _ = h.path_forward(eps, p0, 2)
    gp, gs, _ = h.path_vjp(2 * (s2 - target))
    np.testing.assert_allclose(params.grad.numpy(), gp, rtol=1e-12, atol=0)
    np.testing.assert_allclose(strains.grad.numpy(), gs, rtol=1e-12, atol=0)
    # and a directional central difference of the torch loss
    d = torch.zeros_like(params)
    d[0, 0], d[0, 3] = 1e7 * 1e-5, 1e4 * 1e-5

    def L(p):
        return float(((RVEPath.apply(p, strains.detach()) - torch.from_numpy(target)) ** 2).sum())
    fd = (L(params.detach() + d) - L(params.detach() - d)) / 2
    ad = float((params.grad * d).sum())
    assert abs(ad - fd) <= 1e-4 * abs(fd), (ad, fd)
    h.close()


def test_j2_path_50cubed_20_steps_checkpoint_5(gpu_lib, capsys):
    """The differentiation workload at full size: one 50^3 J2 RVE with 8 seeded spheres (r = 0.12, elastic),
    a 20-step seeded cyclic strain path of amplitude 8e-3, checkpoints every 5 steps; the adjoint gradient of
    L with respect to the matrix's E and Sy and the spheres' E against central differences (measured once for
    all four (E, nu, yield, hardening): agreement within 2e-9 of the largest |dL/dlog theta|)."""
    import time
    n = 50
    mats = [mg.material(1, 1e7, 0.3, 1e5, 1e4), mg.material(0, 1e8, 0.25), mg.material(0, 1e7, 0.25)]
    h = mg.Micropp(mg.config(n, mats=mats, coupling=[mg.FE_FULL], elem_type=wl.spheres(n, 8, 0.12, seed=5),
                             lin_stress=0, calc_ctan_lin=0, nr_max_its=20, nr_max_tol=1e-30, nr_rel_tol=1e-10,
                             cg_rel_tol=1e-10, cg_max_its=5000))
    rng = np.random.default_rng(11)
    d = rng.uniform(-1, 1, 6)
    d /= np.max(np.abs(d))
    k = np.arange(1, 21)
    eps = np.outer(8e-3 * np.sin(2 * np.pi * k / 10), d)  # two load cycles
    p0 = np.array([[1e7, 0.3, 0.0, 1e4, 1e5], [1e8, 0.25, 0.0, 0.0, 0.0], [1e7, 0.25, 0.0, 0.0, 0.0]])
    target, rc = h.path_forward(eps, p0 * 1.05, 5)
    assert rc == 0, [h.path_newton(k) for k in range(20)]
    t0 = time.perf_counter()
    sig, rc = h.path_forward(eps, p0, 5)
    t1 = time.perf_counter()
    gp, gs, rc2 = h.path_vjp(2 * (sig - target))
    t2 = time.perf_counter()
    assert rc == 0 and rc2 == 0
    checks = [(0, 0), (0, 3), (1, 0)]
    fd = {}
    for ph, q in checks:
        step = 1e-5 * p0[ph, q]
        pp, pm = p0.copy(), p0.copy()
        pp[ph, q] += step
        pm[ph, q] -= step
        lp = np.sum((h.path_forward(eps, pp, 5)[0] - target) ** 2)
        lm = np.sum((h.path_forward(eps, pm, 5)[0] - target) ** 2)
        fd[(ph, q)] = (lp - lm) / (2 * step)
    ref = max(abs(fd[c]) * p0[c] for c in checks)
    with capsys.disabled():
        print(f"\n50^3 J2, 20 steps: forward {t1 - t0:.2f} s, reverse (2 recomputed segments per checkpoint) "
              f"{t2 - t1:.2f} s")
        for c in checks:
            print(f"  dL/dtheta{c}: adjoint {gp[c]:.9e}  central difference {fd[c]:.9e}  "
                  f"rel. to max |dL/dlog theta| {abs(gp[c] - fd[c]) * p0[c] / ref:.2e}")
    for c in checks:
        assert abs(gp[c] - fd[c]) * p0[c] <= TOL_GRAD * ref, (c, gp[c], fd[c])
    h.close()
