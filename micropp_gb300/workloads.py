"""Seeded synthetic RVE inputs of the benchmark and parity cases.

The reference's micro types do not include the two microstructures of these workloads, so they are given as
element phase maps (``micropp3_config.elem_type``), the way a caller of the library would:

* ``layers_z(n)``   -- 4 parallel stiff layers normal to z, 0.1 thick, centred at z = .125, .375, .625,
  .875 (phase 1 where |z_centroid - c| < 0.05, else 0);
* ``spheres(n, k, r, seed)`` -- k non-overlapping spheres of radius r with seeded uniform centres
  (rejection sampling, fully inside the cube), phase 1 inside.

Damage-law parameters: the reference damage law has a single threshold parameter Xt (material.cpp:227-268)
and a softening table hard-wired to Ey = 1e5.  With Xt < 1e5 it fully damages Gauss points (the reference
itself returns NaN stresses); with Xt > 1e5 the damaged stress jumps by q(r)/r at first loading.  The
benchmark's damage matrix therefore uses Xt = 1e5, where the law is continuous.
"""
import numpy as np


def centroids(n):
    c = (np.arange(n) + 0.5) / n
    return c


def layers_z(n, centres=(0.125, 0.375, 0.625, 0.875), half_width=0.05):
    """Phase map (nelem,) int32 in glo_elem order (ez slowest)."""
    zc = centroids(n)
    lay = np.zeros(n, dtype=bool)
    for c in centres:
        lay |= np.abs(zc - c) < half_width
    et = np.zeros((n, n, n), dtype=np.int32)
    et[lay, :, :] = 1
    return et.reshape(-1)


def sphere_centres(k, r, seed):
    rng = np.random.default_rng(seed)
    out = []
    tries = 0
    while len(out) < k:
        tries += 1
        if tries > 100000:
            raise RuntimeError("could not place non-overlapping spheres")
        c = rng.uniform(r, 1 - r, size=3)
        if all(np.linalg.norm(c - o) >= 2 * r for o in out):
            out.append(c)
    return np.array(out)


def spheres(n, k=8, r=0.12, seed=0):
    cs = sphere_centres(k, r, seed)
    c = centroids(n)
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    inside = np.zeros_like(x, dtype=bool)
    for cc in cs:
        inside |= (x - cc[0]) ** 2 + (y - cc[1]) ** 2 + (z - cc[2]) ** 2 < r * r
    return inside.astype(np.int32).reshape(-1)


def damage_thresholds(count, seed, lo=1e5, hi=3e5):
    return np.random.default_rng(seed).uniform(lo, hi, size=count)


def monotone_path(target, steps):
    """Strain at steps 1..steps toward `target` (6,)."""
    target = np.asarray(target, dtype=np.float64)
    return [target * (s / steps) for s in range(1, steps + 1)]


def random_targets(count, seed, amp):
    return np.random.default_rng(seed).uniform(-amp, amp, size=(count, 6))


def damage_layers_rves(n, rves, seed):
    """The headline workload's RVEs: phase map (4 layers normal to z), damage thresholds and seeded strain
    targets ~ U[-2.5e-2, 2.5e-2]^6.

    The reference's damage law is continuous at first loading only for Xt = 1e5, its hard-wired Ey
    (material.cpp:205-268): a larger Xt makes the stress jump by q(r)/r (5x at Xt = 2.35e5) and a smaller
    one fully damages points (NaN).  Every RVE therefore uses Xt = 1e5; the RVEs differ by their seeded
    strain targets."""
    xts = np.full(rves, 1e5)
    targets = random_targets(rves, seed + 1, 2.5e-2)
    return layers_z(n), xts, targets


def damage_layers_materials(mg, xt=1e5):
    """Materials of the headline workload: damage matrix (E = 1e7, nu = 0.25, Xt), stiff elastic layers
    (E = 1e8, nu = 0.25); `mg` is the micropp_gb300 module."""
    return [mg.material(2, 1e7, 0.25, 0, 0, xt), mg.material(0, 1e8, 0.25), mg.material(0, 1e7, 0.25)]


# Options of the fast form of the headline: FP32 Jacobian and multigrid-preconditioned CG inside FP64
# refinement, Newton to 1e-8 of its initial residual, ctan by implicit differentiation.
FAST_FORM = dict(precision=1, ctan_mode=1, nr_max_its=20, nr_max_tol=1e-30, nr_rel_tol=1e-8, precond=1)
