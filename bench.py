#!/usr/bin/env python
"""RVE homogenizations/s (stress + ctan) at 60^3 on one GB300: the fast form against the plain form.

Workload (default): R = 32 damage RVEs of 60^3 elements (226,981 nodes, 680,943 DOF each): 4 stiff layers
normal to z (E = 1e8, nu = 0.25, 0.1 thick), damage matrix (E = 1e7, nu = 0.25, Xt = 1e5), FE_FULL coupling
with lin_stress off.  Each RVE has a seeded macro strain target ~ U[-2.5e-2, 2.5e-2]^6.  Set-up loads every
RVE to half its target and accepts the step; a bench step is one macro iteration: every RVE is homogenized
(stress and ctan) at its target strain through the public C ABI.  Inputs are synthetic.

Two forms are measured on the same workload, one after the other (FORMS below):
  fast  -- FP32 Jacobian and multigrid-preconditioned CG inside FP64 refinement, ctan by implicit
           differentiation (headline `value`);
  plain -- the reference algorithm in FP64 (Newton + DPCG at the reference's tolerances, ctan from six
           perturbed Newton solves), the drop-in form.
`value` is device-timed throughput (CUDA events on the handles' streams); `e2e` the wall-clock throughput of
the same C-ABI calls with host strain/stress/ctan buffers; `forms` holds both forms' figures and
`fast_over_plain` their ratio.  `--impl reference` times the reference's CPU algorithm (the oracle port of
it, since the compiled reference cannot run on this host) on all host cores, on a bounded sample.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RVE homogenizations/s (stress+ctan) at 60^3, adjoint+batched vs plain, 1 GB300"
UNIT = "homogenizations/s"

# CG iterations of one stress+ctan homogenization by the reference algorithm (the plain form), averaged over
# the 32 RVEs of the default workload (n = 60, seed 2024), as measured on a GB300.  The GPU arm measures its
# own figure every run; the reference arm converts its bounded CPU sample (one Newton iteration per RVE) into
# homogenizations/s with this one.
CG_ITS_PER_HOM = {60: 1588.1}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--size", type=int, default=60, help="elements per axis")
    p.add_argument("--rves", type=int, default=32, help="RVEs per GPU")
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--cpu-sample-rves", type=int, default=0, help="RVEs in the CPU sample (default: host cores)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--forms", default="fast,plain", help="forms to measure; the first is the headline value")
    p.add_argument("--workload", default="rve60", choices=["rve60", "mixed", "precision"],
                   help="rve60: the headline (R damage RVEs of --size^3); mixed: 256 RVEs of mixed sizes, "
                        "microstructures and laws, 5 increments; precision: one J2 RVE of --precision-size^3 "
                        "along a 20-step uniaxial path, fast form against plain FP64 (neither is the headline)")
    p.add_argument("--precision-size", type=int, default=100)
    p.add_argument("--precision-steps", type=int, default=20)
    p.add_argument("--mixed-rves", type=int, default=256)
    return p.parse_args()


# ---------------------------------------------------------------------------------------------------------
# workload

def workload(n, rves, seed, rank):
    """Phase map, damage thresholds and strain targets of the RVEs of one rank.

    The reference's damage law is continuous at first loading only for Xt = 1e5, its hard-wired Ey
    (material.cpp:205-268): a larger Xt makes the stress jump by q(r)/r (5x at Xt = 2.35e5) and a smaller
    one fully damages points (NaN).  Every RVE therefore uses Xt = 1e5; the RVEs differ by their seeded
    strain targets."""
    from micropp_gb300 import workloads as wl
    xts = np.full(rves, 1e5)
    targets = wl.random_targets(rves, seed + 1000 * rank + 1, 2.5e-2)
    return wl.layers_z(n), xts, targets


# The two forms.  plain: the reference algorithm in FP64 (Newton to the reference's tolerances, ctan from six
# perturbed Newton solves).  fast: FP32 Jacobian and CG inside FP64 refinement, Newton converged to 1e-8 of the
# initial residual (average stress within 1e-7 of the converged FP64 solution), ctan by implicit
# differentiation (one 6-RHS tangent solve), both FP32 solves preconditioned by a geometric multigrid V-cycle.
# fast_jacobi (not in the default run): the same with the Jacobi preconditioner.
# `batched`: all RVEs are Gauss points of one handle, homogenized together by one micropp3_homogenize call
# (lockstep Newton and CG over the batch with per-RVE convergence masks); otherwise each RVE has its own
# handle and they are homogenized one after the other, as a macro code calls one micro point at a time.
# plain_batched (not in the default run) is the plain algorithm with batching alone.  The mixed-size workload
# was measured with fast_jacobi (--workload mixed --forms fast_jacobi,plain).
FORMS = {
    "plain": dict(batched=False, cfg=dict(precision=0, ctan_mode=0, nr_max_its=12, nr_max_tol=1e-5)),
    "fast": dict(batched=True, cfg=dict(precision=1, ctan_mode=1, nr_max_its=20, nr_max_tol=1e-30, nr_rel_tol=1e-8,
                                        precond=1)),
    "fast_jacobi": dict(batched=True, cfg=dict(precision=1, ctan_mode=1, nr_max_its=20, nr_max_tol=1e-30,
                                               nr_rel_tol=1e-8, precond=0)),
    "plain_batched": dict(batched=True, cfg=dict(precision=0, ctan_mode=0, nr_max_its=12, nr_max_tol=1e-5)),
}


def gpu_config(n, et, xt, form="plain", ngp=1):
    import micropp_gb300 as mg
    mats = [mg.material(2, 1e7, 0.25, 0, 0, xt), mg.material(0, 1e8, 0.25), mg.material(0, 1e7, 0.25)]
    return mg.config(n, ngp=ngp, mats=mats, coupling=[2] * ngp, elem_type=et, lin_stress=0, calc_ctan_lin=0,
                     **FORMS[form]["cfg"])


# ---------------------------------------------------------------------------------------------------------
# clocks sampled during the timed region

class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.rows, self.proc, self.gpu = [], None, gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------------------------------------------------
# CPU sample: one Newton iteration per RVE on the oracle (the reference algorithm), OpenMP over RVEs

def cpu_sample(n, xts, targets, cores):
    """Times one Newton iteration (1 residual, 1 assembly, 1 DPCG solve, 1 residual) of `cores` RVEs of the
    workload in parallel on the oracle, starting from u = 0 at half the target strain.  Returns (seconds, CG
    iterations summed over the sample RVEs)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as orc
    from micropp_gb300 import workloads as wl
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    et = wl.layers_z(n)
    # All RVEs share the materials, so one handle with `cores` Gauss points holds the sample and the
    # reference's own OpenMP loop over Gauss points (homogenize.cpp:72) runs them in parallel.
    mats = [orc.material(2, 1e7, 0.25, 0, 0, float(xts[0])), orc.material(0, 1e8, 0.25), orc.material(0, 1e7, 0.25)]
    cfg = orc.make_config(n, ngp=cores, mats=mats, coupling=[1] * cores, elem_type=et, lin_stress=0, nr_max_its=1,
                          nr_max_tol=1e-5, calc_ctan_lin=0)
    r = orc.OracleRVE(cfg)
    for gp in range(cores):
        r.set_strain(gp, 0.5 * targets[gp % len(targets)])
    t0 = time.perf_counter()
    r.homogenize()
    dt = time.perf_counter() - t0
    its = sum(r.newton(gp)[1] for gp in range(cores))
    r.close()
    return dt, its


def cpu_cg_its_per_homogenization(n, xts, targets):
    """CG iterations of one full stress+ctan homogenization of the first RVE of the workload, on the oracle
    (affordable only for small n)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as orc
    from micropp_gb300 import workloads as wl
    mats = [orc.material(2, 1e7, 0.25, 0, 0, float(xts[0])), orc.material(0, 1e8, 0.25), orc.material(0, 1e7, 0.25)]
    r = orc.OracleRVE(orc.make_config(n, coupling=[2], elem_type=wl.layers_z(n), mats=mats, lin_stress=0,
                                      nr_max_its=12, nr_max_tol=1e-5, calc_ctan_lin=0))
    r.set_strain(0, 0.5 * targets[0])
    r.homogenize()
    r.update_vars()
    r.set_strain(0, targets[0])
    r.homogenize()
    # cost counts the main solve's CG iterations 7 times (homogenize.cpp:269); the Newton record has the
    # main solve alone, so the perturbed solves are estimated as 6 x main.
    its = r.newton(0)[1]
    r.close()
    return 7.0 * max(its, 1)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------------------------------------

def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x, world):
    if pg is None or world == 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if pg.get_backend() == "nccl" else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    world, rank, local, pg = dist_setup(args)
    if rank != 0:
        return
    cores = host_cores()
    n = args.size
    _, xts, targets = workload(n, args.rves, args.seed, 0)
    per_hom = CG_ITS_PER_HOM.get(n)
    if per_hom is None and n <= 24:
        per_hom = cpu_cg_its_per_homogenization(n, xts, targets)
    if per_hom is None:
        print(json.dumps({"impl": "reference", "metric": METRIC, "unavailable":
                          f"no measured CG-iterations-per-homogenization figure for n={n}"}))
        return
    samples = []
    for _ in range(args.warmup + args.steps):
        dt, its = cpu_sample(n, xts, targets, cores)
        samples.append((dt, its))
    timed = samples[args.warmup:]
    tot_t = sum(s[0] for s in timed)
    tot_its = sum(s[1] for s in timed)
    value = tot_its / per_hom / tot_t
    sample = (f"{args.steps} steps; each: one Newton iteration (residual, assembly, DPCG, residual) of {cores} "
              f"RVEs of the workload in parallel (OpenMP over RVEs as the reference), "
              f"{tot_its // max(args.steps, 1)} CG its per step; scaled by {per_hom:.0f} CG its per stress+ctan "
              f"homogenization")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.rves} damage RVEs of {n}^3, 4 layers normal to z, stress+ctan",
                   "n": n, "rves": args.rves},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def load_traffic(n, family="spmv", fp32=False):
    """DRAM bytes of one RVE's launch of the kernel from a committed ncu summary (profiles/*_traffic.json)."""
    name = {("spmv", False): "spmv_fp64", ("spmv", True): "spmv_fp32", ("spmv6", True): "spmv6_fp32"}.get((family, fp32))
    p = os.path.join(ROOT, "profiles", f"{name}_traffic.json") if name else ""
    if name and os.path.exists(p):
        d = json.load(open(p))
        return d.get("bytes_per_launch_at_n", {}).get(str(n))
    return None


def measure_form(args, form, et, xts, targets, L, pg, world, local):
    """Set up R RVEs in `form`, run W warm-up and K timed steps; returns the figures of this form."""
    import ctypes

    import micropp_gb300 as mg
    n, R = args.size, args.rves
    batched = FORMS[form]["batched"]
    if batched:
        # one handle, RVE i = Gauss point i (the RVEs share materials and microstructure)
        handles = [mg.Micropp(gpu_config(n, et, float(xts[0]), form, ngp=R))]
        points = [(handles[0], i) for i in range(R)]
    else:
        handles = [mg.Micropp(gpu_config(n, et, float(xts[i]), form)) for i in range(R)]
        points = [(h, 0) for h in handles]
    # Set-up: load each RVE to half its target and accept the step; grow the target until it is nonlinear.
    tg = [t.copy() for t in targets]
    pending = list(range(R))
    for _ in range(4):
        for i in pending:
            h, gp = points[i]
            h.set_strain(gp, 0.5 * tg[i])
        for h in {id(points[i][0]): points[i][0] for i in pending}.values():
            h.homogenize()
        still = []
        for i in pending:
            h, gp = points[i]
            if not h.is_non_linear(gp):
                tg[i] *= 1.5
                still.append(i)
        if not still:
            break
        pending = still
    for h in handles:
        h.update_vars()
    nonlinear = sum(h.is_non_linear(gp) for h, gp in points)
    strain_bufs = [np.ascontiguousarray(t, dtype=np.float64) for t in tg]
    out_s = np.zeros((R, 6))
    out_c = np.zeros((R, 36))
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731

    def step(k):
        dev_ms = 0.0
        if batched:
            h = handles[0]
            for i in range(R):
                e = strain_bufs[i] * (1.0 + 1e-3 * k)
                L.micropp3_set_strain(ctypes.byref(h.h), i, dp(e))
            L.micropp3_homogenize(ctypes.byref(h.h))
            for i in range(R):
                L.micropp3_get_stress(ctypes.byref(h.h), i, dp(out_s[i]))
                L.micropp3_get_ctan(ctypes.byref(h.h), i, dp(out_c[i]))
            return L.micropp3_last_homogenize_ms(ctypes.byref(h.h))
        for i, h in enumerate(handles):
            e = strain_bufs[i] * (1.0 + 1e-3 * k)
            L.micropp3_set_strain(ctypes.byref(h.h), 0, dp(e))
            L.micropp3_homogenize(ctypes.byref(h.h))
            L.micropp3_get_stress(ctypes.byref(h.h), 0, dp(out_s[i]))
            L.micropp3_get_ctan(ctypes.byref(h.h), 0, dp(out_c[i]))
            dev_ms += L.micropp3_last_homogenize_ms(ctypes.byref(h.h))
        return dev_ms

    for k in range(args.warmup):
        step(k)
    for h in handles:
        h.set_kernel_timing(True)
    cg0 = sum(h.total_cg_its() for h in handles)
    l0 = sum(h.kernel_launches() for h in handles)
    barrier(pg)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        dev_ms = 0.0
        for k in range(args.steps):
            dev_ms += step(args.warmup + k)
        wall = time.perf_counter() - t0
    barrier(pg)
    cg_its = sum(h.total_cg_its() for h in handles) - cg0
    launches = sum(h.kernel_launches() for h in handles) - l0
    if L.micropp3_last_error():
        raise RuntimeError(L.micropp3_last_error().decode())
    status = [h.status(gp) for h, gp in points]
    newton = [h.newton(gp) for h, gp in points]  # (Newton its, CG its, converged) of the last solve
    finite = bool(np.isfinite(out_s).all() and np.isfinite(out_c).all())
    stats = {}
    for fam in ("spmv", "spmv6", "cg_update", "cg6_update", "mg", "mg6", "mg_coarse", "assembly", "residual"):
        tot = [h.kernel_stats(fam) for h in handles]
        stats[fam] = (sum(t[0] for t in tot), sum(t[1] for t in tot), sum(t[2] for t in tot))
    for h in handles:
        h.close()
    dev_s = max_over_ranks(pg, dev_ms / 1e3, world)
    wall_s = max_over_ranks(pg, wall, world)
    homs = R * args.steps * world
    return {"form": form, "batched": batched, "value": homs / dev_s, "e2e": homs / wall_s, "dev_s": dev_s,
            "wall_s": wall_s, "cg_its": cg_its, "launches": launches, "stats": stats, "clocks": clk.summary(),
            "nonlinear": nonlinear, "status": status, "newton": newton, "finite": finite, "stress": out_s.copy(),
            "ctan": out_c.copy()}


def roofline_of(res, n, peak, peak_kind):
    """Roofline record of the form's dominant linear-algebra kernel (most device time)."""
    nrow = 3 * (n + 1) ** 3
    fp32 = FORMS[res["form"]]["cfg"]["precision"] == 1
    cands = {k: res["stats"][k] for k in ("spmv", "spmv6", "mg", "mg6")}
    fam = max(cands, key=lambda k: cands[k][1])
    nk, ms, by = cands[fam]
    achieved = by / (ms / 1e3) / 1e9 if ms > 0 else None
    # algorithmic bytes of one RVE's SpMV: 81 values per row, x read once, y written once (per right-hand side);
    # the multigrid level-0 passes also read b
    if fam == "spmv6":
        name, per = "k_cg6_spmv (FP32 ELL SpMV, 6 right-hand sides)", nrow * (81 * 4 + 12 * 4)
    elif fam == "mg6":
        name, per = "k_mg_resid / k_mg_post0 (FP32 ELL SpMV of the V-cycle's fine level, 6 right-hand sides)", \
            nrow * (81 * 4 + 18 * 4)
    elif fam == "mg":
        name, per = "k_mg_resid / k_mg_post0 (FP32 ELL SpMV of the V-cycle's fine level)", nrow * (81 * 4 + 3 * 4)
    elif fp32:
        name, per = "k_cg32_spmv (FP32 ELL SpMV + p.Ap)", nrow * (81 * 4 + 2 * 4)
    else:
        name, per = "k_cg_spmv (FP64 ELL SpMV + p.Ap)", nrow * (81 * 8 + 2 * 8)
    rves_per_launch = by / nk / per if nk else None
    traffic = load_traffic(n, fam, fp32)  # DRAM bytes of one RVE's SpMV (ncu)
    if traffic is not None and rves_per_launch:
        traffic *= rves_per_launch
    return {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": by / nk if nk else None, "algorithmic_bytes_per_rve": per,
            "rves_per_launch": rves_per_launch, "launches": nk, "avg_us": 1e3 * ms / nk if nk else None}


def run_gpu(args):
    world, rank, local, pg = dist_setup(args)
    import micropp_gb300 as mg
    from micropp_gb300 import build
    build.build()
    L = mg.load()
    if world > 1:
        import torch
        torch.cuda.set_device(local)
    n, R = args.size, args.rves
    et, xts, targets = workload(n, R, args.seed, rank)
    forms = [f for f in args.forms.split(",") if f]
    results = [measure_form(args, f, et, xts, targets, L, pg, world, local) for f in forms]
    if rank != 0:
        return
    head = results[0]
    peaks = {}
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        peaks = json.load(open(pp))
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_kind = "measured" if "hbm_gbs" in peaks else "fallback"
    nrow = 3 * (n + 1) ** 3
    cpu = None
    if not args.no_cpu_baseline:
        cores = args.cpu_sample_rves or host_cores()
        plain = next((r for r in results if r["form"] == "plain"), None)
        ref_its = (plain["cg_its"] / (R * args.steps)) if plain else CG_ITS_PER_HOM.get(n)
        if ref_its:
            dt, its = cpu_sample(n, xts, targets, cores)
            cpu_val = its / ref_its / dt
            cpu = {"value": cpu_val, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": (f"one Newton iteration (residual, assembly, DPCG of {its // cores} its avg, residual) of "
                              f"{cores} RVEs of the workload at half strain, OpenMP over RVEs, {dt:.1f} s; scaled by "
                              f"{ref_its:.0f} CG its per stress+ctan homogenization of the reference algorithm "
                              f"(the plain form, measured in this run)")}

    def form_record(r):
        return {"value": r["value"], "e2e": r["e2e"], "batched": r["batched"],
                "ms_per_step": 1e3 * r["dev_s"] / args.steps,
                "cg_its_per_homogenization": r["cg_its"] / (R * args.steps),
                "cg_its_per_s": r["cg_its"] * world / r["dev_s"],
                "dof_updates_per_s": r["cg_its"] * nrow * world / r["dev_s"],
                "nonlinear_rves": r["nonlinear"], "finite": r["finite"],
                "status_counts": {str(k): r["status"].count(k) for k in sorted(set(r["status"]))},
                "newton_its_mean_max": [float(np.mean([x[0] for x in r["newton"]])), max(x[0] for x in r["newton"])],
                "newton_cg_its_mean_max": [float(np.mean([x[1] for x in r["newton"]])),
                                           max(x[1] for x in r["newton"])],
                "gpu_launches": r["launches"], "roofline": roofline_of(r, n, peak, peak_kind),
                "kernels": {k: {"launches": v[0], "ms": v[1], "avg_us": 1e3 * v[1] / v[0] if v[0] else None,
                                "algorithmic_GBps": v[2] / (v[1] / 1e3) / 1e9 if v[1] else None}
                            for k, v in r["stats"].items() if v[0]}}

    extra = {r["form"]: form_record(r) for r in results}
    ratio = None
    if len(results) > 1:
        ratio = results[0]["value"] / results[1]["value"]
        s0, s1 = results[0]["stress"], results[1]["stress"]
        extra["stress_rel_diff_between_forms"] = float(np.max(np.abs(s0 - s1)) / np.max(np.abs(s1)))
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * head["dev_s"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if FORMS[head["form"]]["cfg"]["precision"] == 1 else "f64",
        "data": "synthetic",
        "config": {"workload": f"{R} damage RVEs of {n}^3 per GPU (4 layers normal to z, Xt=1e5), "
                               f"FE_FULL stress+ctan, one homogenization per RVE per step",
                   "n": n, "rves_per_gpu": R, "form": head["form"], "forms_measured": forms,
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (221-441 MB ELL per RVE)"},
        "e2e": {"value": head["e2e"], "unit": UNIT, "h2d_bytes_per_step": R * 6 * 8, "d2h_bytes_per_step": R * 42 * 8},
        "roofline": roofline_of(head, n, peak, peak_kind),
        "cpu_baseline": cpu,
        "clocks": head["clocks"],
        "gpu_launches": head["launches"],
        "fast_over_plain": ratio,
        "forms": extra,
    }
    print(json.dumps(line))


def run_mixed(args):
    """256 RVEs of uneven size drawn from {20,30,40,50,60}^3, each a centred sphere (r = 0.2) or 4 layers normal
    to z, with an elastic, damage or J2 matrix; every RVE is taken through 5 increments to a seeded strain
    target (~U[-5e-3, 5e-3], damage ~U[-2.5e-2, 2.5e-2] so that it loads).  RVEs that share size,
    microstructure and law are Gauss points of one handle (one batch), and micropp3_homogenize_many runs the
    handles concurrently.  Value: stress + ctan homogenizations/s over the 5 increments (wall clock)."""
    import ctypes

    import micropp_gb300 as mg
    from micropp_gb300 import build
    from micropp_gb300 import workloads as wl
    build.build()
    L = mg.load()
    rng = np.random.default_rng(args.seed)
    R = args.mixed_rves
    sizes = rng.choice([20, 30, 40, 50, 60], size=R)
    micro = rng.integers(0, 2, R)
    law = rng.integers(0, 3, R)
    groups = {}
    for i in range(R):
        groups.setdefault((int(sizes[i]), int(micro[i]), int(law[i])), []).append(i)
    targets = np.zeros((R, 6))
    for i in range(R):
        targets[i] = rng.uniform(-1, 1, 6) * (2.5e-2 if law[i] == 1 else 5e-3)
    lawmat = {0: mg.material(0, 1e7, 0.25), 1: mg.material(2, 1e7, 0.25, 0, 0, 1e5),
              2: mg.material(1, 1e7, 0.3, 1e5, 1e4)}
    out = []
    for form in [f for f in args.forms.split(",") if f in FORMS and f != "plain_batched"]:
        handles, members = [], []
        for (n, mi, lw), idx in sorted(groups.items()):
            mats = [lawmat[lw], mg.material(0, 1e8, 0.25), mg.material(0, 1e7, 0.25)]
            kw = dict(FORMS[form]["cfg"])
            et = wl.layers_z(n) if mi == 1 else None
            cfg = mg.config(n, ngp=len(idx), micro_type=mg.MIC_SPHERE if mi == 0 else mg.MIC_HOMOGENEOUS,
                            geo=(0.2, 0.1, 0.1, 0.1), mats=mats, coupling=[2] * len(idx), elem_type=et, lin_stress=0,
                            calc_ctan_lin=0, **kw)
            handles.append(mg.Micropp(cfg))
            members.append(idx)
        arr = (ctypes.POINTER(mg.Handle) * len(handles))(*[ctypes.pointer(h.h) for h in handles])

        def set_inc(k):
            for h, idx in zip(handles, members):
                for gp, i in enumerate(idx):
                    h.set_strain(gp, targets[i] * k / 5.0)
        set_inc(1)
        L.micropp3_homogenize_many(arr, len(handles))  # warm-up: workspace, graphs (state not accepted)
        cg0 = sum(h.total_cg_its() for h in handles)
        with ClockSampler(0) as clk:
            t0 = time.perf_counter()
            for k in range(1, 6):
                set_inc(k)
                L.micropp3_homogenize_many(arr, len(handles))
                for h in handles:
                    h.update_vars()
            wall = time.perf_counter() - t0
        if L.micropp3_last_error():
            raise RuntimeError(L.micropp3_last_error().decode())
        cg = sum(h.total_cg_its() for h in handles) - cg0
        status = [h.status(gp) for h, idx in zip(handles, members) for gp in range(len(idx))]
        out.append({"form": form, "value": 5 * R / wall, "wall_s": wall, "cg_its": cg, "handles": len(handles),
                    "status_counts": {str(k): status.count(k) for k in sorted(set(status))}, "clocks": clk.summary()})
        for h in handles:
            h.close()
    head = out[0]
    print(json.dumps({
        "metric": "RVE homogenizations/s (stress+ctan), 256 RVEs of mixed sizes, microstructures and laws, 1 GB300",
        "value": head["value"], "unit": UNIT, "n_gpus": 1, "steps": 5, "warmup": 1,
        "ms_per_step": 1e3 * head["wall_s"] / 5, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if FORMS[head["form"]]["cfg"]["precision"] == 1 else "f64", "data": "synthetic",
        "config": {"workload": f"{R} RVEs, sizes {{20..60}}^3, sphere or layers, elastic/damage/J2, 5 increments",
                   "groups": len(groups), "form": head["form"]},
        "forms": {o["form"]: {k: v for k, v in o.items() if k != "form"} for o in out}}))


def run_precision(args):
    """One RVE of n^3 elements (default 100^3, 3,090,903 DOF): J2 matrix (E = 1e7, nu = 0.3, Sy = 1e4,
    Ka = 1e5) with 8 seeded non-overlapping elastic spheres (r = 0.12, E = 1e8, nu = 0.25), uniaxial strain
    eps_xx to 1e-2 in 20 steps (--precision-steps), every step accepted (FE_ONE_WAY: average stress per step).  The plain FP64 form
    (the reference algorithm, parity-tested against the oracle) and the fast form run the same path with tight
    tolerances (Newton 1e-10 relative, CG 1e-10); reports the fast form's stress error per step relative to the
    largest stress entry, and both forms' device time."""
    import micropp_gb300 as mg
    from micropp_gb300 import build
    from micropp_gb300 import workloads as wl
    build.build()
    n = args.precision_size
    et = wl.spheres(n, 8, 0.12, seed=args.seed)
    mats = [mg.material(1, 1e7, 0.3, 1e5, 1e4), mg.material(0, 1e8, 0.25), mg.material(0, 1e7, 0.25)]
    tight = dict(coupling=[1], elem_type=et, lin_stress=0, calc_ctan_lin=0, nr_max_its=30, nr_max_tol=1e-30,
                 nr_rel_tol=1e-10, cg_rel_tol=1e-10, cg_max_its=20000, mats=mats)
    res = {}
    for form, prec in (("plain", 0), ("fast", 1)):
        h = mg.Micropp(mg.config(n, precision=prec, **tight))
        sig, ms, its = [], 0.0, []
        ns = args.precision_steps
        with ClockSampler(0) as clk:
            for k in range(1, ns + 1):
                h.set_strain(0, [1e-2 * k / ns, 0, 0, 0, 0, 0])
                h.homogenize()
                ms += h.last_homogenize_ms()
                sig.append(h.get_stress(0))
                its.append(h.newton(0)[:2] + (h.has_converged(0),))
                h.update_vars()
                print(f"{form} step {k}: sigma_xx {sig[-1][0]:.9e} newton {its[-1]} {ms / 1e3:.1f} s", file=sys.stderr,
                      flush=True)
        res[form] = {"sigma": np.array(sig), "device_s": ms / 1e3, "newton": its, "clocks": clk.summary()}
        h.close()
    sp, sf = res["plain"]["sigma"], res["fast"]["sigma"]
    err = [float(np.max(np.abs(sf[k] - sp[k])) / np.max(np.abs(sp[k]))) for k in range(len(sp))]
    print(json.dumps({
        "workload": f"precision: one J2 RVE of {n}^3 with 8 spheres, uniaxial eps_xx to 1e-2 in "
                    f"{args.precision_steps} steps",
        "dof": 3 * (n + 1) ** 3, "stress_rel_err_per_step": err, "max_stress_rel_err": max(err),
        "plain_device_s": res["plain"]["device_s"], "fast_device_s": res["fast"]["device_s"],
        "plain_newton": res["plain"]["newton"], "fast_newton": res["fast"]["newton"],
        "sigma_xx_final": float(sp[-1][0]), "clocks": res["fast"]["clocks"]}))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "mixed":
        run_mixed(args)
    elif args.workload == "precision":
        run_precision(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
