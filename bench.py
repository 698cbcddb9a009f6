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

# Operations of one stress+ctan homogenization (FE_FULL, homogenize.cpp:188-282) by the reference algorithm,
# per RVE, averaged over the 32 RVEs of the default workload (n = 60, seed 2024): the main Newton solve and
# the six perturbed ones, each Newton iteration a residual, a Jacobian assembly and a DPCG solve.  Counted by
# the oracle's full homogenizations of those RVEs (`python bench.py --impl reference --cpu-full --rves 32`);
# the counts are a property of the algorithm and the inputs, the same on every host.
REF_OPS_PER_HOM = {60: {"residual": 15.34375, "assembly": 8.34375, "cg_setup": 8.34375, "cg_iter": 1590.8125,
                        "ave_stress": 7.0, "vars": 1.0, "homogenize": 1.0}}

OPS = ("residual", "assembly", "cg_setup", "cg_iter", "ave_stress", "vars")

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
    p.add_argument("--cpu-full", action="store_true",
                   help="with --impl reference: time full stress+ctan homogenizations of --rves RVEs on the host "
                        "cores (minutes per RVE at 60^3) and compare them with the cost model of the bounded sample")
    p.add_argument("--forms", default="fast,plain", help="forms to measure; the first is the headline value")
    p.add_argument("--accuracy-rves", type=int, default=2,
                   help="RVEs of the workload whose fast-form stress and ctan are checked, after the timed region, "
                        "against the plain FP64 form converged to CG 1e-12 / Newton 1e-11 (0: skip)")
    p.add_argument("--workload", default="rve60", choices=["rve60", "mixed", "precision"],
                   help="rve60: the headline (R damage RVEs of --size^3); mixed: 256 RVEs of mixed sizes, "
                        "microstructures and laws, 5 increments; precision: one J2 RVE of --precision-size^3 "
                        "along a 20-step uniaxial path, fast form against plain FP64 (neither is the headline)")
    p.add_argument("--precision-size", type=int, default=100)
    p.add_argument("--precision-nr-tol", type=float, default=1e-10,
                   help="Newton tolerance (relative to the initial residual) of the fast form in the precision "
                        "workload")
    p.add_argument("--precision-steps", type=int, default=20)
    p.add_argument("--mixed-rves", type=int, default=256)
    return p.parse_args()


# ---------------------------------------------------------------------------------------------------------
# workload

def workload(n, rves, seed, rank):
    """Phase map, damage thresholds and strain targets of the RVEs of one rank (workloads.damage_layers_rves)."""
    from micropp_gb300 import workloads as wl
    return wl.damage_layers_rves(n, rves, seed + 1000 * rank)


# The two forms.  plain: the reference algorithm in FP64 (Newton to the reference's tolerances, ctan from six
# perturbed Newton solves).  fast: FP32 Jacobian and CG inside FP64 refinement, Newton converged to 1e-8 of the
# initial residual (average stress within 1e-7 of the converged FP64 solution), ctan by implicit
# differentiation (one 6-RHS tangent solve), both FP32 solves preconditioned by a geometric multigrid V-cycle.
# fast_jacobi (not in the default run): the same with the Jacobi preconditioner.  fast_half: the multigrid
# whose two level-0 smoothing passes read an FP16 copy of the fine operator (MICROPP3_PRECOND_MG_HALF).
# `batched`: all RVEs are Gauss points of one handle, homogenized together by one micropp3_homogenize call
# (lockstep Newton and CG over the batch with per-RVE convergence masks); otherwise each RVE has its own
# handle and they are homogenized one after the other, as a macro code calls one micro point at a time.
# plain_batched (not in the default run) is the plain algorithm with batching alone.  The mixed-size workload
# was measured with fast_jacobi (--workload mixed --forms fast_jacobi,plain).
FORMS = {
    "plain": dict(batched=False, cfg=dict(precision=0, ctan_mode=0, nr_max_its=12, nr_max_tol=1e-5)),
    "fast": dict(batched=True, cfg=dict(precision=1, ctan_mode=1, nr_max_its=20, nr_max_tol=1e-30, nr_rel_tol=1e-8,
                                        precond=1)),  # = workloads.FAST_FORM
    "fast_jacobi": dict(batched=True, cfg=dict(precision=1, ctan_mode=1, nr_max_its=20, nr_max_tol=1e-30,
                                               nr_rel_tol=1e-8, precond=0)),
    "fast_half": dict(batched=True, cfg=dict(precision=1, ctan_mode=1, nr_max_its=20, nr_max_tol=1e-30,
                                             nr_rel_tol=1e-8, precond=2)),
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
# The reference algorithm on the host cores: the oracle, the C restatement of the reference CPU path (the
# compiled reference cannot be built on the GPU host).  A full stress+ctan homogenization at 60^3 takes
# minutes per core, so a bench step times a bounded sample of its operations, every sample RVE on its own core
# at once (OpenMP over RVEs, as the reference parallelises over macro points, homogenize.cpp:72, so the cores
# share memory bandwidth as in a full run), and a cost model composes them:
#   seconds per homogenization per core = sum over operations of (count per homogenization) x (seconds each)
# plus the per-call overhead (allocation of the ELL matrix and vectors, copies).  The counts per
# homogenization are REF_OPS_PER_HOM; `--cpu-full` times real full homogenizations against the model.

SAMPLE_NEWTON_ITS = 2   # Newton iterations per sample RVE: 3 residuals, 2 assemblies, 2 DPCG solves
SAMPLE_CG_ITS = 40      # DPCG iterations per solve in the sample (capped; the per-iteration cost is constant)


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as orc
    return orc


def _oracle_mats(orc, xt):
    return [orc.material(2, 1e7, 0.25, 0, 0, float(xt)), orc.material(0, 1e8, 0.25), orc.material(0, 1e7, 0.25)]


def cpu_sample(n, xts, targets, cores):
    """One bounded sample: `cores` RVEs of the workload as Gauss points of one oracle handle (the reference's
    OpenMP loop over points runs them on all cores), SAMPLE_NEWTON_ITS Newton iterations each from u = 0 at
    half the target strain, DPCG capped at SAMPLE_CG_ITS iterations.  Returns (wall seconds, {op: (count,
    seconds)} summed over the RVEs, with op "homogenize" the whole per-RVE call)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    orc = _oracle()
    from micropp_gb300 import workloads as wl
    cfg = orc.make_config(n, ngp=cores, mats=_oracle_mats(orc, xts[0]), coupling=[1] * cores,
                          elem_type=wl.layers_z(n), lin_stress=0, nr_max_its=SAMPLE_NEWTON_ITS, nr_max_tol=1e-30,
                          nr_rel_tol=1e-30, cg_max_its=SAMPLE_CG_ITS, calc_ctan_lin=0)
    r = orc.OracleRVE(cfg)
    for gp in range(cores):
        r.set_strain(gp, 0.5 * targets[gp % len(targets)])
    t0 = time.perf_counter()
    r.homogenize()
    dt = time.perf_counter() - t0
    per = [r.ops(gp) for gp in range(cores)]
    r.close()
    agg = {k: (sum(p[k][0] for p in per), sum(p[k][1] for p in per)) for k in per[0]}
    return dt, agg


def cpu_model(agg, per_hom):
    """Seconds of one homogenization on one core from a sample's op timings and the counts per
    homogenization; returns (seconds, seconds per op, overhead seconds per call)."""
    unit = {k: agg[k][1] / agg[k][0] for k in OPS}
    overhead = (agg["homogenize"][1] - sum(agg[k][1] for k in OPS)) / agg["homogenize"][0]
    sec = sum(per_hom[k] * unit[k] for k in OPS) + per_hom.get("homogenize", 1.0) * overhead
    return sec, unit, overhead


def cpu_full(n, xts, targets, rves, cores):
    """Full stress+ctan homogenizations (FE_FULL, homogenize.cpp:188-282) of `rves` RVEs of the workload on
    the oracle, OpenMP over RVEs.  As in the GPU bench's set-up, each RVE first takes the step to half its
    target (target grown by 1.5 until that step is nonlinear) and accepts it; that step runs FE_ONE_WAY, whose
    accepted state equals FE_FULL's, and is carried over by a restart file.  Returns (wall seconds of the
    timed homogenization, per-RVE {op: (count, seconds)}, statuses, targets used)."""
    import tempfile
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    orc = _oracle()
    from micropp_gb300 import workloads as wl
    et = wl.layers_z(n)
    common = dict(ngp=rves, mats=_oracle_mats(orc, xts[0]), elem_type=et, lin_stress=0, nr_max_its=12,
                  nr_max_tol=1e-5, calc_ctan_lin=0)
    a = orc.OracleRVE(orc.make_config(n, coupling=[1] * rves, **common))
    tg = [np.array(t, dtype=np.float64) for t in targets[:rves]]
    for _ in range(4):
        for i in range(rves):
            a.set_strain(i, 0.5 * tg[i])
        a.homogenize()
        lin = [i for i in range(rves) if not a.is_non_linear(i)]
        if not lin:
            break
        for i in lin:
            tg[i] *= 1.5
    a.update_vars()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "state.bin")
        a.write_restart(path)
        a.close()
        b = orc.OracleRVE(orc.make_config(n, coupling=[2] * rves, **common))
        b.read_restart(path)
    for i in range(rves):
        b.set_strain(i, tg[i])
    b.reset_ops()
    t0 = time.perf_counter()
    b.homogenize()
    wall = time.perf_counter() - t0
    per = [b.ops(i) for i in range(rves)]
    conv = [b.has_converged(i) for i in range(rves)]
    b.close()
    return wall, per, conv, tg


def ops_per_hom(n, xts, targets, cores):
    """Counts per homogenization of the workload at size n: the committed counts, or for small grids
    (n <= 24, seconds of CPU work) counted here by full homogenizations of up to 4 RVEs; None otherwise."""
    if n in REF_OPS_PER_HOM:
        return REF_OPS_PER_HOM[n]
    if n > 24:
        return None
    k = max(1, min(4, cores, len(targets)))
    _, per, _, _ = cpu_full(n, xts, targets, k, cores)
    return {op: float(np.mean([p[op][0] for p in per])) for op in per[0]}


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
    cores = args.cpu_sample_rves or host_cores()
    n = args.size
    _, xts, targets = workload(n, args.rves, args.seed, 0)
    if args.cpu_full:
        run_cpu_full(args, n, xts, targets, cores)
        return
    per_hom = ops_per_hom(n, xts, targets, cores)
    if per_hom is None:
        print(json.dumps({"impl": "reference", "metric": METRIC, "unavailable":
                          f"no counted operations per homogenization for n={n} (bench.py --cpu-full counts them)"}))
        return
    samples = [cpu_sample(n, xts, targets, cores) for _ in range(args.warmup + args.steps)]
    timed = samples[args.warmup:]
    agg = {k: (sum(t[1][k][0] for t in timed), sum(t[1][k][1] for t in timed)) for k in timed[0][1]}
    sec, unit, overhead = cpu_model(agg, per_hom)
    value = cores / sec
    tot_t = sum(t[0] for t in timed)
    sample = (f"{args.steps} steps; each: {cores} RVEs of the workload on {cores} cores at once (OpenMP over RVEs "
              f"as the reference), {SAMPLE_NEWTON_ITS} Newton iterations from u = 0 at half strain with DPCG capped "
              f"at {SAMPLE_CG_ITS} its, every operation timed; composed with the counts of one stress+ctan "
              f"homogenization ({per_hom['residual']:.1f} residuals, {per_hom['assembly']:.1f} assemblies, "
              f"{per_hom['cg_iter']:.0f} DPCG its; counted by full oracle runs) into {sec:.1f} s per homogenization "
              f"per core")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.rves} damage RVEs of {n}^3, 4 layers normal to z, stress+ctan",
                   "n": n, "rves": args.rves},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "cpu_model": {"seconds_per_homogenization_per_core": sec, "seconds_per_op": unit,
                      "overhead_s_per_call": overhead, "ops_per_homogenization": per_hom},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_cpu_full(args, n, xts, targets, cores):
    """--cpu-full: real full homogenizations against the cost model on this host."""
    rves = args.rves
    wall, per, conv, _ = cpu_full(n, xts, targets, rves, cores)
    counts = {k: [p[k][0] for p in per] for k in per[0]}
    secs = [p["homogenize"][1] for p in per]
    mean = {k: float(np.mean(v)) for k, v in counts.items()}
    samples = [cpu_sample(n, xts, targets, min(cores, rves)) for _ in range(2)]
    agg = {k: (sum(t[1][k][0] for t in samples), sum(t[1][k][1] for t in samples)) for k in samples[0][1]}
    model_sec, unit, overhead = cpu_model(agg, mean)
    rounds = -(-rves // cores)
    print(json.dumps({
        "impl": "reference", "mode": "cpu-full", "n": n, "rves": rves, "cores": cores, "wall_s": wall,
        "measured_homogenizations_per_s": rves / wall,
        "model_homogenizations_per_s": min(cores, rves) / model_sec,
        "model_over_measured": (min(cores, rves) / model_sec) / (rves / wall) if rounds == 1 else None,
        "per_rve_seconds_mean_max": [float(np.mean(secs)), float(np.max(secs))],
        "model_seconds_per_homogenization": model_sec, "seconds_per_op_model": unit,
        "seconds_per_op_full": {k: sum(p[k][1] for p in per) / max(sum(p[k][0] for p in per), 1) for k in OPS},
        "ops_per_homogenization_mean": mean, "ops_per_rve": counts, "converged": conv}))


def load_traffic(n, family="spmv", fp32=False):
    """DRAM bytes of one RVE's launch of the kernel from a committed ncu summary (profiles/*_traffic.json)."""
    name = {("spmv", False): "spmv_fp64", ("spmv", True): "spmv_fp32", ("spmv6", True): "spmv6_fp32",
            ("mg6", True): "mg6_fp32", ("mg", True): "mg_fp32", ("mg6_half", True): "mg6_fp16",
            ("mg_half", True): "mg_fp16"}.get((family, fp32))
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
    last_s, last_c = out_s.copy(), out_c.copy()  # results of the last timed step
    stats = {}
    for fam in ("spmv", "spmv6", "cg_update", "cg6_update", "mg", "mg6", "mg_coarse", "assembly", "mg_rap", "residual",
                "tangent"):
        tot = [h.kernel_stats(fam) for h in handles]
        stats[fam] = (sum(t[0] for t in tot), sum(t[1] for t in tot), sum(t[2] for t in tot))
    status = [h.status(gp) for h, gp in points]
    newton = [h.newton(gp) for h, gp in points]  # (Newton its, CG its, converged) of the last solve
    finite = bool(np.isfinite(out_s).all() and np.isfinite(out_c).all())
    graphs = None
    if batched:
        # the same K steps again with the per-kernel timers off, so that the CG iteration chunks replay as CUDA
        # graphs (the timers need the kernels launched one by one); not the headline
        for h in handles:
            h.set_kernel_timing(False)
            h.set_cuda_graphs(True)
        step(args.warmup + args.steps)  # captures the graphs of this batch size
        barrier(pg)
        g_ms = 0.0
        for k in range(args.steps):
            g_ms += step(args.warmup + args.steps + 1 + k)
        barrier(pg)
        g_s = max_over_ranks(pg, g_ms / 1e3, world)
        graphs = {"value": R * args.steps * world / g_s, "unit": UNIT, "ms_per_step": 1e3 * g_s / args.steps,
                  "what": "the same steps with kernel timers off: CG iteration chunks replayed as CUDA graphs"}
    if L.micropp3_last_error():
        raise RuntimeError(L.micropp3_last_error().decode())
    for h in handles:
        h.close()
    dev_s = max_over_ranks(pg, dev_ms / 1e3, world)
    wall_s = max_over_ranks(pg, wall, world)
    homs = R * args.steps * world
    return {"form": form, "batched": batched, "value": homs / dev_s, "e2e": homs / wall_s, "dev_s": dev_s,
            "wall_s": wall_s, "cg_its": cg_its, "launches": launches, "stats": stats, "clocks": clk.summary(),
            "nonlinear": nonlinear, "status": status, "newton": newton, "finite": finite, "stress": last_s,
            "ctan": last_c, "graphs": graphs}


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
    elif fam in ("mg6", "mg"):
        # the V-cycle's two level-0 passes; MICROPP3_PRECOND_MG_HALF reads the FP16 copy of the operator
        half = FORMS[res["form"]]["cfg"].get("precond") == 2
        vb, kind = (2, "FP16") if half else (4, "FP32")
        nr = 6 if fam == "mg6" else 1
        name = (f"k_mg_resid{'6' if nr == 6 else ''} / k_mg_post0{'6' if nr == 6 else ''} ({kind} ELL SpMV of the "
                f"V-cycle's fine level, {nr} right-hand side{'s' if nr == 6 else ''})")
        per = nrow * (81 * vb + 3 * nr * 4)
        fam_key = fam + ("_half" if half else "")
    elif fp32:
        name, per = "k_cg32_spmv (FP32 ELL SpMV + p.Ap)", nrow * (81 * 4 + 2 * 4)
    else:
        name, per = "k_cg_spmv (FP64 ELL SpMV + p.Ap)", nrow * (81 * 8 + 2 * 8)
    rves_per_launch = by / nk / per if nk else None
    traffic = load_traffic(n, fam_key if fam in ("mg6", "mg") else fam, fp32)  # DRAM bytes per RVE launch (ncu)
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
    from micropp_gb300 import workloads as wl
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
    cores = args.cpu_sample_rves or host_cores()
    per_hom = None if args.no_cpu_baseline else ops_per_hom(n, xts, targets, cores)
    if per_hom is not None:
        dt, agg = cpu_sample(n, xts, targets, cores)
        sec, _, _ = cpu_model(agg, per_hom)
        cpu = {"value": cores / sec, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": (f"{cores} RVEs of the workload on {cores} cores at once (OpenMP over RVEs), "
                          f"{SAMPLE_NEWTON_ITS} Newton iterations from u = 0 at half strain, DPCG capped at "
                          f"{SAMPLE_CG_ITS} its, {dt:.1f} s, every operation timed; composed with the operation "
                          f"counts of one stress+ctan homogenization (full oracle runs) into {sec:.1f} s per "
                          f"homogenization per core")}

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
                "timers_off_graphs_on": r["graphs"],
                "kernels": {k: {"launches": v[0], "ms": v[1], "avg_us": 1e3 * v[1] / v[0] if v[0] else None,
                                "algorithmic_GBps": v[2] / (v[1] / 1e3) / 1e9 if v[1] else None}
                            for k, v in r["stats"].items() if v[0]}}

    extra = {r["form"]: form_record(r) for r in results}
    fast_err = None
    head_cfg = FORMS[head["form"]]["cfg"]
    if args.accuracy_rves > 0 and head_cfg["precision"] == 1:
        from micropp_gb300 import accuracy
        k = min(args.accuracy_rves, R)
        mats = wl.damage_layers_materials(mg, float(xts[0]))
        fast_err = accuracy.fast_vs_fp64(n, mats, et, [0.5 * targets[i] for i in range(k)],
                                         [targets[i] for i in range(k)], head_cfg)
        fast_err["rves_checked"] = k
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
        "fast_error_vs_fp64": fast_err,
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
    """The precision configuration: one RVE of n^3 elements (default 100^3, 3,090,903 DOF), J2 matrix
    (E = 1e7, nu = 0.3, Sy = 1e4, Ka = 1e5) with 8 seeded non-overlapping elastic spheres (r = 0.12,
    E = 1e8, nu = 0.25), uniaxial strain eps_xx to 1e-2 in 20 steps (--precision-steps), every step accepted.

    fast:  the headline's fast form (FP32 Jacobian and multigrid-preconditioned CG inside FP64 refinement,
           implicit ctan) with Newton to --precision-nr-tol (1e-10), FE_FULL: stress and ctan at every step.
    FP64:  the library's FP64 path solver (micropp3_path_forward: FP64 Newton with the exact consistent
           tangent, BiCGSTAB corrections, Newton 1e-11 / linear solves 1e-12): the stress of every step.  The
           reference's own FP64 Newton (forward-difference tangent, CG) does not converge on this path.
    ctan:  at the last step against central differences (h = 1e-7) of the stress converged to Newton 1e-12,
           13 FE_ONE_WAY points of the mixed form along the same path (every converged FP64 residual has the
           same solution whatever solves its corrections).
    Reports the fast form's stress error per step and its ctan error at the last step, relative to the
    largest entry, and the device time of each run."""
    import micropp_gb300 as mg
    from micropp_gb300 import accuracy, build
    from micropp_gb300 import workloads as wl
    build.build()
    n, ns = args.precision_size, args.precision_steps
    et = wl.spheres(n, 8, 0.12, seed=args.seed)
    mats = [mg.material(1, 1e7, 0.3, 1e5, 1e4), mg.material(0, 1e8, 0.25), mg.material(0, 1e7, 0.25)]
    path = np.array([[1e-2 * k / ns, 0, 0, 0, 0, 0] for k in range(1, ns + 1)])
    common = dict(elem_type=et, lin_stress=0, calc_ctan_lin=0, mats=mats)

    def log(msg):
        print(msg, file=sys.stderr, flush=True)

    # fast form, stress + ctan every step
    h = mg.Micropp(mg.config(n, coupling=[mg.FE_FULL], **common,
                             **dict(wl.FAST_FORM, nr_rel_tol=args.precision_nr_tol)))
    sig_f, ctan_f, ms_f, newton_f = [], [], 0.0, []
    with ClockSampler(0) as clk:
        for k in range(ns):
            h.set_strain(0, path[k])
            h.homogenize()
            ms_f += h.last_homogenize_ms()
            sig_f.append(h.get_stress(0))
            ctan_f.append(h.get_ctan(0))
            newton_f.append(h.newton(0)[:2] + (h.status(0),))
            h.update_vars()
            log(f"fast step {k + 1}: sigma_xx {sig_f[-1][0]:.9e} newton {newton_f[-1]} {ms_f / 1e3:.1f} s")
    h.close()
    # FP64 path solver
    h = mg.Micropp(mg.config(n, **common, **{k: v for k, v in accuracy.TIGHT.items()
                                            if k not in ("calc_ctan_lin", "lin_stress")}))
    params = np.array([[m.E, m.nu, m.Xt, m.Sy, m.Ka] for m in mats])
    t0 = time.perf_counter()
    sig_64, rc = h.path_forward(path, params, checkpoint_every=ns)
    t_64 = time.perf_counter() - t0
    newton_64 = [h.path_newton(k) for k in range(ns)]
    h.close()
    log(f"FP64 path: {t_64:.1f} s, rc {rc}")
    # central-difference ctan at the last step
    tight = dict(wl.FAST_FORM, nr_rel_tol=1e-12, nr_max_its=40)
    h = mg.Micropp(mg.config(n, ngp=13, coupling=[mg.FE_ONE_WAY] * 13, **common, **tight))
    t0 = time.perf_counter()
    for k in range(ns):
        for gp in range(13):
            e = path[k].copy()
            if k == ns - 1 and gp > 0:
                e[(gp - 1) // 2] += accuracy.H if gp % 2 else -accuracy.H
            h.set_strain(gp, e)
        h.homogenize()
        if k < ns - 1:
            h.update_vars()
    ctan_fd = np.zeros((6, 6))
    for j in range(6):
        ctan_fd[:, j] = (h.get_stress(1 + 2 * j) - h.get_stress(2 + 2 * j)) / (2 * accuracy.H)
    fd_status = max(h.status(gp) for gp in range(13))
    t_fd = time.perf_counter() - t0
    h.close()
    err = [accuracy.rel_err(sig_f[k], sig_64[k]) for k in range(ns)]
    print(json.dumps({
        "workload": f"precision: one J2 RVE of {n}^3 with 8 spheres, uniaxial eps_xx to 1e-2 in {ns} steps",
        "dof": 3 * (n + 1) ** 3, "fast_nr_rel_tol": args.precision_nr_tol,
        "fast_stress_rel_err_per_step": err, "fast_stress_max_rel_err": max(err),
        "fast_ctan_rel_err_last_step": accuracy.rel_err(ctan_f[-1], ctan_fd),
        "fast_device_s": ms_f / 1e3, "fast_newton_cg_status": newton_f, "fp64_path_s": t_64, "fp64_path_rc": rc,
        "fp64_path_newton": newton_64, "ctan_fd_s": t_fd, "ctan_fd_status": fd_status,
        "sigma_xx_final": float(sig_64[-1][0]), "clocks": clk.summary()}))


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
