"""Build recipe of the GB300 library: micropp_gb300/libmicropp_gb300.so (in-tree).

CUDA sources are compiled by nvcc for sm_103a only; host C++ by g++; the whole library links the CUDA
runtime statically, so it depends on nothing but the NVIDIA kernel driver (libcuda).  Translation units
compile in parallel and a unit is rebuilt only when it or a header changed.  Run as ``python -m micropp_gb300.build`` or through
``__graft_entry__.build()``.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmicropp_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the GB300 library needs the CUDA toolkit to build")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.hpp")) + \
        glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INC, "*.h*"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _jobs(nvcc):
    inc = ["-I", INC, "-I", CSRC]
    jobs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
               *inc, "-c", src, "-o", obj]
        jobs.append((src, obj, cmd))
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        # Host FP64 formulas are rounded like the reference's: no fused multiply-add contraction.
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
               "-Wno-unused-parameter", *inc, "-I", cuda_inc, "-c", src, "-o", obj]
        jobs.append((src, obj, cmd))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.c"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-ffp-contract=off", "-Wall", *inc, "-c", src, "-o", obj]
        jobs.append((src, obj, cmd))
    return jobs


def build(force=False, verbose=False):
    """Compile (incrementally) and link the library; returns its path."""
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    hdrs = _headers()
    jobs = [j for j in _jobs(nvcc) if force or _stale(j[1], [j[0], *hdrs])]
    logs = []

    def run(job):
        src, obj, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r

    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for src, r in ex.map(run, jobs):
            logs.append((src, r.stdout + r.stderr))
            if r.returncode != 0:
                raise RuntimeError(f"compiling {src} failed:\n{r.stdout}\n{r.stderr}")
    objs = [j[1] for j in _jobs(nvcc)]
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking {LIB} failed:\n{r.stdout}\n{r.stderr}")
    with open(os.path.join(OBJ, "ptxas.log"), "a") as f:
        for src, text in logs:
            if text.strip():
                f.write(f"== {src}\n{text}\n")
    if verbose:
        for src, text in logs:
            if "ptxas" in text:
                print(f"== {os.path.basename(src)}\n{text}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
