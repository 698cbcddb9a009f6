// ell_api.cpp -- standalone Jacobi-preconditioned CG on a stencil ELL matrix in device memory.
//
// The counterpart of the reference's ell_solve_cgpd (ell.hpp:63, ell.cpp:66-122) for callers that hold a
// matrix in this library's layout: the same iteration, the same stop rule (x0 = 0, stop when ||z|| falls
// below abs_tol or rel_tol * ||z0||, or after max_its iterations), with the solver's work vectors allocated
// per call on the device.
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "device.cuh"
#include "ell_api.h"
#include "launch.h"
#include "micropp_gb300.h"

namespace mgb {

namespace {

void chk(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw CudaFailure(e, what);
}

}  // namespace

// Mesh of an nx x ny x nz node grid on the unit cube (only the node counts matter to the CG kernels).
MeshDev stencil_mesh(const int nodes[3]) {
  MeshDev m{};
  m.nx = nodes[0];
  m.ny = nodes[1];
  m.nz = nodes[2];
  m.nxny = m.nx * m.ny;
  m.nn = m.nx * m.ny * m.nz;
  m.np = (m.nn + 31) & ~31;
  m.nex = m.nx - 1;
  m.ney = m.ny - 1;
  m.nez = m.nz - 1;
  m.nelem = m.nex * m.ney * m.nez;
  return m;
}

// Runs DPCG on the listed single instance whose device view is d_inst[0]; returns the iteration count.
// `count_h` receives the number of still-running instances at each poll (host memory, pageable is fine).
int run_dpcg(const MeshDev &m, Inst *d_inst, int *d_list, unsigned int *d_count, CgState *d_cg, InstOut *d_out,
             double rel_tol, double abs_tol, int max_its, cudaStream_t s) {
  CgState c{};
  c.min_err = abs_tol;
  c.rel_err = rel_tol;
  c.max_its = max_its;
  chk(cudaMemcpyAsync(d_cg, &c, sizeof(c), cudaMemcpyHostToDevice, s), "cg state");
  chk((cudaError_t)mgb_launch_cg_setup(&m, d_inst, d_list, 1, s), "cg setup");
  const int chunk = (m.nn > 200000) ? 8 : 32;
  unsigned int count = 0;
  for (int done = 0; done <= max_its; done += chunk) {
    for (int it = 0; it < chunk; ++it) {
      if (it == chunk - 1) chk(cudaMemsetAsync(d_count, 0, sizeof(unsigned int), s), "count reset");
      chk((cudaError_t)mgb_launch_cg_spmv(&m, d_inst, d_list, 1, s), "cg spmv");
      chk((cudaError_t)mgb_launch_cg_update(&m, d_inst, d_list, 1, s), "cg update");
      chk((cudaError_t)mgb_launch_cg_pupdate(&m, d_inst, d_list, 1, d_count, s), "cg p-update");
    }
    chk(cudaMemcpyAsync(&count, d_count, sizeof(count), cudaMemcpyDeviceToHost, s), "count");
    chk(cudaStreamSynchronize(s), "sync");
    if (count == 0) break;
  }
  InstOut o{};
  chk(cudaMemcpyAsync(&o, d_out, sizeof(o), cudaMemcpyDeviceToHost, s), "out");
  chk(cudaStreamSynchronize(s), "sync");
  return o.cg_its;
}

}  // namespace mgb

using namespace mgb;

extern "C" int micropp3_ell_solve_cgpd(const int nodes[3], const double *vals, const double *b, double *x,
                                       double rel_tol, double abs_tol, int max_its, int *its, void *stream) {
  if (!nodes || !vals || !b || !x || nodes[0] < 2 || nodes[1] < 2 || nodes[2] < 2 || max_its < 0) return -1;
  const MeshDev m = stencil_mesh(nodes);
  const size_t nd = (size_t)m.nn * 3;
  const int nblocks = (int)((nd + kNodeBlock - 1) / kNodeBlock) + 8;
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<void *> bufs;
  auto alloc = [&](size_t bytes) {
    void *p = nullptr;
    chk(cudaMalloc(&p, bytes), "cudaMalloc");
    bufs.push_back(p);
    return p;
  };
  int rc = 0;
  try {
    Inst I{};
    I.vals = const_cast<double *>(vals);
    I.b = const_cast<double *>(b);
    I.du = x;
    I.r = (double *)alloc(nd * sizeof(double));
    I.z = (double *)alloc(nd * sizeof(double));
    I.p = (double *)alloc(nd * sizeof(double));
    I.Ap = (double *)alloc(nd * sizeof(double));
    I.kinv = (double *)alloc(nd * sizeof(double));
    I.red = (double *)alloc((size_t)nblocks * kRedStride * sizeof(double));
    I.ticket = (unsigned int *)alloc(sizeof(unsigned int));
    I.cg = (CgState *)alloc(sizeof(CgState));
    I.out = (InstOut *)alloc(sizeof(InstOut));
    Inst *d_inst = (Inst *)alloc(sizeof(Inst));
    int *d_list = (int *)alloc(sizeof(int));
    unsigned int *d_count = (unsigned int *)alloc(sizeof(unsigned int));
    const int zero = 0;
    chk(cudaMemsetAsync(I.ticket, 0, sizeof(unsigned int), s), "ticket");
    chk(cudaMemsetAsync(I.out, 0, sizeof(InstOut), s), "out");
    chk(cudaMemcpyAsync(d_inst, &I, sizeof(Inst), cudaMemcpyHostToDevice, s), "inst");
    chk(cudaMemcpyAsync(d_list, &zero, sizeof(int), cudaMemcpyHostToDevice, s), "list");
    const int n = run_dpcg(m, d_inst, d_list, d_count, I.cg, I.out, rel_tol, abs_tol, max_its, s);
    if (its) *its = n;
  } catch (const CudaFailure &f) {
    rc = (int)f.code;
  }
  cudaStreamSynchronize(s);
  for (void *p : bufs) cudaFree(p);
  return rc;
}
