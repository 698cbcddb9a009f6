// cg_kernels.cu -- Jacobi-preconditioned CG on the stencil ELL matrix (sm_103a, FP64).
//
// The iteration is the reference's ell_solve_cgpd (ell.cpp:66-122) step for step:
//   k = 1/diag(A); x = 0; r = b; z = k r; p = z; rz = r.z; pnorm0 = ||z||
//   while its < max_its and not (pnorm < min_err or pnorm < pnorm0*rel_err):
//     Ap = A p; alpha = rz / p.Ap; x += alpha p; r -= alpha Ap; z = k r; pnorm = ||z||; rz' = r.z;
//     beta = rz'/rz; p = z + beta p; rz = rz'
// with the scalars kept on the device: each kernel's last block (reduce.cuh) derives alpha or beta and the
// stop flag, and every block of a finished instance returns at once.  The host only polls the number of
// unfinished instances every few iterations; no kernel waits on another.
//
// One thread owns one node (its 3 rows).  ELL entry (s, fi, fj) of node n is vals[(s*9+fi*3+fj)*np + n], so
// the 81 value streams of a warp are coalesced; the 27 neighbour columns are implicit (structured grid)
// and their x values come through L1/L2.  Boundary rows are identity rows.
#include <cuda_runtime.h>

#include "device.cuh"
#include "launch.h"
#include "reduce.cuh"

namespace mgb {

constexpr int kUpdRows = 4;  // rows per thread of the vector update

__device__ __forceinline__ bool node_boundary(const MeshDev &m, int n, int &i, int &j, int &k) {
  i = n % m.nx;
  j = (n / m.nx) % m.ny;
  k = n / m.nxny;
  return i == 0 || j == 0 || k == 0 || i == m.nx - 1 || j == m.ny - 1 || k == m.nz - 1;
}

__global__ void __launch_bounds__(kNodeBlock) k_cg_setup(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[2] = {0.0, 0.0};  // r.z, z.z
  if (n < m.nn) {
    int i, j, k;
    const bool bnd = node_boundary(m, n, i, j, k);
    const double *__restrict__ vals = I.vals;
    const double *__restrict__ b = I.b;
    double *__restrict__ kinv = I.kinv;
    double *__restrict__ x = I.du;
    double *__restrict__ rv = I.r;
    double *__restrict__ zv = I.z;
    double *__restrict__ pv = I.p;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int row = n * 3 + d;
      const double kd = bnd ? 1.0 : 1 / vals[(size_t)(13 * 9 + d * 3 + d) * m.np + n];
      const double r = b[row];
      const double z = kd * r;
      kinv[row] = kd;
      x[row] = 0.0;
      rv[row] = r;
      zv[row] = z;
      pv[row] = z;
      acc[0] += r * z;
      acc[1] += z * z;
    }
  }
  double tot[2];
  if (grid_sum<2>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    CgState *c = I.cg;
    c->rz = tot[0];
    c->pnorm0 = sqrt(tot[1]);
    c->pnorm = c->pnorm0;
    c->its = 0;
    c->beta = 0.0;
    c->done = !(c->its < c->max_its) || c->pnorm < c->min_err || c->pnorm < c->pnorm0 * c->rel_err;
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      c->done = 1;
      I.out->nonfinite = 1;
    }
  }
}

// Ap = A p and p.Ap; the last block sets alpha = rz / p.Ap.
__global__ void __launch_bounds__(kNodeBlock) k_cg_spmv(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  if (I.cg->done) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[1] = {0.0};
  if (n < m.nn) {
    int i, j, k;
    const double *__restrict__ p = I.p;
    double *__restrict__ Ap = I.Ap;
    if (node_boundary(m, n, i, j, k)) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const double pv = p[n * 3 + d];
        Ap[n * 3 + d] = pv;
        acc[0] += pv * pv;
      }
    } else {
      const double *__restrict__ v = I.vals + n;
      const size_t np = m.np;
      double y0 = 0.0, y1 = 0.0, y2 = 0.0;
#pragma unroll
      for (int s = 0; s < 27; ++s) {
        const int nb = n + (s / 9 - 1) * m.nxny + ((s / 3) % 3 - 1) * m.nx + (s % 3 - 1);
        const double x0 = p[nb * 3 + 0], x1 = p[nb * 3 + 1], x2 = p[nb * 3 + 2];
        const double *vs = v + (size_t)(s * 9) * np;
        y0 += __ldcs(vs + 0 * np) * x0;
        y0 += __ldcs(vs + 1 * np) * x1;
        y0 += __ldcs(vs + 2 * np) * x2;
        y1 += __ldcs(vs + 3 * np) * x0;
        y1 += __ldcs(vs + 4 * np) * x1;
        y1 += __ldcs(vs + 5 * np) * x2;
        y2 += __ldcs(vs + 6 * np) * x0;
        y2 += __ldcs(vs + 7 * np) * x1;
        y2 += __ldcs(vs + 8 * np) * x2;
      }
      Ap[n * 3 + 0] = y0;
      Ap[n * 3 + 1] = y1;
      Ap[n * 3 + 2] = y2;
      acc[0] = p[n * 3 + 0] * y0 + p[n * 3 + 1] * y1 + p[n * 3 + 2] * y2;
    }
  }
  double tot[1];
  if (grid_sum<1>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    CgState *c = I.cg;
    c->pAp = tot[0];
    c->alpha = c->rz / tot[0];
  }
}

// x += alpha p; r -= alpha Ap; z = k r; then ||z|| and r.z; the last block sets beta and the stop flag.
__global__ void __launch_bounds__(kNodeBlock) k_cg_update(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const CgState *cs = I.cg;
  if (cs->done) return;
  const double alpha = cs->alpha;
  const int nrow = m.nn * 3;
  double *__restrict__ x = I.du;
  double *__restrict__ rv = I.r;
  double *__restrict__ zv = I.z;
  const double *__restrict__ p = I.p;
  const double *__restrict__ Ap = I.Ap;
  const double *__restrict__ kinv = I.kinv;
  double acc[2] = {0.0, 0.0};  // z.z, r.z
  // kUpdRows rows per thread, strided by the grid so that every load is coalesced; all loads first.
  const int stride = gridDim.x * blockDim.x;
  for (int row0 = blockIdx.x * blockDim.x + threadIdx.x; row0 < nrow; row0 += kUpdRows * stride) {
    double pv[kUpdRows], av[kUpdRows], rr[kUpdRows], xv[kUpdRows], kv[kUpdRows];
#pragma unroll
    for (int q = 0; q < kUpdRows; ++q) {
      const int row = row0 + q * stride;
      if (row < nrow) {
        pv[q] = p[row]; av[q] = Ap[row]; rr[q] = rv[row]; xv[q] = x[row]; kv[q] = kinv[row];
      }
    }
#pragma unroll
    for (int q = 0; q < kUpdRows; ++q) {
      const int row = row0 + q * stride;
      if (row < nrow) {
        x[row] = xv[q] + alpha * pv[q];
        const double r = rr[q] - alpha * av[q];
        const double z = kv[q] * r;
        rv[row] = r;
        zv[row] = z;
        acc[0] += z * z;
        acc[1] += r * z;
      }
    }
  }
  double tot[2];
  if (grid_sum<2>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    CgState *c = I.cg;
    c->pnorm = sqrt(tot[0]);
    c->beta = tot[1] / c->rz;
    c->rz = tot[1];
    c->its += 1;
    c->done = !(c->its < c->max_its) || c->pnorm < c->min_err || c->pnorm < c->pnorm0 * c->rel_err;
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      c->done = 1;
      I.out->nonfinite = 1;
    }
    if (c->done) {
      I.out->cg_its = c->its;
      I.out->cg_maxed = !(c->its < c->max_its) && !(c->pnorm < c->min_err || c->pnorm < c->pnorm0 * c->rel_err);
    }
  }
}

// p = z + beta p (skipped once the instance has stopped: p is not used again).
__global__ void __launch_bounds__(kNodeBlock) k_cg_pupdate(MeshDev m, const Inst *insts, const int *list,
                                                           unsigned int *active_count) {
  const Inst &I = insts[list[blockIdx.y]];
  const CgState *cs = I.cg;
  if (cs->done) return;
  const double beta = cs->beta;
  const int nrow = m.nn * 3;
  double *__restrict__ p = I.p;
  const double *__restrict__ z = I.z;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < nrow; row += gridDim.x * blockDim.x)
    p[row] = z[row] + beta * p[row];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(active_count, 1u);
}

// Setup leaves out.cg_its = 0 for instances that stop before the first iteration.
__global__ void k_cg_init_out(const Inst *insts, const int *list, int nlist) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nlist) {
    const Inst &I = insts[list[t]];
    I.out->cg_its = 0;
    I.out->cg_maxed = 0;
  }
}

}  // namespace mgb

using namespace mgb;

static inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

extern "C" {

int mgb_launch_cg_setup(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg_init_out<<<cdiv(nlist, 128), 128, 0, s>>>(insts, list, nlist);
  k_cg_setup<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

// One CG iteration = spmv (+ p.Ap, alpha), update (+ ||z||, r.z, beta, stop flag), p-update.
int mgb_launch_cg_spmv(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg_spmv<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_cg_update(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg_update<<<dim3(cdiv((size_t)m->nn * 3, (size_t)kUpdRows * kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts,
                                                                                                      list);
  return (int)cudaGetLastError();
}

// active_count receives +1 for every instance that is still iterating.
int mgb_launch_cg_pupdate(const MeshDev *m, const Inst *insts, const int *list, int nlist, unsigned int *active_count,
                          cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg_pupdate<<<dim3(cdiv((size_t)m->nn * 3, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list,
                                                                                         active_count);
  return (int)cudaGetLastError();
}

}  // extern "C"
