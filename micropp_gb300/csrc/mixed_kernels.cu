// mixed_kernels.cu -- the mixed-precision form (sm_103a): FP32 Jacobian CG inside FP64 refinement, and the
// implicit-differentiation ctan.
//
// Newton (mixed): the residual b and its norm stay FP64 (fe_kernels.cu); the Jacobian is assembled in FP32
// (k_elem_mat<float>) and K du = b is solved by Jacobi-preconditioned CG with FP32 vectors and FP64 dot-product
// accumulation.  The FP64 Newton residual is the refinement residual: each Newton step corrects the FP32 solve.
//
// ctan (implicit): at the converged state, with K_t the consistent tangent (FP64 Gauss-point tangents, FP32
// assembly), the derivative of the displacement with respect to macro strain component i is
//   du/deps_i = w_i + x_i,   K_II x_i = f_i = -K_IB w_i,
// where w_i is the affine boundary field of the unit strain e_i (micro3D.cpp:26-78 with eps = e_i) and x_i
// vanishes on the boundary.  The six systems are solved together (one pass over K per iteration serves all
// six) by FP32 CG, refined with FP64 residuals f_i - K x_i, and
//   ctan[v][i] = (1/V) sum_e sum_gp wg (C_gp B (w_i + x_i)_e)_v
// is accumulated in FP64.  This replaces the six perturbed Newton solves of homogenize.cpp:256-275.
#include <cuda_runtime.h>

#include "device.cuh"
#include "launch.h"
#include "laws.cuh"
#include "reduce.cuh"

namespace mgb {

namespace {

__device__ __constant__ int c_corner6[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                              {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

__device__ __forceinline__ bool bnd(const MeshDev &m, int n, int &i, int &j, int &k) {
  i = n % m.nx;
  j = (n / m.nx) % m.ny;
  k = n / m.nxny;
  return i == 0 || j == 0 || k == 0 || i == m.nx - 1 || j == m.ny - 1 || k == m.nz - 1;
}

// Coordinates a boundary node takes in the affine boundary condition (same face priority as k_set_bc).
__device__ __forceinline__ void bc_coords(const MeshDev &m, int i, int j, int k, double c[3]) {
  if (i == m.nx - 1) {
    c[0] = m.lx; c[1] = j * m.dy; c[2] = k * m.dz;
  } else if (i == 0) {
    c[0] = 0; c[1] = j * m.dy; c[2] = k * m.dz;
  } else if (j == m.ny - 1) {
    c[0] = i * m.dx; c[1] = m.ly; c[2] = k * m.dz;
  } else if (j == 0) {
    c[0] = i * m.dx; c[1] = 0; c[2] = k * m.dz;
  } else if (k == m.nz - 1) {
    c[0] = i * m.dx; c[1] = j * m.dy; c[2] = m.lz;
  } else {
    c[0] = i * m.dx; c[1] = j * m.dy; c[2] = 0;
  }
}

// Boundary displacement of the unit Voigt strain e_r (engineering shear: e_3 gives eps_xy = 1/2).
__device__ __forceinline__ void lift(const double c[3], int r, double w[3]) {
  w[0] = w[1] = w[2] = 0.0;
  switch (r) {
    case 0: w[0] = c[0]; break;
    case 1: w[1] = c[1]; break;
    case 2: w[2] = c[2]; break;
    case 3: w[0] = 0.5 * c[1]; w[1] = 0.5 * c[0]; break;
    case 4: w[0] = 0.5 * c[2]; w[2] = 0.5 * c[0]; break;
    default: w[1] = 0.5 * c[2]; w[2] = 0.5 * c[1]; break;
  }
}

__device__ __forceinline__ int nb_of(const MeshDev &m, int n, int s) {
  return n + (s / 9 - 1) * m.nxny + ((s / 3) % 3 - 1) * m.nx + (s % 3 - 1);
}

}  // namespace

// ---------------------------------------------------------------------------------------------------
// Single right-hand side FP32 CG (the Newton correction of the mixed form).

__global__ void __launch_bounds__(kNodeBlock) k_cg32_setup(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[2] = {0.0, 0.0};
  if (n < m.nn) {
    int i, j, k;
    const bool b = bnd(m, n, i, j, k);
    const float *__restrict__ vals = I.vals32;
    const double *__restrict__ bb = I.b;
    float *__restrict__ kinv = I.kinv32;
    float *__restrict__ du = I.du32;
    float *__restrict__ rv = I.r32;
    float *__restrict__ zv = I.z32;
    float *__restrict__ pv = I.p32;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int row = n * 3 + d;
      const float kd = b ? 1.0f : 1.0f / vals[(size_t)(13 * 9 + d * 3 + d) * m.np + n];
      const float r = (float)bb[row];
      const float z = kd * r;
      kinv[row] = kd;
      du[row] = 0.0f;
      rv[row] = r;
      zv[row] = z;
      pv[row] = z;
      acc[0] += (double)r * (double)z;
      acc[1] += (double)z * (double)z;
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

__global__ void __launch_bounds__(kNodeBlock) k_cg32_spmv(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  if (I.cg->done) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[1] = {0.0};
  if (n < m.nn) {
    int i, j, k;
    const float *__restrict__ p = I.p32;
    float *__restrict__ Ap = I.Ap32;
    if (bnd(m, n, i, j, k)) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float pv = p[n * 3 + d];
        Ap[n * 3 + d] = pv;
        acc[0] += (double)pv * (double)pv;
      }
    } else {
      const float *__restrict__ v = I.vals32 + n;
      const size_t np = m.np;
      float y0 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll
      for (int s = 0; s < 27; ++s) {
        const int nb = nb_of(m, n, s);
        const float x0 = p[nb * 3 + 0], x1 = p[nb * 3 + 1], x2 = p[nb * 3 + 2];
        const float *vs = v + (size_t)(s * 9) * np;
        y0 = fmaf(__ldcs(vs + 0 * np), x0, y0);
        y0 = fmaf(__ldcs(vs + 1 * np), x1, y0);
        y0 = fmaf(__ldcs(vs + 2 * np), x2, y0);
        y1 = fmaf(__ldcs(vs + 3 * np), x0, y1);
        y1 = fmaf(__ldcs(vs + 4 * np), x1, y1);
        y1 = fmaf(__ldcs(vs + 5 * np), x2, y1);
        y2 = fmaf(__ldcs(vs + 6 * np), x0, y2);
        y2 = fmaf(__ldcs(vs + 7 * np), x1, y2);
        y2 = fmaf(__ldcs(vs + 8 * np), x2, y2);
      }
      Ap[n * 3 + 0] = y0;
      Ap[n * 3 + 1] = y1;
      Ap[n * 3 + 2] = y2;
      acc[0] = (double)(p[n * 3 + 0] * y0 + p[n * 3 + 1] * y1 + p[n * 3 + 2] * y2);
    }
  }
  double tot[1];
  if (grid_sum<1>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    CgState *c = I.cg;
    c->pAp = tot[0];
    c->alpha = c->rz / tot[0];
  }
}

__global__ void __launch_bounds__(kNodeBlock) k_cg32_update(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const CgState *cs = I.cg;
  if (cs->done) return;
  const float alpha = (float)cs->alpha;
  const int nrow = m.nn * 3;
  float *__restrict__ du = I.du32;
  float *__restrict__ rv = I.r32;
  float *__restrict__ zv = I.z32;
  const float *__restrict__ p = I.p32;
  const float *__restrict__ Ap = I.Ap32;
  const float *__restrict__ kinv = I.kinv32;
  double acc[2] = {0.0, 0.0};
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < nrow; row += gridDim.x * blockDim.x) {
    du[row] = fmaf(alpha, p[row], du[row]);
    const float r = fmaf(-alpha, Ap[row], rv[row]);
    const float z = kinv[row] * r;
    rv[row] = r;
    zv[row] = z;
    acc[0] += (double)(z * z);
    acc[1] += (double)(r * z);
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

__global__ void __launch_bounds__(kNodeBlock) k_cg32_pupdate(MeshDev m, const Inst *insts, const int *list,
                                                             unsigned int *active_count) {
  const Inst &I = insts[list[blockIdx.y]];
  const CgState *cs = I.cg;
  if (cs->done) return;
  const float beta = (float)cs->beta;
  const int nrow = m.nn * 3;
  float *__restrict__ p = I.p32;
  const float *__restrict__ z = I.z32;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < nrow; row += gridDim.x * blockDim.x)
    p[row] = fmaf(beta, p[row], z[row]);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(active_count, 1u);
}

__global__ void k_add_du32(int nndim, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  double *__restrict__ u = I.u;
  const float *__restrict__ du = I.du32;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nndim; t += gridDim.x * blockDim.x) u[t] += (double)du[t];
}

// ---------------------------------------------------------------------------------------------------
// Six right-hand sides of the implicit ctan.

// f_i = -K_IB w_i on interior rows (FP64 accumulation of the FP32 tangent), 0 on boundary rows; x_i = 0.
__global__ void __launch_bounds__(kNodeBlock) k_t6_rhs(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  if (n < m.nn) {
    int i, j, k;
    double f[6][3];
#pragma unroll
    for (int r = 0; r < 6; ++r) f[r][0] = f[r][1] = f[r][2] = 0.0;
    if (!bnd(m, n, i, j, k)) {
      const float *__restrict__ v = I.vals32 + n;
      const size_t np = m.np;
#pragma unroll 1
      for (int s = 0; s < 27; ++s) {
        const int nb = nb_of(m, n, s);
        int bi, bj, bk;
        if (!bnd(m, nb, bi, bj, bk)) continue;
        double c[3];
        bc_coords(m, bi, bj, bk, c);
        double Kb[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) Kb[q] = (double)v[(size_t)(s * 9 + q) * np];
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          double w[3];
          lift(c, r, w);
#pragma unroll
          for (int fi = 0; fi < 3; ++fi) f[r][fi] -= Kb[fi * 3 + 0] * w[0] + Kb[fi * 3 + 1] * w[1] + Kb[fi * 3 + 2] * w[2];
        }
      }
    }
    double *__restrict__ F6 = I.F6;
    double *__restrict__ X6 = I.X6;
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const size_t idx = ((size_t)n * 6 + r) * 3 + d;
        F6[idx] = f[r][d];
        X6[idx] = 0.0;
        acc[r] += f[r][d] * f[r][d];
      }
    // Jacobi inverse of the tangent for the 6-RHS CG (boundary rows are identity rows)
    float *__restrict__ kinv = I.kinv32;
    const bool b = bnd(m, n, i, j, k);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      kinv[n * 3 + d] = b ? 1.0f : 1.0f / I.vals32[(size_t)(13 * 9 + d * 3 + d) * m.np + n];
  }
  double tot[6];
  if (grid_sum<6>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0)
    for (int r = 0; r < 6; ++r) I.out->f6[r] = sqrt(tot[r]);
}

// Refinement residual RF = F - K X (FP64 accumulation), start of a 6-RHS CG on it:
// R = RF (FP32), D = 0, Z = kinv R, P = Z; the last block initialises the six CG states.
__global__ void __launch_bounds__(kNodeBlock) k_t6_residual(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[18];
#pragma unroll
  for (int q = 0; q < 18; ++q) acc[q] = 0.0;  // [0,6): r.z  [6,12): z.z  [12,18): |RF|^2
  if (n < m.nn) {
    int i, j, k;
    const bool b = bnd(m, n, i, j, k);
    double rf[6][3];
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) rf[r][d] = b ? 0.0 : I.F6[((size_t)n * 6 + r) * 3 + d];
    float kd[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) kd[d] = I.kinv32[n * 3 + d];
    if (!b) {
      const float *__restrict__ v = I.vals32 + n;
      const size_t np = m.np;
#pragma unroll 1
      for (int s = 0; s < 27; ++s) {
        const int nb = nb_of(m, n, s);
        double Kb[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) Kb[q] = (double)v[(size_t)(s * 9 + q) * np];
        const double *x = I.X6 + (size_t)nb * 18;
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          const double x0 = x[r * 3], x1 = x[r * 3 + 1], x2 = x[r * 3 + 2];
#pragma unroll
          for (int fi = 0; fi < 3; ++fi) rf[r][fi] -= Kb[fi * 3] * x0 + Kb[fi * 3 + 1] * x1 + Kb[fi * 3 + 2] * x2;
        }
      }
    }
    float *__restrict__ R6 = I.R6;
    float *__restrict__ Z6 = I.Z6;
    float *__restrict__ P6 = I.P6;
    float *__restrict__ D6 = I.D6;
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const size_t idx = ((size_t)n * 6 + r) * 3 + d;
        const float rr = (float)rf[r][d];
        const float z = kd[d] * rr;
        R6[idx] = rr;
        Z6[idx] = z;
        P6[idx] = z;
        D6[idx] = 0.0f;
        acc[r] += (double)rr * (double)z;
        acc[6 + r] += (double)z * (double)z;
        acc[12 + r] += rf[r][d] * rf[r][d];
      }
  }
  double tot[18];
  if (grid_sum<18>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    Cg6State *c = I.cg6;
    c->its = 0;
    int all = 1;
    for (int r = 0; r < 6; ++r) {
      c->rz[r] = tot[r];
      c->pnorm0[r] = sqrt(tot[6 + r]);
      c->pnorm[r] = c->pnorm0[r];
      c->beta[r] = 0.0;
      c->alpha[r] = 0.0;
      c->done[r] = !(0 < c->max_its) || c->pnorm[r] <= c->min_err || !isfinite(tot[r]) || !isfinite(tot[6 + r]);
      all &= c->done[r];
      I.out->res6[r] = sqrt(tot[12 + r]);
      if (!isfinite(tot[12 + r])) I.out->nonfinite = 1;
    }
    c->all_done = all;
    I.out->cg6_its = 0;
  }
}

// AP = K P for the six right-hand sides, one pass over K; the last block sets alpha_r.
__global__ void __launch_bounds__(kNodeBlock) k_cg6_spmv(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  if (I.cg6->all_done) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  if (n < m.nn) {
    int i, j, k;
    const float *__restrict__ P = I.P6;
    float y[18];
    if (bnd(m, n, i, j, k)) {
#pragma unroll
      for (int q = 0; q < 18; ++q) y[q] = P[(size_t)n * 18 + q];
    } else {
#pragma unroll
      for (int q = 0; q < 18; ++q) y[q] = 0.f;
      const float *__restrict__ v = I.vals32 + n;
      const size_t np = m.np;
#pragma unroll 3
      for (int s = 0; s < 27; ++s) {
        const int nb = nb_of(m, n, s);
        float Kb[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) Kb[q] = __ldcs(v + (size_t)(s * 9 + q) * np);
        const float2 *x2 = reinterpret_cast<const float2 *>(P + (size_t)nb * 18);
        float x[18];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
          const float2 t = x2[q];
          x[2 * q] = t.x;
          x[2 * q + 1] = t.y;
        }
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
          for (int fi = 0; fi < 3; ++fi) {
            float a = y[r * 3 + fi];
            a = fmaf(Kb[fi * 3 + 0], x[r * 3 + 0], a);
            a = fmaf(Kb[fi * 3 + 1], x[r * 3 + 1], a);
            a = fmaf(Kb[fi * 3 + 2], x[r * 3 + 2], a);
            y[r * 3 + fi] = a;
          }
      }
    }
    float2 *__restrict__ ap2 = reinterpret_cast<float2 *>(I.AP6 + (size_t)n * 18);
    const float2 *p2 = reinterpret_cast<const float2 *>(P + (size_t)n * 18);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      ap2[q] = make_float2(y[2 * q], y[2 * q + 1]);
      const float2 pv = p2[q];
      acc[(2 * q) / 3] += (double)(pv.x * y[2 * q]);
      acc[(2 * q + 1) / 3] += (double)(pv.y * y[2 * q + 1]);
    }
  }
  double tot[6];
  if (grid_sum<6>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    Cg6State *c = I.cg6;
    for (int r = 0; r < 6; ++r) c->alpha[r] = c->done[r] ? 0.0 : c->rz[r] / tot[r];
  }
}

// D += alpha P; R -= alpha AP; Z = kinv R per right-hand side; the last block sets beta_r and the stop flags.
__global__ void __launch_bounds__(kNodeBlock) k_cg6_update(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const Cg6State *cs = I.cg6;
  if (cs->all_done) return;
  float alpha[6];
#pragma unroll
  for (int r = 0; r < 6; ++r) alpha[r] = (float)cs->alpha[r];
  double acc[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) acc[q] = 0.0;  // [0,6): z.z  [6,12): r.z
  float *__restrict__ D6 = I.D6;
  float *__restrict__ R6 = I.R6;
  float *__restrict__ Z6 = I.Z6;
  const float *__restrict__ P6 = I.P6;
  const float *__restrict__ AP6 = I.AP6;
  const float *__restrict__ kinv = I.kinv32;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < m.nn; n += gridDim.x * blockDim.x) {
    float kd[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) kd[d] = kinv[n * 3 + d];
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const size_t idx = ((size_t)n * 6 + r) * 3 + d;
        D6[idx] = fmaf(alpha[r], P6[idx], D6[idx]);
        const float rr = fmaf(-alpha[r], AP6[idx], R6[idx]);
        const float z = kd[d] * rr;
        R6[idx] = rr;
        Z6[idx] = z;
        acc[r] += (double)(z * z);
        acc[6 + r] += (double)(rr * z);
      }
  }
  double tot[12];
  if (grid_sum<12>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    Cg6State *c = I.cg6;
    c->its += 1;
    int all = 1;
    for (int r = 0; r < 6; ++r) {
      if (!c->done[r]) {
        c->pnorm[r] = sqrt(tot[r]);
        c->beta[r] = tot[6 + r] / c->rz[r];
        c->rz[r] = tot[6 + r];
        c->done[r] = !(c->its < c->max_its) || c->pnorm[r] < c->min_err || c->pnorm[r] < c->pnorm0[r] * c->rel_err ||
                     !isfinite(tot[r]);
      }
      all &= c->done[r];
    }
    c->all_done = all;
    if (all) I.out->cg6_its = c->its;
  }
}

__global__ void __launch_bounds__(kNodeBlock) k_cg6_pupdate(MeshDev m, const Inst *insts, const int *list,
                                                            unsigned int *active_count) {
  const Inst &I = insts[list[blockIdx.y]];
  const Cg6State *cs = I.cg6;
  if (cs->all_done) return;
  float beta[6];
  bool live[6];
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    beta[r] = (float)cs->beta[r];
    live[r] = !cs->done[r];
  }
  float *__restrict__ P6 = I.P6;
  const float *__restrict__ Z6 = I.Z6;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < m.nn; n += gridDim.x * blockDim.x) {
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      if (!live[r]) continue;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const size_t idx = ((size_t)n * 6 + r) * 3 + d;
        P6[idx] = fmaf(beta[r], P6[idx], Z6[idx]);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(active_count, 1u);
}

// X += D (FP64 accumulation of the FP32 correction).
__global__ void k_t6_accumulate(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const size_t total = (size_t)m.nn * 18;
  double *__restrict__ X6 = I.X6;
  const float *__restrict__ D6 = I.D6;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x)
    X6[t] += (double)D6[t];
}

// ctan[v][i] = (1/V) sum over Gauss points of wg (C_gp B (w_i + x_i))_v, one thread per Gauss point, FP64.
__global__ void __launch_bounds__(128) k_ctan_avg(MeshDev m, Mats mats, const int8_t *etype, const double *dsh_g,
                                                  const Inst *insts, const int *list) {
  __shared__ double dsh[8 * 24];
  for (int t = threadIdx.x; t < 192; t += blockDim.x) dsh[t] = dsh_g[t];
  __syncthreads();
  const Inst &I = insts[list[blockIdx.y]];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[36];
#pragma unroll
  for (int q = 0; q < 36; ++q) acc[q] = 0.0;
  if (t < m.nelem * 8) {
    const int e = t >> 3, g = t & 7;
    const int ex = e % m.nex, ey = (e / m.nex) % m.ney, ez = e / (m.nex * m.ney);
    const int n0 = ez * m.nxny + ey * m.nx + ex;
    const double *dg = &dsh[g * 24];
    const MatDev &mat = mats.m[etype[e]];
    int nodes[8];
    bool nb_bnd[8];
    double cc[8][3];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      nodes[a] = n0 + c_corner6[a][2] * m.nxny + c_corner6[a][1] * m.nx + c_corner6[a][0];
      int bi, bj, bk;
      nb_bnd[a] = bnd(m, nodes[a], bi, bj, bk);
      if (nb_bnd[a]) bc_coords(m, bi, bj, bk, cc[a]);
    }
    double ue[24], eps[6], C[36];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int d = 0; d < 3; ++d) ue[a * 3 + d] = I.u[nodes[a] * 3 + d];
    {
      double e0 = 0, e1 = 0, e2 = 0, e3 = 0, e4 = 0, e5 = 0;
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const double gx = dg[a * 3], gy = dg[a * 3 + 1], gz = dg[a * 3 + 2];
        e0 += gx * ue[a * 3]; e1 += gy * ue[a * 3 + 1]; e2 += gz * ue[a * 3 + 2];
        e3 += gy * ue[a * 3] + gx * ue[a * 3 + 1];
        e4 += gz * ue[a * 3] + gx * ue[a * 3 + 2];
        e5 += gz * ue[a * 3 + 1] + gy * ue[a * 3 + 2];
      }
      eps[0] = e0; eps[1] = e1; eps[2] = e2; eps[3] = e3; eps[4] = e4; eps[5] = e5;
    }
    law_ctan_exact(mat, eps, I.vars_old ? I.vars_old + ((size_t)e * 8 + g) * kNvarGp : nullptr, C);
#pragma unroll 1
    for (int r = 0; r < 6; ++r) {
      double s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0;
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const double *x = I.X6 + ((size_t)nodes[a] * 6 + r) * 3;
        double ux = x[0], uy = x[1], uz = x[2];
        if (nb_bnd[a]) {
          double w[3];
          lift(cc[a], r, w);
          ux += w[0];
          uy += w[1];
          uz += w[2];
        }
        const double gx = dg[a * 3], gy = dg[a * 3 + 1], gz = dg[a * 3 + 2];
        s0 += gx * ux; s1 += gy * uy; s2 += gz * uz;
        s3 += gy * ux + gx * uy;
        s4 += gz * ux + gx * uz;
        s5 += gz * uy + gy * uz;
      }
      const double st[6] = {s0, s1, s2, s3, s4, s5};
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        double sv = 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q) sv += C[v * 6 + q] * st[q];
        acc[v * 6 + r] += sv * m.wg;
      }
    }
  }
  double tot[36];
  if (grid_sum<36>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    bool bad = false;
    for (int q = 0; q < 36; ++q) {
      I.out->ctan[q] = tot[q] / m.vol_tot;
      bad |= !isfinite(tot[q]);
    }
    if (bad) I.out->nonfinite = 1;
  }
}

}  // namespace mgb

using namespace mgb;

static inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

extern "C" {

int mgb_launch_cg32_setup(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg32_setup<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_cg32_spmv(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg32_spmv<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_cg32_update(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg32_update<<<dim3(cdiv((size_t)m->nn * 3, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_cg32_pupdate(const MeshDev *m, const Inst *insts, const int *list, int nlist,
                            unsigned int *active_count, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg32_pupdate<<<dim3(cdiv((size_t)m->nn * 3, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list,
                                                                                           active_count);
  return (int)cudaGetLastError();
}

int mgb_launch_add_du32(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const int nndim = m->nn * 3;
  k_add_du32<<<dim3(cdiv(nndim, 4 * kNodeBlock), nlist), kNodeBlock, 0, s>>>(nndim, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_t6_rhs(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_t6_rhs<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_t6_residual(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_t6_residual<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_cg6_spmv(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg6_spmv<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_cg6_update(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg6_update<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_cg6_pupdate(const MeshDev *m, const Inst *insts, const int *list, int nlist,
                           unsigned int *active_count, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg6_pupdate<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list, active_count);
  return (int)cudaGetLastError();
}

int mgb_launch_t6_accumulate(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_t6_accumulate<<<dim3(cdiv((size_t)m->nn * 18, kNodeBlock * 8), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_ctan_avg(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh, const Inst *insts,
                        const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_ctan_avg<<<dim3(cdiv((size_t)m->nelem * 8, 128), nlist), 128, 0, s>>>(*m, *mats, etype, dsh, insts, list);
  return (int)cudaGetLastError();
}

}  // extern "C"
