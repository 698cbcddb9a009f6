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
// six) by FP32 CG, refined with residuals f_i - K x_i in double-float arithmetic (x_i and f_i are held as pairs
// of floats, hi + lo), and ctan follows from the tangent fields w_i + x_i: as the element-energy sum (elastic and
// damage phases) or the FP64 Gauss-point average of C_gp B (w_i + x_i) (a J2 phase).  This replaces the six
// perturbed Newton solves of homogenize.cpp:256-275.
#include <cuda_runtime.h>

#include "bc.cuh"
#include "device.cuh"
#include "df.cuh"
#include "launch.h"
#include "laws.cuh"
#include "reduce.cuh"

namespace mgb {

namespace {

__device__ __constant__ int c_corner6[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                              {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

__device__ __forceinline__ int nb_of(const MeshDev &m, int n, int s) {
  return n + (s / 9 - 1) * m.nxny + ((s / 3) % 3 - 1) * m.nx + (s % 3 - 1);
}

// The 3x3 block (row-major fi, fj) of FP32 ELL row n at stencil slot s.
template <typename T>
__device__ __forceinline__ void ell32_block(const MeshDev &m, const float *__restrict__ vals, int n, int s, T (&K)[9]) {
#pragma unroll
  for (int q = 0; q < 9; ++q) K[q] = (T)vals[(size_t)(s * 9 + q) * m.np + n];
}

// Entry index of diagonal entry (d, d) of row n's own block in the FP32 ELL.
__device__ __forceinline__ size_t ell32_diag(const MeshDev &m, int n, int d) {
  return (size_t)(13 * 9 + d * 3 + d) * m.np + n;
}

// lift (bc.cuh) on double-float coordinates (ch + cl): w = e_r X with engineering shear, which only selects and
// halves coordinates (exact).
__device__ __forceinline__ void lift_df(const float (&ch)[3], const float (&cl)[3], int r, float (&wh)[3],
                                        float (&wl)[3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) wh[d] = wl[d] = 0.f;
  if (r < 3) {
    wh[r] = ch[r];
    wl[r] = cl[r];
  } else {
    const int a = (r == 5) ? 1 : 0, b = (r == 3) ? 1 : 2;
    wh[a] = 0.5f * ch[b];
    wl[a] = 0.5f * cl[b];
    wh[b] = 0.5f * ch[a];
    wl[b] = 0.5f * cl[a];
  }
}

}  // namespace

// ---------------------------------------------------------------------------------------------------
// Single right-hand side FP32 CG (the Newton correction of the mixed form).
//
// Dot products: each thread sums its few products in FP32, the grid reduction adds the thread sums in FP32
// within a warp and in FP64 above (grid_sum_f).

constexpr int kRowsPerThread = 4;   // vector kernels: rows per thread
constexpr int kSpmvNodes = 4;       // FP32 SpMV: consecutive nodes per thread (one 16-byte load per entry)
// Block sizes of the two SpMVs are template parameters (64, 128 or 256 threads), picked per RVE size and batch
// by the engine's autotuner.
constexpr int kSpmv6Nodes = 2;      // 6-RHS SpMV: consecutive nodes per thread (one 8-byte load per entry)

// mg: a V-cycle follows; z is then its pre-smoothed level-0 iterate, the smoother's inverse diagonal (lv[0].kinv)
// times r, and the V-cycle's last kernel sets p and rz.  ||D^-1 r|| with the plain diagonal stays the norm of the
// stop test either way.
__global__ void __launch_bounds__(kNodeBlock) k_cg32_setup(MeshDev m, const Inst *insts, const int *list, int mg) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  float acc[2] = {0.f, 0.f};
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
    const float *__restrict__ ks = mg ? I.mg->lv[0].kinv : nullptr;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int row = n * 3 + d;
      const float kd = b ? 1.0f : 1.0f / vals[ell32_diag(m, n, d)];
      const float r = (float)bb[row];
      const float zj = kd * r;
      const float z = mg ? ks[row] * r : zj;
      kinv[row] = kd;
      du[row] = 0.0f;
      rv[row] = r;
      zv[row] = z;
      pv[row] = z;
      acc[0] = fmaf(r, z, acc[0]);
      acc[1] = fmaf(zj, zj, acc[1]);
    }
  }
  double tot[2];
  if (grid_sum_f<2>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
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

// Ap = K p for kSpmvNodes consecutive nodes per thread.  Each ELL entry of the group is one 16-byte load
// (np is a multiple of 32 and the group starts at a multiple of 4), and the 6 neighbours a group row needs
// along x are loaded once for the 3 x-slots.  A boundary node of the group is an identity row: its stencil
// sum (taken over clamped neighbour indices) is discarded.
template <int B>
__global__ void __launch_bounds__(B) k_cg32_spmv(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  if (I.cg->done) return;
  const int n0 = (blockIdx.x * blockDim.x + threadIdx.x) * kSpmvNodes;
  float acc[1] = {0.f};
  if (n0 < m.nn) {
    const float *__restrict__ p = I.p32;
    float *__restrict__ Ap = I.Ap32;
    bool bn[kSpmvNodes];
    bool any_interior = false;
#pragma unroll
    for (int q = 0; q < kSpmvNodes; ++q) {
      int i, j, k;
      bn[q] = (n0 + q >= m.nn) || bnd(m, n0 + q, i, j, k);
      any_interior |= !bn[q];
    }
    float y[kSpmvNodes][3];
#pragma unroll
    for (int q = 0; q < kSpmvNodes; ++q) y[q][0] = y[q][1] = y[q][2] = 0.f;
    if (any_interior) {
      const size_t np4 = (size_t)m.np / 4;
      const float4 *__restrict__ v4 = reinterpret_cast<const float4 *>(I.vals32 + n0);
      const int last = m.nn - 1;
#pragma unroll 1
      for (int zy = 0; zy < 9; ++zy) {
        const int base = n0 + (zy / 3 - 1) * m.nxny + (zy % 3 - 1) * m.nx - 1;
        float x[kSpmvNodes + 2][3];
#pragma unroll
        for (int w = 0; w < kSpmvNodes + 2; ++w) {
          const int nb = min(max(base + w, 0), last);
          x[w][0] = p[nb * 3 + 0];
          x[w][1] = p[nb * 3 + 1];
          x[w][2] = p[nb * 3 + 2];
        }
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
          const float4 *vs = v4 + (size_t)((zy * 3 + dx) * 9) * np4;
#pragma unroll
          for (int e = 0; e < 9; ++e) {
            const float4 a = __ldcs(vs + e * np4);
            const int fi = e / 3, fj = e % 3;
            y[0][fi] = fmaf(a.x, x[0 + dx][fj], y[0][fi]);
            y[1][fi] = fmaf(a.y, x[1 + dx][fj], y[1][fi]);
            y[2][fi] = fmaf(a.z, x[2 + dx][fj], y[2][fi]);
            y[3][fi] = fmaf(a.w, x[3 + dx][fj], y[3][fi]);
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kSpmvNodes; ++q) {
      const int n = n0 + q;
      if (n >= m.nn) break;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float pv = p[n * 3 + d];
        const float yv = bn[q] ? pv : y[q][d];
        Ap[n * 3 + d] = yv;
        acc[0] = fmaf(pv, yv, acc[0]);
      }
    }
  }
  double tot[1];
  if (grid_sum_f<1>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    CgState *c = I.cg;
    c->pAp = tot[0];
    c->alpha = c->rz / tot[0];
  }
}

// du += alpha p; r -= alpha Ap; z = kinv r, kRowsPerThread rows per thread (loads of all rows first); the
// last block sets beta, the norms and the stop flag.
// mg: a V-cycle follows; z is its pre-smoothed level-0 iterate (the smoother's inverse diagonal times r) and
// beta, rz are left to the V-cycle's last kernel.  The stop test uses ||D^-1 r|| in both cases.
__global__ void __launch_bounds__(kNodeBlock) k_cg32_update(MeshDev m, const Inst *insts, const int *list, int mg) {
  const Inst &I = insts[list[blockIdx.y]];
  const CgState *cs = I.cg;
  if (cs->done) return;
  const float alpha = (float)cs->alpha;
  const float *__restrict__ ks = mg ? I.mg->lv[0].kinv : nullptr;
  const int nrow = m.nn * 3;
  float *__restrict__ du = I.du32;
  float *__restrict__ rv = I.r32;
  float *__restrict__ zv = I.z32;
  const float *__restrict__ p = I.p32;
  const float *__restrict__ Ap = I.Ap32;
  const float *__restrict__ kinv = I.kinv32;
  const int stride = gridDim.x * blockDim.x;
  float acc[2] = {0.f, 0.f};
  for (int row0 = blockIdx.x * blockDim.x + threadIdx.x; row0 < nrow; row0 += kRowsPerThread * stride) {
    float pv[kRowsPerThread], av[kRowsPerThread], rr[kRowsPerThread], dv[kRowsPerThread], kv[kRowsPerThread];
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
      const int row = row0 + q * stride;
      if (row < nrow) {
        pv[q] = p[row]; av[q] = Ap[row]; rr[q] = rv[row]; dv[q] = du[row]; kv[q] = kinv[row];
      }
    }
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
      const int row = row0 + q * stride;
      if (row < nrow) {
        du[row] = fmaf(alpha, pv[q], dv[q]);
        const float r = fmaf(-alpha, av[q], rr[q]);
        const float zj = kv[q] * r;
        const float z = mg ? ks[row] * r : zj;
        rv[row] = r;
        zv[row] = z;
        acc[0] = fmaf(zj, zj, acc[0]);
        acc[1] = fmaf(r, z, acc[1]);
      }
    }
  }
  double tot[2];
  if (grid_sum_f<2>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    CgState *c = I.cg;
    c->pnorm = sqrt(tot[0]);
    if (!mg) {
      c->beta = tot[1] / c->rz;
      c->rz = tot[1];
    }
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
  const int stride = gridDim.x * blockDim.x;
  for (int row0 = blockIdx.x * blockDim.x + threadIdx.x; row0 < nrow; row0 += kRowsPerThread * stride) {
    float pv[kRowsPerThread], zv[kRowsPerThread];
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
      const int row = row0 + q * stride;
      if (row < nrow) {
        pv[q] = p[row];
        zv[q] = z[row];
      }
    }
#pragma unroll
    for (int q = 0; q < kRowsPerThread; ++q) {
      const int row = row0 + q * stride;
      if (row < nrow) p[row] = fmaf(beta, pv[q], zv[q]);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(active_count, 1u);
}

// u += a du32 of one instance (the step length of the mixed form's line search).
__global__ void k_axpy_du32(int nndim, double *u, const float *du, double a) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nndim; t += gridDim.x * blockDim.x)
    u[t] += a * (double)du[t];
}

__global__ void k_add_du32(int nndim, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  double *__restrict__ u = I.u;
  const float *__restrict__ du = I.du32;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nndim; t += gridDim.x * blockDim.x) u[t] += (double)du[t];
}

// ---------------------------------------------------------------------------------------------------
// Six right-hand sides of the implicit ctan.  The vectors are component-major, V[c6(i, d, np) + n].

// X = 0, F = 0 and the Jacobi inverse of the tangent (boundary rows: identity rows) on every node; the right-hand
// sides of the interior nodes next to the boundary follow (k_t6_rhs_near).
__global__ void __launch_bounds__(kNodeBlock) k_t6_clear(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  int i, j, k;
  const bool b = bnd(m, n, i, j, k);
  const size_t np = m.np;
#pragma unroll
  for (int c = 0; c < 18; ++c) {
    const size_t idx = (size_t)c * np + n;
    I.F6h[idx] = 0.f;
    I.F6l[idx] = 0.f;
    I.X6h[idx] = 0.f;
    I.X6l[idx] = 0.f;
  }
  float *__restrict__ kinv = I.kinv32;
#pragma unroll
  for (int d = 0; d < 3; ++d) kinv[n * 3 + d] = b ? 1.0f : 1.0f / I.vals32[ell32_diag(m, n, d)];
}

// f_i = -K_IB w_i in double-float arithmetic on the interior nodes that have boundary neighbours -- the only
// nonzero rows -- one thread per node of the list `near`; ||f_i||.  The boundary coordinates are split into float
// pairs once per neighbour; the lift of a unit strain only selects and halves them (exact).
__global__ void __launch_bounds__(kNodeBlock) k_t6_rhs_near(MeshDev m, const int *near, int nnear, const Inst *insts,
                                                            const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (t < nnear) {
    const int n = near[t];
    int i, j, k;
    bnd(m, n, i, j, k);
    const size_t np = m.np;
    float fh[6][3], fl[6][3];
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) fh[r][d] = fl[r][d] = 0.f;
#pragma unroll 1
    for (int s = 0; s < 27; ++s) {
      const int bi = i + s % 3 - 1, bj = j + (s / 3) % 3 - 1, bk = k + s / 9 - 1;
      if (!(bi == 0 || bj == 0 || bk == 0 || bi == m.nx - 1 || bj == m.ny - 1 || bk == m.nz - 1)) continue;
      double c[3];
      bc_coords(m, bi, bj, bk, c);
      float ch[3], cl[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) df_split(c[d], ch[d], cl[d]);
      float Kb[9];
      ell32_block(m, I.vals32, n, s, Kb);
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        float wh[3], wl[3];
        lift_df(ch, cl, r, wh, wl);
#pragma unroll
        for (int fi = 0; fi < 3; ++fi)
#pragma unroll
          for (int fj = 0; fj < 3; ++fj) df_sub_prod(fh[r][fi], fl[r][fi], Kb[fi * 3 + fj], wh[fj], wl[fj]);
      }
    }
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const size_t idx = c6(r, d, np) + n;
        float h, l;
        two_sum(fh[r][d], fl[r][d], h, l);
        I.F6h[idx] = h;
        I.F6l[idx] = l;
        acc[r] = fmaf(h, h, acc[r]);
      }
  }
  double tot[6];
  if (grid_sum_f<6>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0)
    for (int r = 0; r < 6; ++r) I.out->f6[r] = sqrt(tot[r]);
}

// Refinement residual RF = F - K X in double-float arithmetic (FP32 operations only: K is FP32, F and X are
// double-float pairs; about 48 bits, enough for a 1e-9 relative residual), start of a 6-RHS CG on it:
// R = RF (FP32), D = 0, Z = kinv R, P = Z; the last block initialises the six CG states.  x_zero: X is
// still 0 (the first sweep), RF = F without the product.
// mg as in k_cg32_setup.
__global__ void __launch_bounds__(kNodeBlock) k_t6_residual(MeshDev m, const Inst *insts, const int *list,
                                                            int x_zero, int mg) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  float acc[18];
#pragma unroll
  for (int q = 0; q < 18; ++q) acc[q] = 0.f;  // [0,6): r.z  [6,12): z.z  [12,18): |RF|^2
  if (n < m.nn) {
    int i, j, k;
    const bool b = bnd(m, n, i, j, k);
    const size_t np = m.np;
    const float *__restrict__ Xh = I.X6h;
    const float *__restrict__ Xl = I.X6l;
    float rh[6][3], rl[6][3];
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        rh[r][d] = b ? 0.f : I.F6h[c6(r, d, np) + n];
        rl[r][d] = b ? 0.f : I.F6l[c6(r, d, np) + n];
      }
    float kd[3], ksm[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      kd[d] = I.kinv32[n * 3 + d];
      ksm[d] = mg ? I.mg->lv[0].kinv[n * 3 + d] : kd[d];
    }
    if (!b && !x_zero) {
#pragma unroll 1
      for (int s = 0; s < 27; ++s) {
        const int nb = nb_of(m, n, s);
        float Kb[9];
        ell32_block(m, I.vals32, n, s, Kb);
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          float xh[3], xl[3];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            xh[d] = Xh[c6(r, d, np) + nb];
            xl[d] = Xl[c6(r, d, np) + nb];
          }
#pragma unroll
          for (int fi = 0; fi < 3; ++fi)
#pragma unroll
            for (int fj = 0; fj < 3; ++fj) df_sub_prod(rh[r][fi], rl[r][fi], Kb[fi * 3 + fj], xh[fj], xl[fj]);
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
        const size_t idx = c6(r, d, np) + n;
        const float rr = __fadd_rn(rh[r][d], rl[r][d]);
        const float zj = kd[d] * rr;
        const float z = ksm[d] * rr;
        R6[idx] = rr;
        Z6[idx] = z;
        P6[idx] = z;
        D6[idx] = 0.0f;
        acc[r] = fmaf(rr, z, acc[r]);
        acc[6 + r] = fmaf(zj, zj, acc[6 + r]);
        acc[12 + r] = fmaf(rr, rr, acc[12 + r]);
      }
  }
  double tot[18];
  if (grid_sum_f<18>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
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

// AP = K P for the six right-hand sides on the full stencil, one pass over K for all six; kSpmv6Nodes
// consecutive nodes per thread, so each ELL entry of the pair is one 8-byte load and the 4 neighbours a pair
// row needs along x are loaded once for the 3 x-slots.  The last block sets alpha_i.
template <int B>
__global__ void __launch_bounds__(B) k_cg6_spmv(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  if (I.cg6->all_done) return;
  const int n0 = (blockIdx.x * blockDim.x + threadIdx.x) * kSpmv6Nodes;
  float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (n0 < m.nn) {
    const size_t np = m.np;
    const float *__restrict__ P = I.P6;
    float *__restrict__ AP = I.AP6;
    bool bn[kSpmv6Nodes];
    bool any_interior = false;
#pragma unroll
    for (int q = 0; q < kSpmv6Nodes; ++q) {
      int i, j, k;
      bn[q] = (n0 + q >= m.nn) || bnd(m, n0 + q, i, j, k);
      any_interior |= !bn[q];
    }
    float y[kSpmv6Nodes][18];
#pragma unroll
    for (int q = 0; q < kSpmv6Nodes; ++q)
#pragma unroll
      for (int c = 0; c < 18; ++c) y[q][c] = 0.f;
    if (any_interior) {
      const size_t np2 = np / 2;
      const float2 *__restrict__ v2 = reinterpret_cast<const float2 *>(I.vals32 + n0);
      const int last = m.nn - 1;
#pragma unroll 1
      for (int zy = 0; zy < 9; ++zy) {
        const int base = n0 + (zy / 3 - 1) * m.nxny + (zy % 3 - 1) * m.nx - 1;
        int nb[kSpmv6Nodes + 2];
#pragma unroll
        for (int w = 0; w < kSpmv6Nodes + 2; ++w) nb[w] = min(max(base + w, 0), last);
        float2 a[3][9];
#pragma unroll
        for (int dx = 0; dx < 3; ++dx)
#pragma unroll
          for (int e = 0; e < 9; ++e) a[dx][e] = __ldcs(v2 + (size_t)((zy * 3 + dx) * 9 + e) * np2);
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          float x[kSpmv6Nodes + 2][3];
#pragma unroll
          for (int w = 0; w < kSpmv6Nodes + 2; ++w)
#pragma unroll
            for (int d = 0; d < 3; ++d) x[w][d] = P[c6(r, d, np) + nb[w]];
#pragma unroll
          for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int e = 0; e < 9; ++e) {
              const int fi = e / 3, fj = e % 3;
              y[0][r * 3 + fi] = fmaf(a[dx][e].x, x[0 + dx][fj], y[0][r * 3 + fi]);
              y[1][r * 3 + fi] = fmaf(a[dx][e].y, x[1 + dx][fj], y[1][r * 3 + fi]);
            }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kSpmv6Nodes; ++q) {
      const int n = n0 + q;
      if (n >= m.nn) break;
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const size_t idx = c6(r, d, np) + n;
          const float pv = P[idx];
          const float yv = bn[q] ? pv : y[q][r * 3 + d];
          AP[idx] = yv;
          acc[r] = fmaf(pv, yv, acc[r]);
        }
    }
  }
  double tot[6];
  if (grid_sum_f<6>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    Cg6State *c = I.cg6;
    for (int r = 0; r < 6; ++r) c->alpha[r] = c->done[r] ? 0.0 : c->rz[r] / tot[r];
  }
}

// The 6-RHS vector updates work on chunks of kVec6Chunk nodes, kVec6PerThread per thread (nodes strided by
// the block size, so every access is coalesced).
constexpr int kVec6PerThread = 4;
constexpr int kVec6Chunk = kVec6PerThread * kNodeBlock;

// D += alpha P; R -= alpha AP; Z = kinv R for the right-hand sides still iterating.  A block takes one node
// chunk through the 18 components in turn (the 16 loads of a component in flight together); an instance has
// nn / kVec6Chunk blocks to reduce, and the last one sets beta_i and the stop flags.
// mg as in k_cg32_update.
__global__ void __launch_bounds__(kNodeBlock) k_cg6_update(MeshDev m, const Inst *insts, const int *list, int mg) {
  const Inst &I = insts[list[blockIdx.y]];
  const Cg6State *cs = I.cg6;
  if (cs->all_done) return;
  float alpha[6];
  bool live[6];
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    alpha[r] = (float)cs->alpha[r];
    live[r] = !cs->done[r];
  }
  float acc[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) acc[q] = 0.f;  // [0,6): z.z  [6,12): r.z
  const size_t np = m.np;
  const int n0 = blockIdx.x * kVec6Chunk + threadIdx.x;
  float kd[kVec6PerThread][3], ksm[kVec6PerThread][3];
#pragma unroll
  for (int q = 0; q < kVec6PerThread; ++q) {
    const int n = n0 + q * kNodeBlock;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      kd[q][d] = (n < m.nn) ? I.kinv32[n * 3 + d] : 0.f;
      ksm[q][d] = (n < m.nn && mg) ? I.mg->lv[0].kinv[n * 3 + d] : kd[q][d];
    }
  }
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    if (!live[r]) continue;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const size_t off = c6(r, d, np);
      float *__restrict__ D6 = I.D6 + off;
      float *__restrict__ R6 = I.R6 + off;
      float *__restrict__ Z6 = I.Z6 + off;
      const float *__restrict__ P6 = I.P6 + off;
      const float *__restrict__ AP6 = I.AP6 + off;
      float pv[kVec6PerThread], av[kVec6PerThread], rv[kVec6PerThread], dv[kVec6PerThread];
#pragma unroll
      for (int q = 0; q < kVec6PerThread; ++q) {
        const int n = n0 + q * kNodeBlock;
        if (n < m.nn) {
          pv[q] = P6[n]; av[q] = AP6[n]; rv[q] = R6[n]; dv[q] = D6[n];
        }
      }
#pragma unroll
      for (int q = 0; q < kVec6PerThread; ++q) {
        const int n = n0 + q * kNodeBlock;
        if (n < m.nn) {
          D6[n] = fmaf(alpha[r], pv[q], dv[q]);
          const float rr = fmaf(-alpha[r], av[q], rv[q]);
          const float zj = kd[q][d] * rr;
          const float z = ksm[q][d] * rr;
          R6[n] = rr;
          Z6[n] = z;
          acc[r] = fmaf(zj, zj, acc[r]);
          acc[6 + r] = fmaf(rr, z, acc[6 + r]);
        }
      }
    }
  }
  double tot[12];
  if (grid_sum_f<12>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    Cg6State *c = I.cg6;
    c->its += 1;
    int all = 1;
    for (int r = 0; r < 6; ++r) {
      if (!c->done[r]) {
        c->pnorm[r] = sqrt(tot[r]);
        if (!mg) {
          c->beta[r] = tot[6 + r] / c->rz[r];
          c->rz[r] = tot[6 + r];
        }
        c->done[r] = !(c->its < c->max_its) || c->pnorm[r] < c->min_err || c->pnorm[r] < c->pnorm0[r] * c->rel_err ||
                     !isfinite(tot[r]);
      }
      all &= c->done[r];
    }
    c->all_done = all;
    if (all) I.out->cg6_its = c->its;
  }
}

// P = Z + beta P for the right-hand sides still iterating, element-wise: block b of an instance handles
// component c = b / nchunk of node chunk b % nchunk.
__global__ void __launch_bounds__(kNodeBlock) k_cg6_pupdate(MeshDev m, const Inst *insts, const int *list,
                                                            unsigned int *active_count) {
  const Inst &I = insts[list[blockIdx.y]];
  const Cg6State *cs = I.cg6;
  if (cs->all_done) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(active_count, 1u);
  const int nchunk = (m.nn + kVec6Chunk - 1) / kVec6Chunk;
  const int c = blockIdx.x / nchunk, chunk = blockIdx.x - c * nchunk, r = c / 3;
  if (cs->done[r]) return;
  const float beta = (float)cs->beta[r];
  const size_t off = (size_t)c * m.np;
  float *__restrict__ P6 = I.P6 + off;
  const float *__restrict__ Z6 = I.Z6 + off;
  const int n0 = chunk * kVec6Chunk + threadIdx.x;
  float pv[kVec6PerThread], zv[kVec6PerThread];
#pragma unroll
  for (int q = 0; q < kVec6PerThread; ++q) {
    const int n = n0 + q * kNodeBlock;
    if (n < m.nn) {
      pv[q] = P6[n];
      zv[q] = Z6[n];
    }
  }
#pragma unroll
  for (int q = 0; q < kVec6PerThread; ++q) {
    const int n = n0 + q * kNodeBlock;
    if (n < m.nn) P6[n] = fmaf(beta, pv[q], zv[q]);
  }
}

// X += D (double-float accumulation of the FP32 correction), one thread per node.
__global__ void k_t6_accumulate(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const size_t np = m.np;
  float *__restrict__ Xh = I.X6h;
  float *__restrict__ Xl = I.X6l;
  const float *__restrict__ D6 = I.D6;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < m.nn; n += gridDim.x * blockDim.x)
#pragma unroll
    for (int c = 0; c < 18; ++c) {
      const size_t idx = (size_t)c * np + n;
      float h = Xh[idx], l = Xl[idx];
      df_add(h, l, D6[idx]);
      Xh[idx] = h;
      Xl[idx] = l;
    }
}

// ctan in the energy form, element by element (FP32 Jacobian assembled by node gather: elastic and damage
// phases, a symmetric tangent).  With v_i = w_i + x_i the tangent field of unit strain i (w_i the boundary lift,
// x_i the interior solution X6h + X6l),
//   ctan[k][i] = (1/V) sum_e sum_g wg eps(v_k)^T C_g eps(v_i),
// C_g the Gauss-point tangent: the phase's elastic C, or for damage a C + c s s^T from the tangent terms the
// residual kernel wrote.  The form is stationary at the exact x, so its error is quadratic in the error of x (the FP32
// solves and the FP32 rounding of the assembled tangent they used).  Summing element energies also avoids the
// cancellation of v^T (K v) over assembled rows -- K v nearly vanishes on interior rows -- whose first-order
// rounding with FP32 rows reached 1e-5 on 60^3 RVEs.  Block: kEnElems elements x 8 threads.  Thread a of an
// element loads node a's six fields as double-float pairs (boundary nodes: the lift of the split coordinates)
// and keeps their differences from node 0 in FP32 (the strains need only differences: sum_a dN_a = 0); then,
// as Gauss point g, it forms the six strains, the tangent products and the 21 energies.  FP32 per element,
// FP64 across elements.
constexpr int kEnElems = 32;
constexpr int kEnStride = 7 * 18 + 1;  // differences of nodes 1..7, 6 fields x 3; odd stride

__global__ void __launch_bounds__(kEnElems * 8) k_ctan_energy(MeshDev m, Mats mats, const int8_t *etype,
                                                             const float *dsh_g, const Inst *insts, const int *list) {
  __shared__ float dv[kEnElems * kEnStride];
  __shared__ float dsh[8 * 24];
  for (int t = threadIdx.x; t < 192; t += blockDim.x) dsh[t] = dsh_g[t];
  const Inst &I = insts[list[blockIdx.y]];
  const int el = threadIdx.x >> 3, sub = threadIdx.x & 7;  // sub: the node (loads), then the Gauss point
  const int e = blockIdx.x * kEnElems + el;
  const bool valid = e < m.nelem;
  const size_t np = m.np;
  float vh[18], vl[18];  // the node's six fields as double-float pairs
#pragma unroll
  for (int q = 0; q < 18; ++q) vh[q] = vl[q] = 0.f;
  if (valid) {
    const int ex = e % m.nex, ey = (e / m.nex) % m.ney, ez = e / (m.nex * m.ney);
    const int n = (ez + c_corner6[sub][2]) * m.nxny + (ey + c_corner6[sub][1]) * m.nx + ex + c_corner6[sub][0];
    int bi, bj, bk;
    if (bnd(m, n, bi, bj, bk)) {
      double X[3];
      bc_coords(m, bi, bj, bk, X);
      float ch[3], cl[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) df_split(X[d], ch[d], cl[d]);
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        float wh[3], wl[3];
        lift_df(ch, cl, r, wh, wl);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          vh[r * 3 + d] = wh[d];
          vl[r * 3 + d] = wl[d];
        }
      }
    } else {
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          vh[r * 3 + d] = I.X6h[c6(r, d, np) + n];
          vl[r * 3 + d] = I.X6l[c6(r, d, np) + n];
        }
    }
  }
  const int lane0 = (threadIdx.x & 31) & ~7;  // node 0 of this element, in the same warp
#pragma unroll
  for (int q = 0; q < 18; ++q) {
    const float h0 = __shfl_sync(0xffffffffu, vh[q], lane0), l0 = __shfl_sync(0xffffffffu, vl[q], lane0);
    if (sub > 0)
      dv[el * kEnStride + (sub - 1) * 18 + q] = __fadd_rn(__fsub_rn(vh[q], h0), __fsub_rn(vl[q], l0));
  }
  __syncthreads();
  float acc[21];
#pragma unroll
  for (int q = 0; q < 21; ++q) acc[q] = 0.f;
  if (valid) {
    const float *dg = dsh + sub * 24;
    const float *dve = dv + el * kEnStride;
    float eps[6][6];
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int c = 0; c < 6; ++c) eps[r][c] = 0.f;
#pragma unroll
    for (int a = 1; a < 8; ++a) {
      const float gx = dg[a * 3], gy = dg[a * 3 + 1], gz = dg[a * 3 + 2];
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        const float ux = dve[(a - 1) * 18 + r * 3], uy = dve[(a - 1) * 18 + r * 3 + 1],
                    uz = dve[(a - 1) * 18 + r * 3 + 2];
        eps[r][0] = fmaf(gx, ux, eps[r][0]);
        eps[r][1] = fmaf(gy, uy, eps[r][1]);
        eps[r][2] = fmaf(gz, uz, eps[r][2]);
        eps[r][3] = fmaf(gy, ux, fmaf(gx, uy, eps[r][3]));
        eps[r][4] = fmaf(gz, ux, fmaf(gx, uz, eps[r][4]));
        eps[r][5] = fmaf(gz, uy, fmaf(gy, uz, eps[r][5]));
      }
    }
    const MatDev &md = mats.m[etype[e]];
    float ta = 1.f, tc = 0.f, s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (md.type == 2) {
      const size_t st = (size_t)8 * m.nelem, o = (size_t)sub * m.nelem + e;
      ta = I.gpd[o];
      tc = I.gpd[st + o];
#pragma unroll
      for (int q = 0; q < 6; ++q) s[q] = I.gpd[(2 + q) * st + o];
    }
    const float lam = (float)md.lambda, mu = (float)md.mu, w = (float)m.wg;
    float sig[6][6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      const float tr = eps[r][0] + eps[r][1] + eps[r][2];
      float se = 0.f;
#pragma unroll
      for (int q = 0; q < 6; ++q) se = fmaf(s[q], eps[r][q], se);
      se *= tc;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const float el_q = (q < 3) ? lam * tr + 2.f * mu * eps[r][q] : mu * eps[r][q];
        sig[r][q] = fmaf(ta, el_q, se * s[q]);
      }
    }
    int q = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
      for (int i = k; i < 6; ++i) {
        float en = 0.f;
#pragma unroll
        for (int c = 0; c < 6; ++c) en = fmaf(eps[i][c], sig[k][c], en);
        acc[q++] = w * en;
      }
  }
  double tot[21];
  if (grid_sum_f<21>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    bool bad = false;
    int q = 0;
    for (int k = 0; k < 6; ++k)
      for (int i = k; i < 6; ++i) {
        const double c = tot[q++] / m.vol_tot;
        I.out->ctan[k * 6 + i] = c;
        I.out->ctan[i * 6 + k] = c;
        bad |= !isfinite(c);
      }
    if (bad) I.out->nonfinite = 1;
  }
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
    const size_t np = m.np;
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
        const size_t i0 = c6(r, 0, np) + nodes[a], i1 = c6(r, 1, np) + nodes[a], i2 = c6(r, 2, np) + nodes[a];
        double ux = (double)I.X6h[i0] + (double)I.X6l[i0], uy = (double)I.X6h[i1] + (double)I.X6l[i1],
               uz = (double)I.X6h[i2] + (double)I.X6l[i2];
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

// CG state of the listed instances at the start of a solve (what the host writes before an uncaptured solve):
// relative tolerance rel_tol[a] for the a-th listed instance, abs_tol, max_its, everything else zero.
__global__ void k_cg32_init(const Inst *insts, const int *list, int nlist, const double *rel_tol, double abs_tol,
                            int max_its) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nlist) return;
  CgState c{};
  c.min_err = abs_tol;
  c.rel_err = rel_tol[a];
  c.max_its = max_its;
  *insts[list[a]].cg = c;
}

__global__ void k_zero_u32(unsigned int *p) { *p = 0u; }

// Condition of the WHILE node of a captured CG solve: another chunk of iterations runs while some instance of
// the batch still iterates (the count of the chunk's last p-update) and fewer than `cap` chunks have run.  The
// CG kernels stop every instance at its max_its, so the count reaches zero by itself; the cap bounds the loop
// all the same.
__global__ void k_cg_continue(cudaGraphConditionalHandle h, const unsigned int *count, unsigned int *chunks,
                              unsigned int cap) {
  const unsigned int c = *chunks + 1u;
  *chunks = c;
  cudaGraphSetConditional(h, (*count != 0u && c < cap) ? 1u : 0u);
}

}  // namespace mgb

using namespace mgb;

static inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

extern "C" {

int mgb_launch_cg32_init(const Inst *insts, const int *list, int nlist, const double *rel_tol, double abs_tol,
                         int max_its, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg32_init<<<cdiv(nlist, 128), 128, 0, s>>>(insts, list, nlist, rel_tol, abs_tol, max_its);
  return (int)cudaGetLastError();
}

int mgb_launch_zero_u32(unsigned int *p, cudaStream_t s) {
  k_zero_u32<<<1, 1, 0, s>>>(p);
  return (int)cudaGetLastError();
}

int mgb_launch_cg_continue(cudaGraphConditionalHandle h, const unsigned int *count, unsigned int *chunks,
                           unsigned int cap, cudaStream_t s) {
  k_cg_continue<<<1, 1, 0, s>>>(h, count, chunks, cap);
  return (int)cudaGetLastError();
}

int mgb_launch_cg32_setup(const MeshDev *m, const Inst *insts, const int *list, int nlist, int mg, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg32_setup<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list, mg);
  return (int)cudaGetLastError();
}

int mgb_launch_cg32_spmv(const MeshDev *m, const Inst *insts, const int *list, int nlist, int block,
                         cudaStream_t s) {
  if (nlist <= 0) return 0;
  const size_t units = cdiv(m->nn, kSpmvNodes);
  if (block == 64)
    k_cg32_spmv<64><<<dim3(cdiv(units, 64), nlist), 64, 0, s>>>(*m, insts, list);
  else if (block == 256)
    k_cg32_spmv<256><<<dim3(cdiv(units, 256), nlist), 256, 0, s>>>(*m, insts, list);
  else
    k_cg32_spmv<128><<<dim3(cdiv(units, 128), nlist), 128, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_cg32_update(const MeshDev *m, const Inst *insts, const int *list, int nlist, int mg, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const unsigned g = cdiv((size_t)m->nn * 3, (size_t)kRowsPerThread * kNodeBlock);
  k_cg32_update<<<dim3(g, nlist), kNodeBlock, 0, s>>>(*m, insts, list, mg);
  return (int)cudaGetLastError();
}

int mgb_launch_cg32_pupdate(const MeshDev *m, const Inst *insts, const int *list, int nlist,
                            unsigned int *active_count, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const unsigned g = cdiv((size_t)m->nn * 3, (size_t)kRowsPerThread * kNodeBlock);
  k_cg32_pupdate<<<dim3(g, nlist), kNodeBlock, 0, s>>>(*m, insts, list, active_count);
  return (int)cudaGetLastError();
}

int mgb_launch_add_du32(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const int nndim = m->nn * 3;
  k_add_du32<<<dim3(cdiv(nndim, 4 * kNodeBlock), nlist), kNodeBlock, 0, s>>>(nndim, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_axpy_du32(const MeshDev *m, double *u, const float *du, double a, cudaStream_t s) {
  const int nndim = m->nn * 3;
  k_axpy_du32<<<cdiv(nndim, 4 * kNodeBlock), kNodeBlock, 0, s>>>(nndim, u, du, a);
  return (int)cudaGetLastError();
}

int mgb_launch_t6_rhs(const MeshDev *m, const int *near, int nnear, const Inst *insts, const int *list, int nlist,
                      cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_t6_clear<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  const int e = (int)cudaGetLastError();
  if (e) return e;
  // at least one block, which publishes ||f_i|| = 0 when no interior node touches the boundary
  const int nb = nnear > 0 ? cdiv(nnear, kNodeBlock) : 1;
  k_t6_rhs_near<<<dim3(nb, nlist), kNodeBlock, 0, s>>>(*m, near, nnear, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_t6_residual(const MeshDev *m, const Inst *insts, const int *list, int nlist, int x_zero, int mg,
                           cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_t6_residual<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list, x_zero, mg);
  return (int)cudaGetLastError();
}

int mgb_launch_cg6_spmv(const MeshDev *m, const Inst *insts, const int *list, int nlist, int block, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const size_t units = cdiv(m->nn, kSpmv6Nodes);
  if (block == 64)
    k_cg6_spmv<64><<<dim3(cdiv(units, 64), nlist), 64, 0, s>>>(*m, insts, list);
  else if (block == 256)
    k_cg6_spmv<256><<<dim3(cdiv(units, 256), nlist), 256, 0, s>>>(*m, insts, list);
  else
    k_cg6_spmv<128><<<dim3(cdiv(units, 128), nlist), 128, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_cg6_update(const MeshDev *m, const Inst *insts, const int *list, int nlist, int mg, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg6_update<<<dim3(cdiv(m->nn, kVec6Chunk), nlist), kNodeBlock, 0, s>>>(*m, insts, list, mg);
  return (int)cudaGetLastError();
}

int mgb_launch_cg6_pupdate(const MeshDev *m, const Inst *insts, const int *list, int nlist,
                           unsigned int *active_count, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_cg6_pupdate<<<dim3(18 * cdiv(m->nn, kVec6Chunk), nlist), kNodeBlock, 0, s>>>(*m, insts, list, active_count);
  return (int)cudaGetLastError();
}

int mgb_launch_t6_accumulate(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_t6_accumulate<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_ctan_energy(const MeshDev *m, const Mats *mats, const int8_t *etype, const float *dsh32,
                           const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_ctan_energy<<<dim3(cdiv(m->nelem, kEnElems), nlist), kEnElems * 8, 0, s>>>(*m, *mats, etype, dsh32, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_ctan_avg(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh, const Inst *insts,
                        const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_ctan_avg<<<dim3(cdiv((size_t)m->nelem * 8, 128), nlist), 128, 0, s>>>(*m, *mats, etype, dsh, insts, list);
  return (int)cudaGetLastError();
}

}  // extern "C"
