// adjoint_kernels.cu -- the adjoint (reverse-mode) pass of a load path on the GPU (FP64).
//
// Step n of a path solves R(u_n; h_{n-1}, theta) = sum_gp w B^T sigma = 0 on the interior rows, with u_n on
// the boundary given by the macro strain eps_n, and updates the history h_n = H(B u_n, h_{n-1}, theta).  For
// L = sum_n g_n . sigma_bar_n, going backwards with mu_n = dL/dh_n (mu_N = 0):
//   K_n^T lambda_n = sum_gp B^T [ (w/V) C^T g_n + H_eps^T mu_n ]                (interior rows; k_adj_rhs)
//   a_gp = (w/V) g_n - w B lambda_n
//   mu_{n-1} = sigma_h^T a + H_h^T mu_n,   dL/dtheta += sigma_theta^T a + H_theta^T mu_n,
//   dL/deps_n,i = sum_gp (C^T a + H_eps^T mu_n) . B w_i                           (k_adj_back)
// with C = d sigma / d eps and the other Jacobians of the law taken column by column with forward-mode dual
// numbers (adjoint_laws.h).  K^T lambda = rhs is solved by Jacobi-preconditioned BiCGSTAB on the transpose of
// the stencil ELL (the reference's J2 tangent is not symmetric in its Voigt convention).
#include <cuda_runtime.h>

#include "adjoint_laws.h"
#include "bc.cuh"
#include "device.cuh"
#include "launch.h"
#include "reduce.cuh"

namespace mgb {

namespace {

__device__ __constant__ int c_cornerA[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                              {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

// B v for the nodal vector v_e (24) at Gauss point gradients dg (8 x 3), Voigt order xx,yy,zz,xy,xz,yz.
__device__ __forceinline__ void strain_of(const double *dg, const double *ve, double *e) {
  double e0 = 0, e1 = 0, e2 = 0, e3 = 0, e4 = 0, e5 = 0;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double gx = dg[a * 3], gy = dg[a * 3 + 1], gz = dg[a * 3 + 2];
    const double ux = ve[a * 3], uy = ve[a * 3 + 1], uz = ve[a * 3 + 2];
    e0 += gx * ux; e1 += gy * uy; e2 += gz * uz;
    e3 += gy * ux + gx * uy;
    e4 += gz * ux + gx * uz;
    e5 += gz * uy + gy * uz;
  }
  e[0] = e0; e[1] = e1; e[2] = e2; e[3] = e3; e[4] = e4; e[5] = e5;
}

__device__ __forceinline__ void element_nodes(const MeshDev &m, int e, int *nodes) {
  const int ex = e % m.nex, ey = (e / m.nex) % m.ney, ez = e / (m.nex * m.ney);
  const int n0 = ez * m.nxny + ey * m.nx + ex;
#pragma unroll
  for (int a = 0; a < 8; ++a) nodes[a] = n0 + c_cornerA[a][2] * m.nxny + c_cornerA[a][1] * m.nx + c_cornerA[a][0];
}

__device__ __forceinline__ void theta_of(const MatDev &md, double *th) {
  th[0] = md.E; th[1] = md.nu; th[2] = md.Xt; th[3] = md.Sy; th[4] = md.Ka;
}

}  // namespace

// Right-hand side of the adjoint system of one step: element blocks -sum_gp B^T rho (the node gather negates
// them into b and zeroes the Dirichlet rows), rho = (w/V) C^T g + H_eps^T mu.
__global__ void __launch_bounds__(kElemBlock) k_adj_rhs(MeshDev m, Mats mats, const int8_t *etype, const double *dsh_g,
                                                        const Inst *insts, const int *list, AdjStep st) {
  __shared__ double dsh[8 * 24];
  for (int t = threadIdx.x; t < 192; t += blockDim.x) dsh[t] = dsh_g[t];
  __syncthreads();
  const Inst &I = insts[list[blockIdx.y]];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelem) return;
  int nodes[8];
  element_nodes(m, e, nodes);
  double ue[24], be[24];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int d = 0; d < 3; ++d) ue[a * 3 + d] = I.u[nodes[a] * 3 + d];
#pragma unroll
  for (int q = 0; q < 24; ++q) be[q] = 0.0;
  const MatDev &md = mats.m[etype[e]];
  double th[adj::kNpar];
  theta_of(md, th);
#pragma unroll 1
  for (int g = 0; g < 8; ++g) {
    const double *dg = &dsh[g * 24];
    double eps[6], h[7], mu[7], rho[6], ds[6], dh[7];
    strain_of(dg, ue, eps);
    const size_t gp = (size_t)e * 8 + g;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      h[k] = I.vars_old ? I.vars_old[gp * kNvarGp + k] : 0.0;
      mu[k] = st.mu_in ? st.mu_in[gp * kNvarGp + k] : 0.0;
    }
#pragma unroll 1
    for (int j = 0; j < 6; ++j) {
      adj::law_column(md.type, th, eps, h, j, ds, dh);
      double c = 0.0;
#pragma unroll
      for (int i = 0; i < 6; ++i) c += st.wgv * st.g[i] * ds[i];
#pragma unroll
      for (int k = 0; k < 7; ++k) c += mu[k] * dh[k];
      rho[j] = c;
    }
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const double gx = dg[a * 3], gy = dg[a * 3 + 1], gz = dg[a * 3 + 2];
      be[a * 3 + 0] -= gx * rho[0] + gy * rho[3] + gz * rho[4];
      be[a * 3 + 1] -= gy * rho[1] + gx * rho[3] + gz * rho[5];
      be[a * 3 + 2] -= gz * rho[2] + gx * rho[4] + gy * rho[5];
    }
  }
#pragma unroll
  for (int q = 0; q < 24; ++q) I.be[(size_t)q * m.nelem + e] = be[q];
}

// Backward step at the Gauss points (see the file comment): mu_{n-1}, and the sums of dL/dtheta and dL/deps_n.
__global__ void __launch_bounds__(kElemBlock) k_adj_back(MeshDev m, Mats mats, const int8_t *etype, const double *dsh_g,
                                                         const Inst *insts, const int *list, AdjStep st) {
  __shared__ double dsh[8 * 24];
  for (int t = threadIdx.x; t < 192; t += blockDim.x) dsh[t] = dsh_g[t];
  __syncthreads();
  const Inst &I = insts[list[blockIdx.y]];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[21];
#pragma unroll
  for (int q = 0; q < 21; ++q) acc[q] = 0.0;
  if (e < m.nelem) {
    int nodes[8];
    element_nodes(m, e, nodes);
    double ue[24], le[24], cc[8][3];
    bool onb[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        ue[a * 3 + d] = I.u[nodes[a] * 3 + d];
        le[a * 3 + d] = st.lam[nodes[a] * 3 + d];
      }
      int bi, bj, bk;
      onb[a] = bnd(m, nodes[a], bi, bj, bk);
      if (onb[a]) bc_coords(m, bi, bj, bk, cc[a]);
    }
    const int ph = etype[e];
    const MatDev &md = mats.m[ph];
    double th[adj::kNpar];
    theta_of(md, th);
#pragma unroll 1
    for (int g = 0; g < 8; ++g) {
      const double *dg = &dsh[g * 24];
      double eps[6], bl[6], av[6], h[7], mu[7], rho[6], ds[6], dh[7];
      strain_of(dg, ue, eps);
      strain_of(dg, le, bl);
#pragma unroll
      for (int i = 0; i < 6; ++i) av[i] = st.wgv * st.g[i] - m.wg * bl[i];
      const size_t gp = (size_t)e * 8 + g;
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        h[k] = I.vars_old ? I.vars_old[gp * kNvarGp + k] : 0.0;
        mu[k] = st.mu_in ? st.mu_in[gp * kNvarGp + k] : 0.0;
      }
#pragma unroll 1
      for (int j = 0; j < adj::kNdir; ++j) {
        adj::law_column(md.type, th, eps, h, j, ds, dh);
        double c = 0.0;
#pragma unroll
        for (int i = 0; i < 6; ++i) c += av[i] * ds[i];
#pragma unroll
        for (int k = 0; k < 7; ++k) c += mu[k] * dh[k];
        if (j < 6)
          rho[j] = c;
        else if (j < 13)
          st.mu_out[gp * kNvarGp + (j - 6)] = c;
        else
          acc[ph * adj::kNpar + (j - 13)] += c;
      }
      // dL/deps_n,i: rho . B w_i, w_i = the boundary field of the unit strain e_i (zero on interior nodes)
#pragma unroll 1
      for (int i = 0; i < 6; ++i) {
        double we[24];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
          double w[3] = {0.0, 0.0, 0.0};
          if (onb[a]) lift(cc[a], i, w);
          we[a * 3] = w[0]; we[a * 3 + 1] = w[1]; we[a * 3 + 2] = w[2];
        }
        double bw[6];
        strain_of(dg, we, bw);
        double c = 0.0;
#pragma unroll
        for (int v = 0; v < 6; ++v) c += rho[v] * bw[v];
        acc[15 + i] += c;
      }
    }
  }
  double tot[21];
  if (grid_sum<21>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0)
    for (int q = 0; q < 21; ++q) st.out[q] = tot[q];
}

// u += deps . X at every node (the affine field of a macro strain increment, engineering shear): the
// predictor of a path step, so that Newton starts from the previous solution moved with the increment.
__global__ void __launch_bounds__(kNodeBlock) k_affine_add(MeshDev m, double *u, Voigt6 de) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  const int i = n % m.nx, j = (n / m.nx) % m.ny, k = n / m.nxny;
  const double x[3] = {i * m.dx, j * m.dy, k * m.dz};
  const double e[3][3] = {{de.v[0], 0.5 * de.v[3], 0.5 * de.v[4]},
                          {0.5 * de.v[3], de.v[1], 0.5 * de.v[5]},
                          {0.5 * de.v[4], 0.5 * de.v[5], de.v[2]}};
#pragma unroll
  for (int a = 0; a < 3; ++a) u[n * 3 + a] += e[a][0] * x[0] + e[a][1] * x[1] + e[a][2] * x[2];
}

// x += a y over n entries (the step length of the path's line search).
__global__ void k_axpy(int n, double *x, const double *y, double a) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) x[t] += a * y[t];
}

// ---------------------------------------------------------------------------------------------------
// BiCGSTAB on K or K^T (interior rows; Dirichlet rows are identity rows and stay zero), Jacobi preconditioner:
// the path's Newton corrections (K) and its adjoint systems (K^T); the reference's J2 tangent is not symmetric.

// (K x)_n, or (K^T x)_n when Transpose: the block of K^T at (n, m) is the transpose of K's block at (m, n),
// stored in row m at the mirrored stencil slot 26 - s.
template <bool Transpose>
__device__ __forceinline__ void spmv_node(const MeshDev &m, const double *__restrict__ vals,
                                          const double *__restrict__ x, int n, double y[3]) {
  y[0] = y[1] = y[2] = 0.0;
  const size_t np = m.np;
#pragma unroll 1
  for (int s = 0; s < 27; ++s) {
    const int nb = n + (s / 9 - 1) * m.nxny + ((s / 3) % 3 - 1) * m.nx + (s % 3 - 1);
    const double x0 = x[nb * 3], x1 = x[nb * 3 + 1], x2 = x[nb * 3 + 2];
    if (Transpose) {
      const double *v = vals + (size_t)((26 - s) * 9) * np + nb;
#pragma unroll
      for (int fi = 0; fi < 3; ++fi)
        y[fi] += v[(0 * 3 + fi) * np] * x0 + v[(1 * 3 + fi) * np] * x1 + v[(2 * 3 + fi) * np] * x2;
    } else {
      const double *v = vals + (size_t)(s * 9) * np + n;
#pragma unroll
      for (int fi = 0; fi < 3; ++fi)
        y[fi] += v[(fi * 3 + 0) * np] * x0 + v[(fi * 3 + 1) * np] * x1 + v[(fi * 3 + 2) * np] * x2;
    }
  }
}

__global__ void __launch_bounds__(kNodeBlock) k_bicg_init(MeshDev m, AdjDev A) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[1] = {0.0};
  if (n < m.nn) {
    int i, j, k;
    const bool b = bnd(m, n, i, j, k);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int row = n * 3 + d;
      const double r = b ? 0.0 : A.b[row];
      A.kinv[row] = b ? 1.0 : 1.0 / A.vals[(size_t)(13 * 9 + d * 3 + d) * m.np + n];
      A.x[row] = 0.0; A.r[row] = r; A.rh[row] = r; A.p[row] = 0.0; A.v[row] = 0.0;
      acc[0] += r * r;
    }
  }
  double tot[1];
  if (grid_sum<1>(acc, A.red, A.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    BicgState *s = A.st;
    s->rho = tot[0];  // (rh, r) with rh = r
    s->rho_old = 1.0;
    s->alpha = 1.0;
    s->omega = 1.0;
    s->beta = 0.0;
    s->r0 = sqrt(tot[0]);
    s->rnorm = s->r0;
    s->its = 0;
    s->converged = !(s->r0 > 0.0);
    s->done = s->converged || !isfinite(tot[0]);
  }
}

// p = r + beta (p - omega v); y = kinv p
__global__ void __launch_bounds__(kNodeBlock) k_bicg_p(MeshDev m, AdjDev A) {
  const BicgState *s = A.st;
  if (s->done) return;
  const double beta = s->beta, omega = s->omega;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < 3 * m.nn; row += gridDim.x * blockDim.x) {
    const double p = A.r[row] + beta * (A.p[row] - omega * A.v[row]);
    A.p[row] = p;
    A.y[row] = A.kinv[row] * p;
  }
}

// v = K y (K^T y); alpha = rho / (rh . v)
template <bool Transpose>
__global__ void __launch_bounds__(kNodeBlock) k_bicg_v(MeshDev m, AdjDev A) {
  const BicgState *s = A.st;
  if (s->done) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[1] = {0.0};
  if (n < m.nn) {
    int i, j, k;
    double y[3];
    if (bnd(m, n, i, j, k)) {
      y[0] = A.y[n * 3]; y[1] = A.y[n * 3 + 1]; y[2] = A.y[n * 3 + 2];
    } else {
      spmv_node<Transpose>(m, A.vals, A.y, n, y);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      A.v[n * 3 + d] = y[d];
      acc[0] += A.rh[n * 3 + d] * y[d];
    }
  }
  double tot[1];
  if (grid_sum<1>(acc, A.red, A.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    BicgState *w = A.st;
    w->alpha = w->rho / tot[0];
    if (!isfinite(w->alpha) || tot[0] == 0.0) w->done = 1;
  }
}

// x += alpha y; s = r - alpha v; z = kinv s
__global__ void __launch_bounds__(kNodeBlock) k_bicg_s(MeshDev m, AdjDev A) {
  const BicgState *st = A.st;
  if (st->done) return;
  const double alpha = st->alpha;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < 3 * m.nn; row += gridDim.x * blockDim.x) {
    A.x[row] += alpha * A.y[row];
    const double sv = A.r[row] - alpha * A.v[row];
    A.s[row] = sv;
    A.z[row] = A.kinv[row] * sv;
  }
}

// t = K z (K^T z); omega = (t . s) / (t . t)
template <bool Transpose>
__global__ void __launch_bounds__(kNodeBlock) k_bicg_t(MeshDev m, AdjDev A) {
  const BicgState *s = A.st;
  if (s->done) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[2] = {0.0, 0.0};
  if (n < m.nn) {
    int i, j, k;
    double t[3];
    if (bnd(m, n, i, j, k)) {
      t[0] = A.z[n * 3]; t[1] = A.z[n * 3 + 1]; t[2] = A.z[n * 3 + 2];
    } else {
      spmv_node<Transpose>(m, A.vals, A.z, n, t);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      A.t[n * 3 + d] = t[d];
      acc[0] += t[d] * A.s[n * 3 + d];
      acc[1] += t[d] * t[d];
    }
  }
  double tot[2];
  if (grid_sum<2>(acc, A.red, A.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    BicgState *w = A.st;
    w->omega = tot[0] / tot[1];
    if (!isfinite(w->omega) || tot[1] == 0.0) w->done = 1;
  }
}

// x += omega z; r = s - omega t; rho_new = rh . r; beta; convergence on |r| <= rel_tol |r0|
__global__ void __launch_bounds__(kNodeBlock) k_bicg_r(MeshDev m, AdjDev A, unsigned int *active) {
  const BicgState *st = A.st;
  if (st->done) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(active, 1u);
  const double omega = st->omega;
  double acc[2] = {0.0, 0.0};
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < 3 * m.nn; row += gridDim.x * blockDim.x) {
    A.x[row] += omega * A.z[row];
    const double r = A.s[row] - omega * A.t[row];
    A.r[row] = r;
    acc[0] += A.rh[row] * r;
    acc[1] += r * r;
  }
  double tot[2];
  if (grid_sum<2>(acc, A.red, A.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    BicgState *w = A.st;
    w->rho_old = w->rho;
    w->rho = tot[0];
    w->beta = (w->rho / w->rho_old) * (w->alpha / w->omega);
    w->rnorm = sqrt(tot[1]);
    w->its += 1;
    w->converged = w->rnorm <= w->rel_tol * w->r0;
    w->done = w->converged || !(w->its < w->max_its) || !isfinite(tot[1]) || w->rho == 0.0;
  }
}

}  // namespace mgb

using namespace mgb;

static inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

extern "C" {

int mgb_launch_adj_rhs(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh, const Inst *insts,
                       const int *list, const AdjStep *st, cudaStream_t s) {
  k_adj_rhs<<<dim3(cdiv(m->nelem, kElemBlock), 1), kElemBlock, 0, s>>>(*m, *mats, etype, dsh, insts, list, *st);
  return (int)cudaGetLastError();
}

int mgb_launch_adj_back(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh, const Inst *insts,
                        const int *list, const AdjStep *st, cudaStream_t s) {
  k_adj_back<<<dim3(cdiv(m->nelem, kElemBlock), 1), kElemBlock, 0, s>>>(*m, *mats, etype, dsh, insts, list, *st);
  return (int)cudaGetLastError();
}

int mgb_launch_affine_add(const MeshDev *m, double *u, const double *deps, cudaStream_t s) {
  Voigt6 de;
  for (int q = 0; q < 6; ++q) de.v[q] = deps[q];
  k_affine_add<<<cdiv(m->nn, kNodeBlock), kNodeBlock, 0, s>>>(*m, u, de);
  return (int)cudaGetLastError();
}

int mgb_launch_axpy(int n, double *x, const double *y, double a, cudaStream_t s) {
  k_axpy<<<cdiv(n, 4 * kNodeBlock), kNodeBlock, 0, s>>>(n, x, y, a);
  return (int)cudaGetLastError();
}

int mgb_launch_bicg_init(const MeshDev *m, const AdjDev *A, cudaStream_t s) {
  k_bicg_init<<<cdiv(m->nn, kNodeBlock), kNodeBlock, 0, s>>>(*m, *A);
  return (int)cudaGetLastError();
}

// One BiCGSTAB iteration (5 launches) on K (transpose = 0) or K^T; `active` receives +1 while the solve is
// still iterating.
int mgb_launch_bicg_iter(const MeshDev *m, const AdjDev *A, unsigned int *active, int transpose, cudaStream_t s) {
  const unsigned gr = cdiv((size_t)3 * m->nn, 4 * kNodeBlock), gn = cdiv(m->nn, kNodeBlock);
  k_bicg_p<<<gr, kNodeBlock, 0, s>>>(*m, *A);
  if (transpose)
    k_bicg_v<true><<<gn, kNodeBlock, 0, s>>>(*m, *A);
  else
    k_bicg_v<false><<<gn, kNodeBlock, 0, s>>>(*m, *A);
  k_bicg_s<<<gr, kNodeBlock, 0, s>>>(*m, *A);
  if (transpose)
    k_bicg_t<true><<<gn, kNodeBlock, 0, s>>>(*m, *A);
  else
    k_bicg_t<false><<<gn, kNodeBlock, 0, s>>>(*m, *A);
  k_bicg_r<<<gr, kNodeBlock, 0, s>>>(*m, *A, active);
  return (int)cudaGetLastError();
}

}  // extern "C"
