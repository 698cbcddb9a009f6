// fe_kernels.cu -- finite-element kernels of the homogenization path (sm_103a): the FP64 form's residual and
// colour-ordered assembly, the mixed form's double-float residual and FP32 assemblies, the history update.
//
// Every kernel runs over a batch: blockIdx.y indexes the list of active instances, blockIdx.x tiles the
// nodes or elements of one RVE.  Summation orders follow the reference where a sum is local (Gauss points of
// an element, elements around a node); only grid-wide reductions use a tree.
#include <cuda_runtime.h>

#include "device.cuh"
#include "df.cuh"
#include "elem_df.cuh"
#include "launch.h"
#include "adjoint_laws.h"
#include "hex_sumfact.h"
#include "laws.cuh"
#include "reduce.cuh"

namespace mgb {

// Local hex8 corner (ox,oy,oz) -> local node index (common.cpp:28-40 numbering).
__device__ __forceinline__ int local_of(int ox, int oy, int oz) { return oz * 4 + (oy ? 3 - ox : ox); }
__device__ __constant__ int c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                             {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

__device__ __forceinline__ bool is_boundary(const MeshDev &m, int i, int j, int k) {
  return i == 0 || j == 0 || k == 0 || i == m.nx - 1 || j == m.ny - 1 || k == m.nz - 1;
}

// strain = B(gp) * u_e with the non-zero terms in the reference's order (common.cpp:57-72).
// dsh: the 8 nodal gradients at this Gauss point, dsh[a*3 + d].
__device__ __forceinline__ void gp_strain(const double *dsh, const double *ue, double *eps) {
  double e0 = 0, e1 = 0, e2 = 0, e3 = 0, e4 = 0, e5 = 0;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const double gx = dsh[a * 3], gy = dsh[a * 3 + 1], gz = dsh[a * 3 + 2];
    const double ux = ue[a * 3], uy = ue[a * 3 + 1], uz = ue[a * 3 + 2];
    e0 += gx * ux;
    e1 += gy * uy;
    e2 += gz * uz;
    e3 += gy * ux;
    e3 += gx * uy;
    e4 += gz * ux;
    e4 += gx * uz;
    e5 += gz * uy;
    e5 += gy * uz;
  }
  eps[0] = e0; eps[1] = e1; eps[2] = e2; eps[3] = e3; eps[4] = e4; eps[5] = e5;
}

// ---------------------------------------------------------------------------------------------------
// Affine displacement boundary condition u = eps_t x on the six faces (micro3D.cpp:26-78).  A node on
// several faces takes the coordinates of the last face written by the reference (x=lx, then x=0, y=ly,
// y=0, z=lz, z=0 in decreasing priority).
__global__ void k_set_bc(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  const int i = n % m.nx, j = (n / m.nx) % m.ny, k = n / m.nxny;
  if (!is_boundary(m, i, j, k)) return;
  double c[3];
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
  const double e[6] = {I.strain[0], I.strain[1], I.strain[2], I.strain[3], I.strain[4], I.strain[5]};
  const double et[3][3] = {{e[0], 0.5 * e[3], 0.5 * e[4]}, {0.5 * e[3], e[1], 0.5 * e[5]}, {0.5 * e[4], 0.5 * e[5], e[2]}};
  double *__restrict__ u = I.u;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double t = 0.0;
#pragma unroll
    for (int b = 0; b < 3; ++b) t += et[a][b] * c[b];
    u[n * 3 + a] = t;
  }
}

// u += du over all unknowns (solve.cpp:73).
__global__ void k_add_du(int nndim, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  double *__restrict__ u = I.u;
  const double *__restrict__ du = I.du;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nndim; t += gridDim.x * blockDim.x) u[t] += du[t];
}

// dst = src for the listed instances; src/dst selected by `which` (0: u <- u_n, 1: u_k <- u).
__global__ void k_copy(int n, const double *const *src, double *const *dst, const int *list) {
  const int y = list[blockIdx.y];
  const double *s = src[y];
  double *d = dst[y];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) d[t] = s[t];
}

// ---------------------------------------------------------------------------------------------------
// Element residual blocks be = sum_gp B^T sigma(B u_e, vars) wg (assembly.cpp:123-138), one thread per
// element, plus the element's share of the volume average of sigma (average.cpp:57-82), reduced over the
// grid into out.sig.  Each term is formed as (g sigma) wg, the reference's order: the FP64 form's iteration
// counts match the reference's.  The mixed form uses k_elem_rhs_df (elastic and damage phases) or
// k_elem_rhs_sf (with a J2 phase).
__global__ void __launch_bounds__(kElemBlock) k_elem_rhs(MeshDev m, Mats mats, const int8_t *etype,
                                                           const double *dsh_g, const Inst *insts,
                                                           const int *list) {
  __shared__ double dsh[8 * 24];
  for (int t = threadIdx.x; t < 192; t += blockDim.x) dsh[t] = dsh_g[t];
  __syncthreads();
  const Inst &I = insts[list[blockIdx.y]];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  double aux[6] = {0, 0, 0, 0, 0, 0};
  if (e < m.nelem) {
    const int ex = e % m.nex, ey = (e / m.nex) % m.ney, ez = e / (m.nex * m.ney);
    const int n0 = ez * m.nxny + ey * m.nx + ex;
    double ue[24];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const int n = n0 + c_corner[a][2] * m.nxny + c_corner[a][1] * m.nx + c_corner[a][0];
#pragma unroll
      for (int d = 0; d < 3; ++d) ue[a * 3 + d] = I.u[n * 3 + d];
    }
    const MatDev &mat = mats.m[etype[e]];
    double be[24];
#pragma unroll
    for (int i = 0; i < 24; ++i) be[i] = 0.0;
    const double wg = m.wg;
#pragma unroll 1
    for (int g = 0; g < 8; ++g) {
      const double *dg = &dsh[g * 24];
      double eps[6], s[6];
      gp_strain(dg, ue, eps);
      const double *vg = I.vars_old ? I.vars_old + ((size_t)e * 8 + g) * kNvarGp : nullptr;
      if (mat.type == 2 && I.gpd) {
        // damage: the same stress as law_stress, plus the tangent terms for the FP32 Jacobian
        double D, ta, tc;
        law_damage_terms(mat, eps, vg, s, &D, &ta, &tc);
        float *__restrict__ gpd = I.gpd;
        const size_t st = (size_t)8 * m.nelem, o = (size_t)g * m.nelem + e;
        gpd[o] = (float)ta;
        gpd[st + o] = (float)tc;
#pragma unroll
        for (int v = 0; v < 6; ++v) gpd[(2 + v) * st + o] = (float)s[v];
        const double f = 1 - D;
#pragma unroll
        for (int v = 0; v < 6; ++v) s[v] *= f;
      } else {
        law_stress(mat, eps, vg, s);
      }
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const double gx = dg[a * 3], gy = dg[a * 3 + 1], gz = dg[a * 3 + 2];
        be[a * 3 + 0] += gx * s[0] * wg;
        be[a * 3 + 0] += gy * s[3] * wg;
        be[a * 3 + 0] += gz * s[4] * wg;
        be[a * 3 + 1] += gy * s[1] * wg;
        be[a * 3 + 1] += gx * s[3] * wg;
        be[a * 3 + 1] += gz * s[5] * wg;
        be[a * 3 + 2] += gz * s[2] * wg;
        be[a * 3 + 2] += gx * s[4] * wg;
        be[a * 3 + 2] += gy * s[5] * wg;
      }
#pragma unroll
      for (int v = 0; v < 6; ++v) aux[v] += s[v] * wg;
    }
    double *__restrict__ bev = I.be;
#pragma unroll
    for (int i = 0; i < 24; ++i) bev[(size_t)i * m.nelem + e] = be[i];
  }
  double tot[6];
  const int nb = gridDim.x;
  if (grid_sum<6>(aux, I.red, I.ticket, nb, tot) && threadIdx.x == 0) {
    bool bad = false;
#pragma unroll
    for (int v = 0; v < 6; ++v) {
      I.out->sig[v] = tot[v] / m.vol_tot;
      bad |= !isfinite(tot[v]);
    }
    if (bad) I.out->nonfinite = 1;
  }
}

// The mixed form's element residual by sum factorisation (hex_sumfact.h): the element's 36 nodal differences
// give the strain at every Gauss point by bilinear interpolation, and the stresses times wg are summed per
// pair of points before the bilinear weights of the transpose.  About 900 FP64 operations per element against
// about 2,100 for the B-matrix products, with the same laws, tangent terms and average stress as k_elem_rhs;
// the rounding differs from the B-matrix order (the FP64 form keeps that order).  The Gauss-point loop is
// unrolled so each point's accumulator slots are fixed at compile time.
__global__ void __launch_bounds__(kElemBlock) k_elem_rhs_sf(MeshDev m, Mats mats, const int8_t *etype,
                                                            const Inst *insts, const int *list) {
  constexpr double kXg = 0.577350269189626;  // Gauss coordinate (params.hpp:34)
  const Inst &I = insts[list[blockIdx.y]];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  double aux[6] = {0, 0, 0, 0, 0, 0};
  if (e < m.nelem) {
    const int ex = e % m.nex, ey = (e / m.nex) % m.ney, ez = e / (m.nex * m.ney);
    const int n0 = ez * m.nxny + ey * m.nx + ex;
    double D[3][3][4];
    {
      double ue[24];
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const int n = n0 + c_corner[a][2] * m.nxny + c_corner[a][1] * m.nx + c_corner[a][0];
#pragma unroll
        for (int d = 0; d < 3; ++d) ue[a * 3 + d] = I.u[n * 3 + d];
      }
      sf::diffs(ue, D);
    }
    const MatDev &mat = mats.m[etype[e]];
    const double inv4h[3] = {0.25 / m.dx, 0.25 / m.dy, 0.25 / m.dz};
    const double wg = m.wg;
    double S[3][3][4];
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int k = 0; k < 4; ++k) S[d][c][k] = 0.0;
#pragma unroll
    for (int g = 0; g < 8; ++g) {
      const int gs[3] = {(g == 1 || g == 2 || g == 5 || g == 6) ? 1 : -1, (g == 2 || g == 3 || g == 6 || g == 7) ? 1 : -1,
                         g >= 4 ? 1 : -1};
      double gr[3][3], eps[6], sg[6];
      sf::grad_at(D, gs, kXg, inv4h, gr);
      sf::strain_of(gr, eps);
      const double *vg = I.vars_old ? I.vars_old + ((size_t)e * 8 + g) * kNvarGp : nullptr;
      if (mat.type == 2 && I.gpd) {
        double Dm, ta, tc;
        law_damage_terms(mat, eps, vg, sg, &Dm, &ta, &tc);
        float *__restrict__ gpd = I.gpd;
        const size_t st = (size_t)8 * m.nelem, o = (size_t)g * m.nelem + e;
        gpd[o] = (float)ta;
        gpd[st + o] = (float)tc;
#pragma unroll
        for (int v = 0; v < 6; ++v) gpd[(2 + v) * st + o] = (float)sg[v];
        const double f = 1 - Dm;
#pragma unroll
        for (int v = 0; v < 6; ++v) sg[v] *= f;
      } else {
        law_stress(mat, eps, vg, sg);
      }
      sf::accumulate(S, gs, sg, wg);
#pragma unroll
      for (int v = 0; v < 6; ++v) aux[v] += sg[v] * wg;
    }
    double be[24];
    sf::finish(S, kXg, inv4h, be);
    double *__restrict__ bev = I.be;
#pragma unroll
    for (int i = 0; i < 24; ++i) bev[(size_t)i * m.nelem + e] = be[i];
  }
  double tot[6];
  if (grid_sum<6>(aux, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    bool bad = false;
#pragma unroll
    for (int v = 0; v < 6; ++v) {
      I.out->sig[v] = tot[v] / m.vol_tot;
      bad |= !isfinite(tot[v]);
    }
    if (bad) I.out->nonfinite = 1;
  }
}

// ---------------------------------------------------------------------------------------------------
// The element residual of k_elem_rhs_sf in double-float arithmetic, for elastic and damage phases: one thread
// per element runs elem_rhs_df (elem_df.cuh).  The FP64 pipe issues 2 operations per SM and cycle, so the FP64
// residual is bound by it; here the nodal displacements are split into float pairs once, and the differences,
// the Gauss-point strains, the laws, the stress sums and their transpose run on the FP32 pipe with about 46
// bits (the residual's rounding stays near 1e-13 of its terms).  Loads, the history, the element blocks and the
// average stress stay FP64.

static ResDf res_df(const MeshDev &m, const Mats &mats) {
  constexpr double kXg = 0.577350269189626;  // Gauss coordinate (params.hpp:34)
  ResDf c;
  for (int ph = 0; ph < 3; ++ph) {
    const MatDev &d = mats.m[ph];
    c.mat[ph] = MatDf{df_of(d.lambda), df_of(d.two_mu), df_of(d.mu),     df_of(d.xt_thr),
                      df_of(d.dmg_r0), df_of(d.dmg_r1), df_of(d.dmg_q0), df_of(d.dmg_q1)};
  }
  c.cm = df_of(1.0 - kXg);
  c.cp = df_of(1.0 + kXg);
  c.inv4h[0] = df_of(0.25 / m.dx);
  c.inv4h[1] = df_of(0.25 / m.dy);
  c.inv4h[2] = df_of(0.25 / m.dz);
  c.wg = df_of(m.wg);
  return c;
}

__global__ void __launch_bounds__(kElemBlock) k_elem_rhs_df(MeshDev m, Mats mats, ResDf cst, const int8_t *etype,
                                                            const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  dfl sav[6];  // the element's sum of wg sigma (the average stress)
#pragma unroll
  for (int v = 0; v < 6; ++v) sav[v] = dfl{0.f, 0.f};
  if (e < m.nelem) {
    const int ex = e % m.nex, ey = (e / m.nex) % m.ney, ez = e / (m.nex * m.ney);
    const int n0 = ez * m.nxny + ey * m.nx + ex;
    double ue[24];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const int n = n0 + c_corner[a][2] * m.nxny + c_corner[a][1] * m.nx + c_corner[a][0];
#pragma unroll
      for (int d = 0; d < 3; ++d) ue[a * 3 + d] = I.u[n * 3 + d];
    }
    const int ph = etype[e];
    float *__restrict__ gpd = I.gpd;
    const size_t st = (size_t)8 * m.nelem;
    auto sink = [&](int g, float ta, float tc, const float *s6) {
      const size_t o = (size_t)g * m.nelem + e;
      gpd[o] = ta;
      gpd[st + o] = tc;
#pragma unroll
      for (int v = 0; v < 6; ++v) gpd[(2 + v) * st + o] = s6[v];
    };
    dfl be[24];
    elem_rhs_df(ue, cst.mat[ph], mats.m[ph].type == 2, cst,
                I.vars_old ? I.vars_old + (size_t)e * 8 * kNvarGp : nullptr, kNvarGp, be, sav, sink);
    double *__restrict__ bev = I.be;
#pragma unroll
    for (int i = 0; i < 24; ++i) bev[(size_t)i * m.nelem + e] = df_to_double(be[i]);
  }
  double tot[6];
  if (grid_sum_df<6>(sav, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    bool bad = false;
#pragma unroll
    for (int v = 0; v < 6; ++v) {
      I.out->sig[v] = tot[v] / m.vol_tot;
      bad |= !isfinite(tot[v]);
    }
    if (bad) I.out->nonfinite = 1;
  }
}

// Node gather of the residual: b = -(sum of the element blocks of the 8 elements around the node, in the
// reference's element order ez, ey, ex), zero on Dirichlet rows (assembly.cpp:27-103), and ||b||_2.
__global__ void __launch_bounds__(kNodeBlock) k_node_rhs(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double sq[1] = {0.0};
  if (n < m.nn) {
    const int i = n % m.nx, j = (n / m.nx) % m.ny, k = n / m.nxny;
    double b0 = 0.0, b1 = 0.0, b2 = 0.0;
    const double *__restrict__ be = I.be;
    double *__restrict__ b = I.b;
    if (!is_boundary(m, i, j, k)) {
#pragma unroll
      for (int dz = -1; dz <= 0; ++dz)
#pragma unroll
        for (int dy = -1; dy <= 0; ++dy)
#pragma unroll
          for (int dx = -1; dx <= 0; ++dx) {
            const int e = ((k + dz) * m.ney + (j + dy)) * m.nex + (i + dx);
            const int a = local_of(-dx, -dy, -dz);
            b0 += be[(size_t)(a * 3 + 0) * m.nelem + e];
            b1 += be[(size_t)(a * 3 + 1) * m.nelem + e];
            b2 += be[(size_t)(a * 3 + 2) * m.nelem + e];
          }
      b0 = -b0;
      b1 = -b1;
      b2 = -b2;
    }
    b[n * 3 + 0] = b0;
    b[n * 3 + 1] = b1;
    b[n * 3 + 2] = b2;
    sq[0] = b0 * b0 + b1 * b1 + b2 * b2;
  }
  double tot[1];
  if (grid_sum<1>(sq, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) {
    I.out->norm = sqrt(tot[0]);
    if (!isfinite(tot[0])) I.out->nonfinite = 1;
  }
}

// ---------------------------------------------------------------------------------------------------
// Jacobian assembly into ELL (assembly.cpp:105-178, ell-common.cpp:166-198).
//
// Elements are processed in 8 colours (parity of ex, ey, ez) so that two elements of one launch never share
// a node: each launch adds its elements' 24x24 blocks into the rows of their interior nodes without atomics,
// and the order in which a matrix entry receives its (up to 8) contributions is fixed.  A block holds
// kMatElems elements x 24 threads; thread p of an element owns row p of its Ke.
//
// Nonlinear laws: per Gauss point the tangent C (FD, 7 stress evaluations) is formed by 8 threads, then
// cxb = (C B) wg is built cooperatively in shared memory and each thread accumulates its row
// Ke[p][:] += B[:,p]^T cxb -- the reference's association (assembly.cpp:159-176).  Elastic-law elements
// scatter the phase's precomputed Ke (identical for every element of a phase: B and wg are uniform).
constexpr int kMatElems = 8;

__device__ __forceinline__ int ell_idx(int s, int fi, int fj) { return s * 9 + fi * 3 + fj; }

template <typename T>
__device__ __forceinline__ T *ell_values(const Inst &I);
template <>
__device__ __forceinline__ double *ell_values<double>(const Inst &I) {
  return I.vals;
}
template <>
__device__ __forceinline__ float *ell_values<float>(const Inst &I) {
  return I.vals32;
}

// T = double: the plain FP64 Jacobian with the reference's forward-difference tangents.  T = float: the mixed
// form's FP32 Jacobian -- the Gauss-point tangents are formed in closed form in FP64 and rounded once; Ke is
// accumulated in FP32.  Dual = true (T = double): the exact derivative of the stress, column by column with
// forward-mode dual numbers (adjoint_laws.h), for the adjoint of a load path (a missing history reads as 0).
template <typename T, bool Dual = false>
__global__ void __launch_bounds__(kMatElems * 24) k_elem_mat(MeshDev m, Mats mats, const int8_t *etype,
                                                              const double *dsh_g, const T *ke_phase,
                                                              const Inst *insts, const int *list, int color) {
  __shared__ double dsh[8 * 24];
  __shared__ double ue[kMatElems][24];
  __shared__ T Cg[kMatElems][8][36];
  __shared__ T cxb[kMatElems][6 * 24];
  for (int t = threadIdx.x; t < 192; t += blockDim.x) dsh[t] = dsh_g[t];
  const Inst &I = insts[list[blockIdx.y]];
  const int cx = color & 1, cy = (color >> 1) & 1, cz = (color >> 2) & 1;
  const int ncx = (m.nex - cx + 1) / 2, ncy = (m.ney - cy + 1) / 2, ncz = (m.nez - cz + 1) / 2;
  const int nce = ncx * ncy * ncz;
  const int el = threadIdx.x / 24, p = threadIdx.x % 24;
  const int ce = blockIdx.x * kMatElems + el;
  const bool valid = ce < nce;
  int ex = 0, ey = 0, ez = 0, e = 0, n0 = 0, law = 0, ph = 0;
  if (valid) {
    ex = 2 * (ce % ncx) + cx;
    ey = 2 * ((ce / ncx) % ncy) + cy;
    ez = 2 * (ce / (ncx * ncy)) + cz;
    e = (ez * m.ney + ey) * m.nex + ex;
    n0 = ez * m.nxny + ey * m.nx + ex;
    ph = etype[e];
    law = mats.m[ph].type;
    const int a = p / 3, d = p % 3;
    const int n = n0 + c_corner[a][2] * m.nxny + c_corner[a][1] * m.nx + c_corner[a][0];
    ue[el][p] = I.u[n * 3 + d];
  }
  __syncthreads();
  const bool nonlin = valid && law != 0;
  // Gauss-point tangents (FP64).
  if (nonlin && p < 8) {
    double eps[6], C[36];
    gp_strain(&dsh[p * 24], ue[el], eps);
    const double *vg = I.vars_old ? I.vars_old + ((size_t)e * 8 + p) * kNvarGp : nullptr;
    if constexpr (Dual) {
      const MatDev &md = mats.m[ph];
      const double theta[adj::kNpar] = {md.E, md.nu, md.Xt, md.Sy, md.Ka};
      double h[7], ds[6], dh[7];
#pragma unroll
      for (int i = 0; i < 7; ++i) h[i] = vg ? vg[i] : 0.0;
#pragma unroll 1
      for (int j = 0; j < 6; ++j) {
        adj::law_column(md.type, theta, eps, h, j, ds, dh);
#pragma unroll
        for (int i = 0; i < 6; ++i) C[i * 6 + j] = ds[i];
      }
    } else if constexpr (sizeof(T) == sizeof(float)) {
      law_ctan_exact(mats.m[ph], eps, vg, C);  // mixed form: closed-form consistent tangent
    } else {
      law_ctan(mats.m[ph], eps, vg, C);  // FP64 form: the reference's forward differences
    }
#pragma unroll
    for (int i = 0; i < 36; ++i) Cg[el][p][i] = (T)C[i];
  }
  __syncthreads();
  T row[24];
  const int a = p / 3, d = p % 3;
  // Non-zero rows m of column p of B in ascending order, and their coefficients.
  const int m0 = d, m1 = (d == 0) ? 3 : (d == 1 ? 3 : 4), m2 = (d == 0) ? 4 : 5;
  if (nonlin) {
#pragma unroll
    for (int q = 0; q < 24; ++q) row[q] = (T)0;
  } else if (valid) {
    const T *K = ke_phase + (size_t)ph * 576 + p * 24;
#pragma unroll
    for (int q = 0; q < 24; ++q) row[q] = K[q];
  }
  const T wg = (T)m.wg;
#pragma unroll 1
  for (int g = 0; g < 8; ++g) {
    const double *dg = &dsh[g * 24];
    // B column p has B[m0][p], B[m1][p], B[m2][p] non-zero.
    const T gx = (T)dg[a * 3], gy = (T)dg[a * 3 + 1], gz = (T)dg[a * 3 + 2];
    const T bp0 = (d == 0) ? gx : (d == 1 ? gy : gz);
    const T bp1 = (d == 0) ? gy : gx;
    const T bp2 = (d == 0) ? gz : (d == 1 ? gz : gy);
    if (nonlin) {
      // cxb[mm][p] = wg * sum_k C[mm][k] B[k][p] over the non-zero k of column p (ascending).
      const T *C = Cg[el][g];
#pragma unroll
      for (int mm = 0; mm < 6; ++mm) {
        T t = (T)0;
        t += C[mm * 6 + m0] * bp0;
        t += C[mm * 6 + m1] * bp1;
        t += C[mm * 6 + m2] * bp2;
        cxb[el][mm * 24 + p] = t * wg;
      }
    }
    __syncthreads();
    if (nonlin) {
#pragma unroll
      for (int q = 0; q < 24; ++q) {
        row[q] += bp0 * cxb[el][m0 * 24 + q];
        row[q] += bp1 * cxb[el][m1 * 24 + q];
        row[q] += bp2 * cxb[el][m2 * 24 + q];
      }
    }
    __syncthreads();
  }
  if (!valid) return;
  // Scatter row p = (local node a, dof d) into the ELL row of node(a), unless it is a boundary row.
  const int ai = c_corner[a][0], aj = c_corner[a][1], ak = c_corner[a][2];
  const int gi = ex + ai, gj = ey + aj, gk = ez + ak;
  if (is_boundary(m, gi, gj, gk)) return;
  const int node = n0 + ak * m.nxny + aj * m.nx + ai;
  T *vals = ell_values<T>(I);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const int s = (c_corner[b][2] - ak + 1) * 9 + (c_corner[b][1] - aj + 1) * 3 + (c_corner[b][0] - ai + 1);
#pragma unroll
    for (int fj = 0; fj < 3; ++fj) {
      T *dst = &vals[(size_t)ell_idx(s, d, fj) * m.np + node];
      *dst += row[b * 3 + fj];
    }
  }
}

// ---------------------------------------------------------------------------------------------------
// FP32 Jacobian by node gather (mixed form, every phase elastic or damage).
//
// Thread (node n, element position ep): of the 8 elements around n it takes the one at ep = dxq + 2 dyq +
// 4 dzq, element (i-1+dxq, j-1+dyq, k-1+dzq), in which n is the local corner a = (1-dxq, 1-dyq, 1-dzq).  It
// forms the 3x3 blocks of that element's matrix coupling a with every corner b of the element:
//   damage  (C_g = a_g C + c_g s_g s_g^T):  Ke_ab = sum_g a_g K0_g,ab + c_g wg (B_a,g^T s_g)(B_b,g^T s_g)^T
//   elastic:                               Ke_ab = sum_g K0_g,ab
// with K0_g = wg B_g^T C_phase B_g precomputed per phase and Gauss point, and (a_g, c_g, s_g) written by the
// residual kernel (k_elem_rhs_df) at the same displacement.  The 8 warps of a block (one element position each) add their
// blocks into the block's 32 node rows (27 slots x 9) in shared memory in a fixed order; the rows are then
// written once, coalesced.  No colouring, atomics or zeroing pass; boundary nodes get their real rows.
constexpr int kAsmNodes = 32;
constexpr int kAsmRow = kEllPerNode + 2;  // 245 floats: odd stride, conflict-free

__host__ __device__ constexpr int corner_x(int b) { return ((b & 3) == 1 || (b & 3) == 2) ? 1 : 0; }
__host__ __device__ constexpr int corner_y(int b) { return (b & 3) >= 2 ? 1 : 0; }
__host__ __device__ constexpr int corner_z(int b) { return b >> 2; }
__host__ __device__ constexpr int local_c(int ox, int oy, int oz) { return oz * 4 + (oy ? 3 - ox : ox); }
// Stencil slot (0..26) of the neighbour at offset (dx,dy,dz).
__host__ __device__ constexpr int slot_of(int dx, int dy, int dz) { return (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1); }

template <int EP, int B>
__device__ __forceinline__ void asm_add_b(float (&acc)[8][9], float A, float cw, const float (&va)[3],
                                          const float *dg, const float (&s)[6], const float *__restrict__ K) {
  constexpr int a = local_c(1 - (EP & 1), 1 - ((EP >> 1) & 1), 1 - (EP >> 2));
  const float gx = dg[B * 3], gy = dg[B * 3 + 1], gz = dg[B * 3 + 2];
  const float vb[3] = {gx * s[0] + gy * s[3] + gz * s[4], gy * s[1] + gx * s[3] + gz * s[5],
                       gz * s[2] + gx * s[4] + gy * s[5]};
#pragma unroll
  for (int fi = 0; fi < 3; ++fi)
#pragma unroll
    for (int fj = 0; fj < 3; ++fj)
      acc[B][fi * 3 + fj] += A * __ldg(&K[(a * 3 + fi) * 24 + B * 3 + fj]) + cw * va[fi] * vb[fj];
}

template <int EP, int B>
__device__ __forceinline__ void asm_add_b_elastic(float (&acc)[8][9], const float *__restrict__ K) {
  constexpr int a = local_c(1 - (EP & 1), 1 - ((EP >> 1) & 1), 1 - (EP >> 2));
#pragma unroll
  for (int q = 0; q < 9; ++q) acc[B][q] += __ldg(&K[(a * 3 + q / 3) * 24 + B * 3 + q % 3]);
}

template <int EP>
__device__ __forceinline__ void asm_ep(const MeshDev &m, const Mats &mats, const int8_t *__restrict__ etype,
                                           const float *__restrict__ k0g, const float *__restrict__ kesum,
                                           const float *dsh, const float *__restrict__ gpd, int i, int j, int k,
                                           float (&acc)[8][9]) {
  constexpr int a = local_c(1 - (EP & 1), 1 - ((EP >> 1) & 1), 1 - (EP >> 2));
  const int ex = i - 1 + (EP & 1), ey = j - 1 + ((EP >> 1) & 1), ez = k - 1 + (EP >> 2);
  if (ex < 0 || ey < 0 || ez < 0 || ex >= m.nex || ey >= m.ney || ez >= m.nez) return;
  const int e = (ez * m.ney + ey) * m.nex + ex;
  const int ph = etype[e];
  if (mats.m[ph].type == 0) {
    const float *K = kesum + ph * 576;
    asm_add_b_elastic<EP, 0>(acc, K); asm_add_b_elastic<EP, 1>(acc, K);
    asm_add_b_elastic<EP, 2>(acc, K); asm_add_b_elastic<EP, 3>(acc, K);
    asm_add_b_elastic<EP, 4>(acc, K); asm_add_b_elastic<EP, 5>(acc, K);
    asm_add_b_elastic<EP, 6>(acc, K); asm_add_b_elastic<EP, 7>(acc, K);
    return;
  }
  const size_t st = (size_t)8 * m.nelem;
  const float wg = (float)m.wg;
#pragma unroll 1
  for (int g = 0; g < 8; ++g) {
    const size_t o = (size_t)g * m.nelem + e;
    const float A = __ldg(&gpd[o]), cw = __ldg(&gpd[st + o]) * wg;
    float s[6];
#pragma unroll
    for (int v = 0; v < 6; ++v) s[v] = __ldg(&gpd[(2 + v) * st + o]);
    const float *dg = dsh + g * 24;
    const float gx = dg[a * 3], gy = dg[a * 3 + 1], gz = dg[a * 3 + 2];
    const float va[3] = {gx * s[0] + gy * s[3] + gz * s[4], gy * s[1] + gx * s[3] + gz * s[5],
                         gz * s[2] + gx * s[4] + gy * s[5]};
    const float *K = k0g + ((size_t)ph * 8 + g) * 576;
    asm_add_b<EP, 0>(acc, A, cw, va, dg, s, K); asm_add_b<EP, 1>(acc, A, cw, va, dg, s, K);
    asm_add_b<EP, 2>(acc, A, cw, va, dg, s, K); asm_add_b<EP, 3>(acc, A, cw, va, dg, s, K);
    asm_add_b<EP, 4>(acc, A, cw, va, dg, s, K); asm_add_b<EP, 5>(acc, A, cw, va, dg, s, K);
    asm_add_b<EP, 6>(acc, A, cw, va, dg, s, K); asm_add_b<EP, 7>(acc, A, cw, va, dg, s, K);
  }
}

template <int EP>
__device__ __forceinline__ void asm_store(const float (&acc)[8][9], float *row) {
  constexpr int a = local_c(1 - (EP & 1), 1 - ((EP >> 1) & 1), 1 - (EP >> 2));
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const int sl = slot_of(corner_x(b) - corner_x(a), corner_y(b) - corner_y(a), corner_z(b) - corner_z(a));
#pragma unroll
    for (int q = 0; q < 9; ++q) row[sl * 9 + q] += acc[b][q];
  }
}

#define MGB_EP_SWITCH(w, CALL) \
  switch (w) {                 \
    case 0: CALL(0); break;    \
    case 1: CALL(1); break;    \
    case 2: CALL(2); break;    \
    case 3: CALL(3); break;    \
    case 4: CALL(4); break;    \
    case 5: CALL(5); break;    \
    case 6: CALL(6); break;    \
    default: CALL(7); break;   \
  }

__global__ void __launch_bounds__(kAsmNodes * 8) k_asm_gather32(MeshDev m, Mats mats, const int8_t *etype,
                                                              const float *k0g, const float *kesum,
                                                              const float *dsh_g, const Inst *insts,
                                                              const int *list, float omega, float csafe,
                                                              int sdiag) {
  __shared__ float rows[kAsmNodes * kAsmRow];
  __shared__ float dsh[8 * 24];
  for (int t = threadIdx.x; t < kAsmNodes * kAsmRow; t += blockDim.x) rows[t] = 0.f;
  for (int t = threadIdx.x; t < 192; t += blockDim.x) dsh[t] = dsh_g[t];
  __syncthreads();
  const Inst &I = insts[list[blockIdx.y]];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n = blockIdx.x * kAsmNodes + lane;
  const bool valid = n < m.nn;
  const int i = n % m.nx, j = (n / m.nx) % m.ny, k = n / m.nxny;
  float acc[8][9];
#pragma unroll
  for (int b = 0; b < 8; ++b)
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[b][q] = 0.f;
  if (valid) {
#define MGB_ASM_CALL(E) asm_ep<E>(m, mats, etype, k0g, kesum, dsh, I.gpd, i, j, k, acc)
    MGB_EP_SWITCH(w, MGB_ASM_CALL)
#undef MGB_ASM_CALL
  }
  // element positions add into the node rows one after the other (fixed summation order)
  for (int p = 0; p < 8; ++p) {
    __syncthreads();
    if (w == p && valid) {
#define MGB_STORE_CALL(E) asm_store<E>(acc, &rows[lane * kAsmRow])
      MGB_EP_SWITCH(w, MGB_STORE_CALL)
#undef MGB_STORE_CALL
    }
  }
  __syncthreads();
  float *__restrict__ vals = I.vals32;
  const size_t np = m.np;
  for (int E = w; E < kEllPerNode; E += 8) vals[(size_t)E * np + (size_t)blockIdx.x * kAsmNodes + lane] = rows[lane * kAsmRow + E];
  // sdiag: the multigrid's level-0 smoother diagonal from the rows in shared memory, warp fi for row fi of each
  // node: 1 / max(a_ii / omega, csafe sum_j |a_ij|) over interior columns, the sums in k_mg_sdiag's order (so
  // the same values bit for bit); boundary rows 1.
  if (sdiag && w < 3 && valid) {
    const int fi = w;
    float *__restrict__ kinv = I.mg->lv[0].kinv;
    if (i == 0 || j == 0 || k == 0 || i == m.nx - 1 || j == m.ny - 1 || k == m.nz - 1) {
      kinv[(size_t)n * 3 + fi] = 1.f;
    } else {
      const float *row = &rows[lane * kAsmRow];
      float l1 = 0.f;
#pragma unroll
      for (int s = 0; s < 27; ++s) {
        const int bi = i + s % 3 - 1, bj = j + (s / 3) % 3 - 1, bk = k + s / 9 - 1;
        if (bi == 0 || bj == 0 || bk == 0 || bi == m.nx - 1 || bj == m.ny - 1 || bk == m.nz - 1) continue;
#pragma unroll
        for (int fj = 0; fj < 3; ++fj) l1 += fabsf(row[s * 9 + fi * 3 + fj]);
      }
      kinv[(size_t)n * 3 + fi] = 1.f / fmaxf(row[13 * 9 + fi * 4] / omega, csafe * l1);
    }
  }
}

// Zero the ELL values of the listed instances (ell_set_zero_mat, ell-common.cpp:200).
template <typename T>
__global__ void k_zero_vals(size_t count, const Inst *insts, const int *list) {
  T *v = ell_values<T>(insts[list[blockIdx.y]]);
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x)
    v[t] = (T)0;
}

// ---------------------------------------------------------------------------------------------------
// Internal-variable update (update.cpp:32-56), one thread per Gauss point; the nonlinear flags are OR-ed
// into out.nonlinear.
__global__ void __launch_bounds__(kNodeBlock) k_evolve(MeshDev m, Mats mats, const int8_t *etype,
                                                         const double *dsh_g, const Inst *insts,
                                                         const int *list) {
  __shared__ double dsh[8 * 24];
  for (int t = threadIdx.x; t < 192; t += blockDim.x) dsh[t] = dsh_g[t];
  __syncthreads();
  const Inst &I = insts[list[blockIdx.y]];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  bool nl = false;
  if (t < m.nelem * 8) {
    const int e = t >> 3, g = t & 7;
    const MatDev &mat = mats.m[etype[e]];
    if (mat.type != 0) {
      const int ex = e % m.nex, ey = (e / m.nex) % m.ney, ez = e / (m.nex * m.ney);
      const int n0 = ez * m.nxny + ey * m.nx + ex;
      double ue[24], eps[6];
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const int n = n0 + c_corner[a][2] * m.nxny + c_corner[a][1] * m.nx + c_corner[a][0];
#pragma unroll
        for (int d = 0; d < 3; ++d) ue[a * 3 + d] = I.u[n * 3 + d];
      }
      gp_strain(&dsh[g * 24], ue, eps);
      const size_t off = ((size_t)e * 8 + g) * kNvarGp;
      nl = law_evolve(mat, eps, I.has_vars_old ? I.vars_old + off : nullptr, I.has_vars_old != 0, I.vars_new + off);
    }
  }
  if (__syncthreads_or(nl) && threadIdx.x == 0) atomicOr(&I.out->nonlinear, 1);
}

// ---------------------------------------------------------------------------------------------------
// Element averages of strain and stress for field output, calc_fields (average.cpp:84-112):
// fields[e*12 + v] = sum_gp strain_v wg * ivol, fields[e*12 + 6 + v] = sum_gp stress_v wg * ivol.
__global__ void __launch_bounds__(kElemBlock) k_elem_fields(MeshDev m, Mats mats, const int8_t *etype,
                                                              const double *dsh_g, const double *u,
                                                              const double *vars, double ivol, double *fields) {
  __shared__ double dsh[8 * 24];
  for (int t = threadIdx.x; t < 192; t += blockDim.x) dsh[t] = dsh_g[t];
  __syncthreads();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelem) return;
  const int ex = e % m.nex, ey = (e / m.nex) % m.ney, ez = e / (m.nex * m.ney);
  const int n0 = ez * m.nxny + ey * m.nx + ex;
  double ue[24];
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int n = n0 + c_corner[a][2] * m.nxny + c_corner[a][1] * m.nx + c_corner[a][0];
#pragma unroll
    for (int d = 0; d < 3; ++d) ue[a * 3 + d] = u[n * 3 + d];
  }
  const MatDev &mat = mats.m[etype[e]];
  double ea[6] = {0, 0, 0, 0, 0, 0}, sa[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll 1
  for (int g = 0; g < 8; ++g) {
    double eps[6], s[6];
    gp_strain(&dsh[g * 24], ue, eps);
    law_stress(mat, eps, vars ? vars + ((size_t)e * 8 + g) * kNvarGp : nullptr, s);
#pragma unroll
    for (int v = 0; v < 6; ++v) {
      ea[v] += eps[v] * m.wg;
      sa[v] += s[v] * m.wg;
    }
  }
#pragma unroll
  for (int v = 0; v < 6; ++v) {
    fields[(size_t)e * 12 + v] = ea[v] * ivol;
    fields[(size_t)e * 12 + 6 + v] = sa[v] * ivol;
  }
}

}  // namespace mgb

// ---------------------------------------------------------------------------------------------------
// Launch wrappers (the C-ABI layer the host engine calls).

using namespace mgb;

static inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

template <typename T, bool Dual = false>
static int launch_assembly(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh, const T *ke_phase,
                           const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const size_t count = (size_t)kEllPerNode * m->np;
  k_zero_vals<T><<<dim3(cdiv(count, 8 * kNodeBlock), nlist), kNodeBlock, 0, s>>>(count, insts, list);
  for (int c = 0; c < 8; ++c) {
    const int cx = c & 1, cy = (c >> 1) & 1, cz = (c >> 2) & 1;
    const int nce = ((m->nex - cx + 1) / 2) * ((m->ney - cy + 1) / 2) * ((m->nez - cz + 1) / 2);
    if (nce <= 0) continue;
    k_elem_mat<T, Dual><<<dim3(cdiv(nce, kMatElems), nlist), kMatElems * 24, 0, s>>>(*m, *mats, etype, dsh, ke_phase,
                                                                                     insts, list, c);
  }
  return (int)cudaGetLastError();
}

extern "C" {

int mgb_launch_set_bc(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_set_bc<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_add_du(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const int nndim = m->nn * 3;
  k_add_du<<<dim3(cdiv(nndim, 4 * kNodeBlock), nlist), kNodeBlock, 0, s>>>(nndim, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_copy(int n, const double *const *src, double *const *dst, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_copy<<<dim3(cdiv(n, 4 * kNodeBlock), nlist), kNodeBlock, 0, s>>>(n, src, dst, list);
  return (int)cudaGetLastError();
}

int mgb_launch_residual(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh,
                        const Inst *insts, const int *list, int nlist, int form, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const dim3 g(cdiv(m->nelem, kElemBlock), nlist);
  if (form == 1)
    k_elem_rhs<<<g, kElemBlock, 0, s>>>(*m, *mats, etype, dsh, insts, list);
  else if (form == 2)
    k_elem_rhs_df<<<g, kElemBlock, 0, s>>>(*m, *mats, res_df(*m, *mats), etype, insts, list);
  else
    k_elem_rhs_sf<<<g, kElemBlock, 0, s>>>(*m, *mats, etype, insts, list);
  k_node_rhs<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_node_gather(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_node_rhs<<<dim3(cdiv(m->nn, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_assembly(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh,
                        const double *ke_phase, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  return launch_assembly<double>(m, mats, etype, dsh, ke_phase, insts, list, nlist, s);
}

int mgb_launch_assembly_dual(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh,
                             const double *ke_phase, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  return launch_assembly<double, true>(m, mats, etype, dsh, ke_phase, insts, list, nlist, s);
}

int mgb_launch_assembly32(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh,
                          const float *ke_phase, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  return launch_assembly<float>(m, mats, etype, dsh, ke_phase, insts, list, nlist, s);
}

int mgb_launch_assembly_gather32(const MeshDev *m, const Mats *mats, const int8_t *etype, const float *k0g,
                              const float *kesum, const float *dsh32, const Inst *insts, const int *list, int nlist,
                              float omega, float csafe, int sdiag, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_asm_gather32<<<dim3(cdiv(m->np, kAsmNodes), nlist), kAsmNodes * 8, 0, s>>>(*m, *mats, etype, k0g, kesum, dsh32,
                                                                             insts, list, omega, csafe, sdiag);
  return (int)cudaGetLastError();
}

int mgb_launch_elem_fields(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh, const double *u,
                           const double *vars, double ivol, double *fields, cudaStream_t s) {
  k_elem_fields<<<cdiv(m->nelem, kElemBlock), kElemBlock, 0, s>>>(*m, *mats, etype, dsh, u, vars, ivol, fields);
  return (int)cudaGetLastError();
}

int mgb_launch_evolve(const MeshDev *m, const Mats *mats, const int8_t *etype, const double *dsh,
                      const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_evolve<<<dim3(cdiv((size_t)m->nelem * 8, kNodeBlock), nlist), kNodeBlock, 0, s>>>(*m, *mats, etype, dsh, insts,
                                                                                     list);
  return (int)cudaGetLastError();
}

}  // extern "C"
