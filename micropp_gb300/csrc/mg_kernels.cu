// mg_kernels.cu -- geometric multigrid preconditioner of the mixed form's FP32 CG solves (1 or 6 right-hand
// sides).
//
// The RVE grid is structured, so a coarse level is again a structured grid: every axis of n elements becomes
// ceil(n / 2) elements, coarse node I sits on fine node 2I (the last coarse interval is one fine element wide
// when n is odd), and the prolongation P is trilinear: a fine node with even index along an axis takes its
// coarse parent with weight 1, an odd one its two neighbours with weight 1/2.  Corrections vanish on boundary
// nodes (Dirichlet rows), so P only couples interior nodes.  The coarse operator is the Galerkin product
// A_c = P^T A P; with trilinear P and a 27-point operator it is again a 27-point operator of 3x3 blocks, so
// every level uses the fine level's stencil ELL layout, vals[(s * 9 + fi * 3 + fj) * np + n].  P is a tensor
// product of 1-D interpolations, so the product is formed one axis at a time (k_mg_rap1).
//
// The preconditioner is one V-cycle with a damped-Jacobi smoother before and after the coarse correction and a
// fixed number of Jacobi sweeps on the coarsest level.  The smoother's diagonal is safeguarded per row:
// d_i = max(a_ii / w, c sum_j |a_ij|) with w = 0.6 and c > 1/2 (k_mg_sdiag).  It is the plain damped diagonal
// wherever that contracts; where the operator is strongly anisotropic (loading damage tangents) the Gershgorin
// bound takes over, since 2 D - A is then diagonally dominant and every sweep contracts for an SPD operator.
// Every step is linear and symmetric, so the V-cycle is a fixed symmetric positive-definite preconditioner and
// the CG recurrences stay those of preconditioned CG.
//
//   level 0:   x0 = D^-1 r                      (written by the CG update kernel)
//   l < L-1:   t_l = b_l - A_l x_l;  b_{l+1} = P^T t_l;  x_{l+1} = D^-1 b_{l+1}
//   coarsest:  (sweeps - 1) x Jacobi sweeps, ping-pong between x and y
//   l >= 1:    t_l = x_l + P x_{l+1};  x_l = t_l + D^-1 (b_l - A_l t_l)
//   level 0:   t_0 = x_0 + P x_1;  z = t_0 + D^-1 (r - A t_0), with r.z and the CG scalars
// (D: the safeguarded smoother diagonal of each level; lv[l].kinv holds its inverse.  The kernels' omega
// argument scales D^-1 and is 1 with it.)
//
// Level 0 vectors are the CG's own: node-interleaved r32/z32 for one right-hand side, component-major R6/Z6
// for six; the level-0 residual and prolongation go to lv[0].t (3 * nn or 18 * np floats).  Every kernel
// writes zeros on boundary nodes, so coarse vectors never carry values there.  Launch order on one stream is
// the only synchronisation; reductions use the last-block ticket of reduce.cuh.
#include <cuda_fp16.h>

#include <algorithm>

#include "device.cuh"
#include "launch.h"
#include "reduce.cuh"

namespace mgb {
namespace {

constexpr int kMgBlock = 128;
constexpr int kMgCoarseBlock = 256;
constexpr int kMgCoarseSmem = 200 * 1024;  // shared memory of the shared-memory coarse sweeps, at most

// The FP16 copy of the level-0 operator (MICROPP3_PRECOND_MG_HALF): scale16 x the FP32 values, streamed by the
// two level-0 smoothing passes; their sums are rescaled by inv16, an exact power of two.
__device__ __forceinline__ float ld_h(const unsigned short *__restrict__ p) {
  return __half2float(__ushort_as_half(__ldcs(p)));
}

// Two consecutive FP16 entries (nodes n0, n0 + 1) in one 4-byte load.
__device__ __forceinline__ float2 ld_h2(const unsigned int *__restrict__ p) {
  const unsigned int b = __ldcs(p);
  return __half22float2(__halves2half2(__ushort_as_half((unsigned short)(b & 0xffffu)),
                                       __ushort_as_half((unsigned short)(b >> 16))));
}

// Index of component (r, d) of node n in a level's vector: node-interleaved for a single right-hand side on
// level 0 (RM), component-major otherwise.
template <bool RM>
__device__ __forceinline__ size_t vix(int r, int d, int n, size_t np) {
  return RM ? (size_t)n * 3 + d : (size_t)(r * 3 + d) * np + n;
}

__device__ __forceinline__ bool on_boundary(const MeshDev &m, int n, int &i, int &j, int &k) {
  i = n % m.nx;
  j = (n / m.nx) % m.ny;
  k = n / m.nxny;
  return i == 0 || j == 0 || k == 0 || i == m.nx - 1 || j == m.ny - 1 || k == m.nz - 1;
}

__device__ __forceinline__ float half_pow(int a) { return a == 0 ? 1.0f : (a == 1 || a == -1) ? 0.5f : 0.0f; }

template <int NR>
__device__ __forceinline__ bool inst_done(const Inst &I) {
  return NR == 1 ? I.cg->done != 0 : I.cg6->all_done != 0;
}

// Buffers of level l of an instance (level 0: the CG's vectors and the fine operator).
struct LvView {
  const float *vals, *kinv;
  float *b, *x, *y, *t;
};

template <int NR>
__device__ __forceinline__ LvView view(const Inst &I, int l) {
  const MgLevel &L = I.mg->lv[l];
  LvView v;
  if (l == 0) {
    v.vals = I.vals32;
    v.kinv = L.kinv;
    v.b = NR == 1 ? I.r32 : I.R6;
    v.x = NR == 1 ? I.z32 : I.Z6;
    v.y = nullptr;
  } else {
    v.vals = L.vals;
    v.kinv = L.kinv;
    v.b = L.b;
    v.x = L.x;
    v.y = L.y;
  }
  v.t = L.t;
  return v;
}

// which: 0 = x, 1 = y, 2 = t
__device__ __forceinline__ float *pick(const LvView &v, int which) { return which == 0 ? v.x : which == 1 ? v.y : v.t; }

// y = A x at interior node n for NR right-hand sides (slot order, then column order, as the CG SpMVs).
template <int NR, bool RM, bool STREAM>
__device__ __forceinline__ void apply_node(const MeshDev &m, const float *__restrict__ vals,
                                           const float *__restrict__ x, int n, float (&y)[NR * 3]) {
  const size_t np = m.np;
#pragma unroll
  for (int c = 0; c < NR * 3; ++c) y[c] = 0.f;
#pragma unroll 3
  for (int s = 0; s < 27; ++s) {
    const int nb = n + (s / 9 - 1) * m.nxny + ((s / 3) % 3 - 1) * m.nx + (s % 3 - 1);
    float K[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const float *a = vals + (size_t)(s * 9 + q) * np + n;
      K[q] = STREAM ? __ldcs(a) : __ldg(a);
    }
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      float xv[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) xv[d] = x[vix<RM>(r, d, nb, np)];
#pragma unroll
      for (int fi = 0; fi < 3; ++fi)
#pragma unroll
        for (int fj = 0; fj < 3; ++fj) y[r * 3 + fi] = fmaf(K[fi * 3 + fj], xv[fj], y[r * 3 + fi]);
    }
  }
}

// apply_node on level 0 with the FP16 copy of the operator (streamed), rescaled once.
template <int NR, bool RM>
__device__ __forceinline__ void apply_node_h(const MeshDev &m, const unsigned short *__restrict__ vals, float inv,
                                             const float *__restrict__ x, int n, float (&y)[NR * 3]) {
  const size_t np = m.np;
#pragma unroll
  for (int c = 0; c < NR * 3; ++c) y[c] = 0.f;
#pragma unroll 3
  for (int s = 0; s < 27; ++s) {
    const int nb = n + (s / 9 - 1) * m.nxny + ((s / 3) % 3 - 1) * m.nx + (s % 3 - 1);
    float K[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) K[q] = ld_h(vals + (size_t)(s * 9 + q) * np + n);
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      float xv[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) xv[d] = x[vix<RM>(r, d, nb, np)];
#pragma unroll
      for (int fi = 0; fi < 3; ++fi)
#pragma unroll
        for (int fj = 0; fj < 3; ++fj) y[r * 3 + fi] = fmaf(K[fi * 3 + fj], xv[fj], y[r * 3 + fi]);
    }
  }
#pragma unroll
  for (int c = 0; c < NR * 3; ++c) y[c] *= inv;
}

// One 1-D step of the separable Galerkin product: P = Px Py Pz (each a 1-D interpolation with the Dirichlet
// rows and columns of its axis removed), so P^T A P = Pz^T (Py^T (Px^T A Px) Py) Pz.  The step along `axis` maps
// the operator on grid mi to the operator on grid mo, mi with that axis coarsened to ceil(n / 2) elements; the
// other axes pass through.  Thread (S, io) forms the 3x3 block of output node io toward its neighbour at offset
// S from at most 7 input blocks:
//   B[io][S] = sum_{a, o} 2^-|a| 2^-|e| A[i][s'],  i = io with 2X + a on the axis, j = i + o on the axis,
//   e = j - 2 (X + S_axis), s' = S with o on the axis,
// over i and j interior along the axis.  Rows and columns on the axis' boundary are zero; in the last step
// (dst = 3, the next level's operator) boundary rows become identity rows.  The order of the additions is
// fixed.  src / dst: 0 = level lf's operator, 1 = mid1, 2 = mid2, 3 = level lf + 1's operator.
__global__ void __launch_bounds__(kMgBlock) k_mg_rap1(MeshDev mi, MeshDev mo, const Inst *insts, const int *list,
                                                      int lf, int axis, int src, int dst) {
  const Inst &I = insts[list[blockIdx.y]];
  const MgInst &G = *I.mg;
  const float *__restrict__ A = src == 0 ? (lf == 0 ? I.vals32 : G.lv[lf].vals) : src == 1 ? G.mid1 : G.mid2;
  float *__restrict__ B = dst == 3 ? G.lv[lf + 1].vals : dst == 1 ? G.mid1 : G.mid2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 27 * mo.nn) return;
  const int S = t / mo.nn, io = t - S * mo.nn;
  int c[3] = {io % mo.nx, (io / mo.nx) % mo.ny, io / mo.nxny};
  const int so[3] = {S % 3 - 1, (S / 3) % 3 - 1, S / 9 - 1};
  const int dimo[3] = {mo.nx, mo.ny, mo.nz}, dimi[3] = {mi.nx, mi.ny, mi.nz};
  const int X = c[axis], JX = X + so[axis];
  bool live = X > 0 && X < dimo[axis] - 1 && JX > 0 && JX < dimo[axis] - 1;
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (d != axis && (c[d] + so[d] < 0 || c[d] + so[d] > dimo[d] - 1)) live = false;
  float acc[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) acc[q] = 0.f;
  if (live) {
    const size_t npi = mi.np;
#pragma unroll
    for (int a = -1; a <= 1; ++a) {
      const int ix = 2 * X + a;
      if (ix <= 0 || ix >= dimi[axis] - 1) continue;
      int f[3] = {c[0], c[1], c[2]};
      f[axis] = ix;
      const int i = f[0] + mi.nx * (f[1] + mi.ny * f[2]);
#pragma unroll
      for (int o = -1; o <= 1; ++o) {
        const int jx = ix + o, e = jx - 2 * JX;
        if (e < -1 || e > 1 || jx <= 0 || jx >= dimi[axis] - 1) continue;
        int off[3] = {so[0], so[1], so[2]};
        off[axis] = o;
        const int sf = (off[2] + 1) * 9 + (off[1] + 1) * 3 + (off[0] + 1);
        const float w = half_pow(a) * half_pow(e);
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q] = fmaf(w, __ldg(A + (size_t)(sf * 9 + q) * npi + i), acc[q]);
      }
    }
  }
  if (dst == 3 && S == 13) {
    int i, j, k;
    if (on_boundary(mo, io, i, j, k)) acc[0] = acc[4] = acc[8] = 1.f;
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) B[(size_t)(S * 9 + q) * mo.np + io] = acc[q];
}

// Inverse of the safeguarded smoother diagonal of level l, per row (n, d):
//   1 / max(a_dd / omega, c * sum_j |a_dj|)
// over the row's interior columns (boundary columns are eliminated by the Dirichlet rows; coarse operators hold
// zeros there).  Boundary rows get 1.
__global__ void __launch_bounds__(kMgBlock) k_mg_sdiag(MeshDev m, const Inst *insts, const int *list, int l,
                                                       float omega, float c) {
  const Inst &I = insts[list[blockIdx.y]];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  const float *__restrict__ vals = (l == 0) ? I.vals32 : I.mg->lv[l].vals;
  float *__restrict__ kinv = I.mg->lv[l].kinv;
  int i, j, k;
  if (on_boundary(m, n, i, j, k)) {
#pragma unroll
    for (int d = 0; d < 3; ++d) kinv[(size_t)n * 3 + d] = 1.f;
    return;
  }
  const size_t np = m.np;
  float l1[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
  for (int s = 0; s < 27; ++s) {
    const int nb = n + (s / 9 - 1) * m.nxny + ((s / 3) % 3 - 1) * m.nx + (s % 3 - 1);
    int bi, bj, bk;
    if (on_boundary(m, nb, bi, bj, bk)) continue;
#pragma unroll
    for (int fi = 0; fi < 3; ++fi)
#pragma unroll
      for (int fj = 0; fj < 3; ++fj) l1[fi] += fabsf(vals[(size_t)(s * 9 + fi * 3 + fj) * np + n]);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float dg = vals[(size_t)(13 * 9 + d * 4) * np + n];
    kinv[(size_t)n * 3 + d] = 1.f / fmaxf(dg / omega, c * l1[d]);
  }
}

// t_l = b_l - A_l x_l (zero on boundary nodes); HALF (level 0): A from the FP16 copy.
template <int NR, bool RM, bool STREAM, bool HALF = false>
__global__ void __launch_bounds__(kMgBlock) k_mg_resid(MeshDev m, const Inst *insts, const int *list, int l) {
  const Inst &I = insts[list[blockIdx.y]];
  if (inst_done<NR>(I)) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  const LvView v = view<NR>(I, l);
  const size_t np = m.np;
  int i, j, k;
  if (on_boundary(m, n, i, j, k)) {
#pragma unroll
    for (int r = 0; r < NR; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) v.t[vix<RM>(r, d, n, np)] = 0.f;
    return;
  }
  float y[NR * 3];
  if constexpr (HALF)
    apply_node_h<NR, RM>(m, I.mg->vals16, I.mg->inv16, v.x, n, y);
  else
    apply_node<NR, RM, STREAM>(m, v.vals, v.x, n, y);
#pragma unroll
  for (int r = 0; r < NR; ++r)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const size_t q = vix<RM>(r, d, n, np);
      v.t[q] = v.b[q] - y[r * 3 + d];
    }
}

// b_{l+1} = P^T t_l; x_{l+1} = w D^-1 b_{l+1} (zero on coarse boundary nodes).  One thread per coarse node.
template <int NR, bool RMF>
__global__ void __launch_bounds__(kMgBlock) k_mg_restrict(MeshDev mf, MeshDev mc, const Inst *insts, const int *list,
                                                          int lf, float omega) {
  const Inst &I = insts[list[blockIdx.y]];
  if (inst_done<NR>(I)) return;
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic >= mc.nn) return;
  const LvView f = view<NR>(I, lf);
  const MgLevel &C = I.mg->lv[lf + 1];
  const size_t npc = mc.np, npf = mf.np;
  int X, Y, Z;
  if (on_boundary(mc, ic, X, Y, Z)) {
#pragma unroll
    for (int c = 0; c < NR * 3; ++c) {
      C.b[(size_t)c * npc + ic] = 0.f;
      C.x[(size_t)c * npc + ic] = 0.f;
    }
    return;
  }
  float acc[NR * 3];
#pragma unroll
  for (int c = 0; c < NR * 3; ++c) acc[c] = 0.f;
#pragma unroll 1
  for (int a = 0; a < 27; ++a) {
    const int ax = a % 3 - 1, ay = (a / 3) % 3 - 1, az = a / 9 - 1;
    const int i = ((2 * Z + az) * mf.ny + (2 * Y + ay)) * mf.nx + (2 * X + ax);
    const float w = half_pow(ax) * half_pow(ay) * half_pow(az);
#pragma unroll
    for (int r = 0; r < NR; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) acc[r * 3 + d] = fmaf(w, f.t[vix<RMF>(r, d, i, npf)], acc[r * 3 + d]);
  }
  float kd[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) kd[d] = C.kinv[(size_t)ic * 3 + d];
#pragma unroll
  for (int r = 0; r < NR; ++r)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const size_t q = (size_t)(r * 3 + d) * npc + ic;
      C.b[q] = acc[r * 3 + d];
      C.x[q] = omega * kd[d] * acc[r * 3 + d];
    }
}

// t_l = x_l + P x_{l+1} on interior fine nodes (zero on boundary nodes).
template <int NR, bool RMF>
__global__ void __launch_bounds__(kMgBlock) k_mg_prolong(MeshDev mf, MeshDev mc, const Inst *insts, const int *list,
                                                         int lf) {
  const Inst &I = insts[list[blockIdx.y]];
  if (inst_done<NR>(I)) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= mf.nn) return;
  const LvView f = view<NR>(I, lf);
  const float *__restrict__ xc = I.mg->lv[lf + 1].x;
  const size_t npf = mf.np, npc = mc.np;
  int i, j, k;
  if (on_boundary(mf, n, i, j, k)) {
#pragma unroll
    for (int r = 0; r < NR; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) f.t[vix<RMF>(r, d, n, npf)] = 0.f;
    return;
  }
  // coarse parents along each axis: even index -> (i / 2, 1); odd -> ((i - 1) / 2, 1/2), ((i + 1) / 2, 1/2)
  const int px0 = i >> 1, px1 = (i + 1) >> 1, py0 = j >> 1, py1 = (j + 1) >> 1, pz0 = k >> 1, pz1 = (k + 1) >> 1;
  const float wx = (i & 1) ? 0.5f : 1.f, wy = (j & 1) ? 0.5f : 1.f, wz = (k & 1) ? 0.5f : 1.f;
  const int nxo = (i & 1) ? 2 : 1, nyo = (j & 1) ? 2 : 1, nzo = (k & 1) ? 2 : 1;
  float acc[NR * 3];
#pragma unroll
  for (int r = 0; r < NR; ++r)
#pragma unroll
    for (int d = 0; d < 3; ++d) acc[r * 3 + d] = f.x[vix<RMF>(r, d, n, npf)];
  for (int cz = 0; cz < nzo; ++cz)
    for (int cy = 0; cy < nyo; ++cy)
      for (int cx = 0; cx < nxo; ++cx) {
        const int J = ((cz ? pz1 : pz0) * mc.ny + (cy ? py1 : py0)) * mc.nx + (cx ? px1 : px0);
        const float w = wx * wy * wz;
#pragma unroll
        for (int c = 0; c < NR * 3; ++c) acc[c] = fmaf(w, xc[(size_t)c * npc + J], acc[c]);
      }
#pragma unroll
  for (int r = 0; r < NR; ++r)
#pragma unroll
    for (int d = 0; d < 3; ++d) f.t[vix<RMF>(r, d, n, npf)] = acc[r * 3 + d];
}

// apply_node (component-major vectors) for an x that the same kernel wrote before a barrier: x is read through
// L2 (ld.global.cg), never through the read-only path.  The same products in the same order.
template <int NR>
__device__ __forceinline__ void apply_node_cg(const MeshDev &m, const float *__restrict__ vals, const float *x, int n,
                                              float (&y)[NR * 3]) {
  const size_t np = m.np;
#pragma unroll
  for (int c = 0; c < NR * 3; ++c) y[c] = 0.f;
#pragma unroll 3
  for (int s = 0; s < 27; ++s) {
    const int nb = n + (s / 9 - 1) * m.nxny + ((s / 3) % 3 - 1) * m.nx + (s % 3 - 1);
    float K[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) K[q] = __ldg(vals + (size_t)(s * 9 + q) * np + n);
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      float xv[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) xv[d] = __ldcg(x + vix<false>(r, d, nb, np));
#pragma unroll
      for (int fi = 0; fi < 3; ++fi)
#pragma unroll
        for (int fj = 0; fj < 3; ++fj) y[r * 3 + fi] = fmaf(K[fi * 3 + fj], xv[fj], y[r * 3 + fi]);
    }
  }
}

// out = in + w D^-1 (b - A in) at node n of level l >= 1 (zero on boundary nodes).  CG: `in` was written by the
// same kernel (k_mg_coarse_sweeps) and is read through L2.
template <int NR, bool CG>
__device__ __forceinline__ void jacobi_node(const MeshDev &m, const LvView &v, const float *in, float *out, int n,
                                            float omega) {
  const size_t np = m.np;
  int i, j, k;
  if (on_boundary(m, n, i, j, k)) {
#pragma unroll
    for (int c = 0; c < NR * 3; ++c) out[(size_t)c * np + n] = 0.f;
    return;
  }
  float y[NR * 3];
  if constexpr (CG)
    apply_node_cg<NR>(m, v.vals, in, n, y);
  else
    apply_node<NR, false, false>(m, v.vals, in, n, y);
#pragma unroll
  for (int r = 0; r < NR; ++r)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const size_t q = (size_t)(r * 3 + d) * np + n;
      const float xin = CG ? __ldcg(in + q) : in[q];
      out[q] = fmaf(omega * v.kinv[(size_t)n * 3 + d], v.b[q] - y[r * 3 + d], xin);
    }
}

// One Jacobi sweep on level l >= 1; in/out select x, y or t.
template <int NR>
__global__ void __launch_bounds__(kMgBlock) k_mg_jacobi(MeshDev m, const Inst *insts, const int *list, int l,
                                                        int src, int dst, float omega) {
  const Inst &I = insts[list[blockIdx.y]];
  if (inst_done<NR>(I)) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  const LvView v = view<NR>(I, l);
  jacobi_node<NR, false>(m, v, pick(v, src), pick(v, dst), n, omega);
}

// The coarsest level's Jacobi sweeps in one block per instance: `pairs` pairs x -> y -> x, each sweep the
// arithmetic of k_mg_jacobi (so the result is the same bit for bit), the block's barrier between sweeps.  For
// levels of at most kMgCoarseNodes nodes, where a launch per sweep costs more than the sweep.
template <int NR>
__global__ void __launch_bounds__(kMgCoarseBlock) k_mg_coarse_sweeps(MeshDev m, const Inst *insts, const int *list,
                                                                     int l, int pairs, float omega) {
  const Inst &I = insts[list[blockIdx.y]];
  if (inst_done<NR>(I)) return;
  const LvView v = view<NR>(I, l);
  for (int p = 0; p < 2 * pairs; ++p) {
    const float *in = (p & 1) ? v.y : v.x;
    float *out = (p & 1) ? v.x : v.y;
    for (int n = threadIdx.x; n < m.nn; n += blockDim.x) jacobi_node<NR, true>(m, v, in, out, n, omega);
    __syncthreads();
  }
}

// k_mg_coarse_sweeps with the level in shared memory: the operator (243 np floats), x, y, b (NR * 3 * np each)
// and the inverse diagonal (3 np) are loaded once, every sweep reads them there, and x goes back at the end.
// The products and sums are those of jacobi_node in the same order, so x is the same bit for bit.
template <int NR>
__global__ void __launch_bounds__(kMgCoarseBlock) k_mg_coarse_sweeps_smem(MeshDev m, const Inst *insts,
                                                                          const int *list, int l, int pairs,
                                                                          float omega) {
  extern __shared__ float sm[];
  const Inst &I = insts[list[blockIdx.y]];
  if (inst_done<NR>(I)) return;
  const LvView v = view<NR>(I, l);
  const size_t np = m.np, nv = (size_t)NR * 3 * np;
  float *A = sm, *xs = A + (size_t)kEllPerNode * np, *ys = xs + nv, *bs = ys + nv, *kd = bs + nv;
  for (size_t t = threadIdx.x; t < (size_t)kEllPerNode * np; t += blockDim.x) A[t] = __ldg(v.vals + t);
  for (size_t t = threadIdx.x; t < nv; t += blockDim.x) {
    xs[t] = v.x[t];
    ys[t] = 0.f;
    bs[t] = v.b[t];
  }
  for (size_t t = threadIdx.x; t < (size_t)3 * m.nn; t += blockDim.x) kd[t] = v.kinv[t];
  __syncthreads();
  for (int p = 0; p < 2 * pairs; ++p) {
    const float *in = (p & 1) ? ys : xs;
    float *out = (p & 1) ? xs : ys;
    for (int n = threadIdx.x; n < m.nn; n += blockDim.x) {
      int i, j, k;
      if (on_boundary(m, n, i, j, k)) {
#pragma unroll
        for (int c = 0; c < NR * 3; ++c) out[(size_t)c * np + n] = 0.f;
        continue;
      }
      float y[NR * 3];
#pragma unroll
      for (int c = 0; c < NR * 3; ++c) y[c] = 0.f;
#pragma unroll 3
      for (int s = 0; s < 27; ++s) {
        const int nb = n + (s / 9 - 1) * m.nxny + ((s / 3) % 3 - 1) * m.nx + (s % 3 - 1);
        float K[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) K[q] = A[(size_t)(s * 9 + q) * np + n];
#pragma unroll
        for (int r = 0; r < NR; ++r) {
          float xv[3];
#pragma unroll
          for (int d = 0; d < 3; ++d) xv[d] = in[(size_t)(r * 3 + d) * np + nb];
#pragma unroll
          for (int fi = 0; fi < 3; ++fi)
#pragma unroll
            for (int fj = 0; fj < 3; ++fj) y[r * 3 + fi] = fmaf(K[fi * 3 + fj], xv[fj], y[r * 3 + fi]);
        }
      }
#pragma unroll
      for (int r = 0; r < NR; ++r)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const size_t q = (size_t)(r * 3 + d) * np + n;
          out[q] = fmaf(omega * kd[(size_t)n * 3 + d], bs[q] - y[r * 3 + d], in[q]);
        }
    }
    __syncthreads();
  }
  for (size_t t = threadIdx.x; t < nv; t += blockDim.x) v.x[t] = xs[t];
}

// Bytes of shared memory k_mg_coarse_sweeps_smem needs on a level of np padded nodes.
static size_t coarse_smem_bytes(size_t np, int nr) { return ((size_t)kEllPerNode + 9 * (size_t)nr + 3) * np * 4; }

// The CG scalars after the level-0 post-smoother (last block of the instance, thread 0): setup sets rz, an
// iteration beta and rz, for the right-hand sides still iterating.
template <int NR>
__device__ __forceinline__ void post0_scalars(const Inst &I, const double (&tot)[NR], int setup) {
  if (NR == 1) {
    CgState *c = I.cg;
    if (!setup) c->beta = tot[0] / c->rz;
    c->rz = tot[0];
    if (!isfinite(tot[0])) {
      c->done = 1;
      I.out->nonfinite = 1;
      I.out->cg_its = c->its;
    }
  } else {
    Cg6State *c = I.cg6;
    for (int r = 0; r < NR; ++r) {
      if (c->done[r]) continue;
      if (!setup) c->beta[r] = tot[r] / c->rz[r];
      c->rz[r] = tot[r];
      if (!isfinite(tot[r])) c->done[r] = 1;
    }
    int all = 1;
    for (int r = 0; r < NR; ++r) all &= c->done[r];
    c->all_done = all;
    if (all) I.out->cg6_its = c->its;
  }
}

// Level-0 post-smoother and the CG scalars: z = t0 + w D^-1 (r - A t0), rz_i = sum r.z.  setup: p = z and
// rz = rz_i (start of a solve); otherwise beta = rz_i / rz, rz = rz_i (right-hand sides still iterating).
template <int NR, bool RM, bool HALF = false>
__global__ void __launch_bounds__(kMgBlock) k_mg_post0(MeshDev m, const Inst *insts, const int *list, float omega,
                                                       int setup) {
  const Inst &I = insts[list[blockIdx.y]];
  if (inst_done<NR>(I)) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  float acc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] = 0.f;
  if (n < m.nn) {
    const LvView v = view<NR>(I, 0);
    float *__restrict__ p = NR == 1 ? I.p32 : I.P6;
    const size_t np = m.np;
    int i, j, k;
    const bool bn = on_boundary(m, n, i, j, k);
    float y[NR * 3];
    if (!bn) {
      if constexpr (HALF)
        apply_node_h<NR, RM>(m, I.mg->vals16, I.mg->inv16, v.t, n, y);
      else
        apply_node<NR, RM, true>(m, v.vals, v.t, n, y);
    }
#pragma unroll
    for (int r = 0; r < NR; ++r)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const size_t q = vix<RM>(r, d, n, np);
        const float rv = v.b[q];
        const float z = bn ? 0.f : fmaf(omega * v.kinv[(size_t)n * 3 + d], rv - y[r * 3 + d], v.t[q]);
        v.x[q] = z;
        if (setup) p[q] = z;
        acc[r] = fmaf(rv, z, acc[r]);
      }
  }
  double tot[NR];
  if (grid_sum_f<NR>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) post0_scalars<NR>(I, tot, setup);
}

// Level-0 residual of the 6-RHS V-cycle with the structure of the tangent CG's SpMV: two consecutive nodes per
// thread (n0 even; np is a multiple of 32, so each ELL entry of the pair is one 8-byte load), the 4 neighbours
// of a pair row along x loaded once for the 3 x-slots, neighbour indices clamped into the grid (the sums of
// boundary nodes are discarded).  Same products and order per row as apply_node.  Held to 128 registers (512
// threads per SM), the residency of the tangent CG's SpMV.
template <bool HALF>
__device__ __forceinline__ void apply_pair6(const MeshDev &m, const float *__restrict__ vals,
                                            const unsigned short *__restrict__ vals16, float inv,
                                            const float *__restrict__ x, int n0, float (&y)[2][18]) {
  const size_t np = m.np, np2 = np / 2;
  const float2 *__restrict__ v2 = reinterpret_cast<const float2 *>(vals + n0);
  const unsigned int *__restrict__ h2 = reinterpret_cast<const unsigned int *>(vals16 + n0);
  const int last = m.nn - 1;
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int c = 0; c < 18; ++c) y[q][c] = 0.f;
#pragma unroll 1
  for (int zy = 0; zy < 9; ++zy) {
    const int base = n0 + (zy / 3 - 1) * m.nxny + (zy % 3 - 1) * m.nx - 1;
    int nb[4];
#pragma unroll
    for (int w = 0; w < 4; ++w) nb[w] = min(max(base + w, 0), last);
    float2 a[3][9];
#pragma unroll
    for (int dx = 0; dx < 3; ++dx)
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        const size_t o = (size_t)((zy * 3 + dx) * 9 + e) * np2;
        if constexpr (HALF)
          a[dx][e] = ld_h2(h2 + o);
        else
          a[dx][e] = __ldcs(v2 + o);
      }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      float xv[4][3];
#pragma unroll
      for (int w = 0; w < 4; ++w)
#pragma unroll
        for (int d = 0; d < 3; ++d) xv[w][d] = x[(size_t)(r * 3 + d) * np + nb[w]];
#pragma unroll
      for (int dx = 0; dx < 3; ++dx)
#pragma unroll
        for (int e = 0; e < 9; ++e) {
          const int fi = e / 3, fj = e % 3;
          y[0][r * 3 + fi] = fmaf(a[dx][e].x, xv[dx][fj], y[0][r * 3 + fi]);
          y[1][r * 3 + fi] = fmaf(a[dx][e].y, xv[1 + dx][fj], y[1][r * 3 + fi]);
        }
    }
  }
  if constexpr (HALF) {
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int c = 0; c < 18; ++c) y[q][c] *= inv;
  }
}

// t0 = r - A x0 for the 6 right-hand sides (zero on boundary nodes), two nodes per thread.
template <int B, bool HALF>
__global__ void __launch_bounds__(B, 512 / B) k_mg_resid6(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  if (I.cg6->all_done) return;
  const int n0 = (blockIdx.x * B + threadIdx.x) * 2;
  if (n0 >= m.nn) return;
  const LvView v = view<6>(I, 0);
  const size_t np = m.np;
  bool bn[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    int i, j, k;
    bn[q] = (n0 + q >= m.nn) || on_boundary(m, n0 + q, i, j, k);
  }
  float y[2][18];
  if (!bn[0] || !bn[1]) apply_pair6<HALF>(m, v.vals, I.mg->vals16, I.mg->inv16, v.x, n0, y);
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int n = n0 + q;
    if (n >= m.nn) break;
#pragma unroll
    for (int c = 0; c < 18; ++c) {
      const size_t idx = (size_t)c * np + n;
      v.t[idx] = bn[q] ? 0.f : v.b[idx] - y[q][c];
    }
  }
}

// Level-0 post-smoother of the 6-RHS V-cycle with the pair structure of k_mg_resid6: z = t0 + w D^-1 (r - A t0)
// and rz_i = sum r.z for two consecutive nodes per thread; setup: p = z.  The CG scalars as in k_mg_post0.
// Bounded to 512 threads per SM like k_mg_resid6 (128 registers; a few words spill to L1): at one 256-thread
// block per SM its loads had too little parallelism.
template <int B, bool HALF>
__global__ void __launch_bounds__(B, 512 / B) k_mg_post06(MeshDev m, const Inst *insts, const int *list,
                                                          float omega, int setup) {
  const Inst &I = insts[list[blockIdx.y]];
  if (I.cg6->all_done) return;
  const int n0 = (blockIdx.x * B + threadIdx.x) * 2;
  float acc[6];
#pragma unroll
  for (int r = 0; r < 6; ++r) acc[r] = 0.f;
  if (n0 < m.nn) {
    const LvView v = view<6>(I, 0);
    float *__restrict__ p = I.P6;
    const size_t np = m.np;
    bool bn[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      int i, j, k;
      bn[q] = (n0 + q >= m.nn) || on_boundary(m, n0 + q, i, j, k);
    }
    float y[2][18];
    if (!bn[0] || !bn[1]) apply_pair6<HALF>(m, v.vals, I.mg->vals16, I.mg->inv16, v.t, n0, y);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int n = n0 + q;
      if (n >= m.nn) break;
      float kd[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) kd[d] = omega * v.kinv[(size_t)n * 3 + d];
#pragma unroll
      for (int c = 0; c < 18; ++c) {
        const size_t idx = (size_t)c * np + n;
        const float rv = v.b[idx];
        const float z = bn[q] ? 0.f : fmaf(kd[c % 3], rv - y[q][c], v.t[idx]);
        v.x[idx] = z;
        if (setup) p[idx] = z;
        acc[c / 3] = fmaf(rv, z, acc[c / 3]);
      }
    }
  }
  double tot[6];
  if (grid_sum_f<6>(acc, I.red, I.ticket, gridDim.x, tot) && threadIdx.x == 0) post0_scalars<6>(I, tot, setup);
}

// The FP16 copy of the level-0 operator: vals16 = fp16(scale16 x vals32), four entries per thread and step
// (243 np entries, np a multiple of 32), clamped to the FP16 range.
__global__ void __launch_bounds__(256) k_mg_half0(MeshDev m, const Inst *insts, const int *list) {
  const Inst &I = insts[list[blockIdx.y]];
  const MgInst &G = *I.mg;
  const size_t count4 = (size_t)kEllPerNode * m.np / 4;
  const float s = G.scale16;
  const float4 *__restrict__ src = reinterpret_cast<const float4 *>(I.vals32);
  uint2 *__restrict__ dst = reinterpret_cast<uint2 *>(G.vals16);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count4; i += (size_t)gridDim.x * blockDim.x) {
    const float4 v = __ldcs(src + i);
    const float c[4] = {v.x, v.y, v.z, v.w};
    unsigned short h[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) h[k] = __half_as_ushort(__float2half_rn(fminf(fmaxf(c[k] * s, -65504.f), 65504.f)));
    dst[i] = make_uint2((unsigned)h[0] | ((unsigned)h[1] << 16), (unsigned)h[2] | ((unsigned)h[3] << 16));
  }
}

inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

template <bool HALF>
void launch_resid6(const MeshDev *m, const Inst *insts, const int *list, int nlist, int block, cudaStream_t s) {
  const size_t pairs = cdiv(m->nn, 2);
  if (block == 64)
    k_mg_resid6<64, HALF><<<dim3(cdiv(pairs, 64), nlist), 64, 0, s>>>(*m, insts, list);
  else if (block == 256)
    k_mg_resid6<256, HALF><<<dim3(cdiv(pairs, 256), nlist), 256, 0, s>>>(*m, insts, list);
  else
    k_mg_resid6<128, HALF><<<dim3(cdiv(pairs, 128), nlist), 128, 0, s>>>(*m, insts, list);
}

// two nodes per thread: at most cdiv(nn, 128) blocks, the reduction partials' capacity
template <bool HALF>
void launch_post06(const MeshDev *m, const Inst *insts, const int *list, int nlist, float omega, int setup, int block,
                   cudaStream_t s) {
  const size_t pairs = cdiv(m->nn, 2);
  if (block == 64)
    k_mg_post06<64, HALF><<<dim3(cdiv(pairs, 64), nlist), 64, 0, s>>>(*m, insts, list, omega, setup);
  else if (block == 256)
    k_mg_post06<256, HALF><<<dim3(cdiv(pairs, 256), nlist), 256, 0, s>>>(*m, insts, list, omega, setup);
  else
    k_mg_post06<128, HALF><<<dim3(cdiv(pairs, 128), nlist), 128, 0, s>>>(*m, insts, list, omega, setup);
}

}  // namespace
}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_launch_mg_rap1(const MeshDev *mi, const MeshDev *mo, const Inst *insts, const int *list, int nlist, int lf,
                       int axis, int src, int dst, cudaStream_t s) {
  if (nlist <= 0) return 0;
  if (axis < 0 || axis > 2 || src < 0 || src > 2 || dst < 1 || dst > 3 || src == dst) return (int)cudaErrorInvalidValue;
  k_mg_rap1<<<dim3(cdiv((size_t)27 * mo->nn, kMgBlock), nlist), kMgBlock, 0, s>>>(*mi, *mo, insts, list, lf, axis, src,
                                                                               dst);
  return (int)cudaGetLastError();
}

int mgb_launch_mg_sdiag(const MeshDev *m, const Inst *insts, const int *list, int nlist, int l, float omega,
                        float c, cudaStream_t s) {
  if (nlist <= 0) return 0;
  k_mg_sdiag<<<dim3(cdiv(m->nn, kMgBlock), nlist), kMgBlock, 0, s>>>(*m, insts, list, l, omega, c);
  return (int)cudaGetLastError();
}

int mgb_launch_mg_half0(const MeshDev *m, const Inst *insts, const int *list, int nlist, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const size_t count4 = (size_t)kEllPerNode * m->np / 4;
  const unsigned blocks = (unsigned)std::min<size_t>(cdiv(count4, 256), 1216);
  k_mg_half0<<<dim3(blocks, nlist), 256, 0, s>>>(*m, insts, list);
  return (int)cudaGetLastError();
}

int mgb_launch_mg_resid(const MeshDev *m, const Inst *insts, const int *list, int nlist, int nr, int l, int block,
                        int half, cudaStream_t s) {
  if (nlist <= 0) return 0;
  if (nr == 6 && l == 0) {
    if (half)
      launch_resid6<true>(m, insts, list, nlist, block, s);
    else
      launch_resid6<false>(m, insts, list, nlist, block, s);
    return (int)cudaGetLastError();
  }
  const dim3 g(cdiv(m->nn, kMgBlock), nlist);
  if (nr == 1) {
    if (l == 0 && half)
      k_mg_resid<1, true, true, true><<<g, kMgBlock, 0, s>>>(*m, insts, list, l);
    else if (l == 0)
      k_mg_resid<1, true, true><<<g, kMgBlock, 0, s>>>(*m, insts, list, l);
    else
      k_mg_resid<1, false, false><<<g, kMgBlock, 0, s>>>(*m, insts, list, l);
  } else {
    k_mg_resid<6, false, false><<<g, kMgBlock, 0, s>>>(*m, insts, list, l);
  }
  return (int)cudaGetLastError();
}

int mgb_launch_mg_restrict(const MeshDev *mf, const MeshDev *mc, const Inst *insts, const int *list, int nlist,
                           int nr, int lf, float omega, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const dim3 g(cdiv(mc->nn, kMgBlock), nlist);
  if (nr == 1) {
    if (lf == 0)
      k_mg_restrict<1, true><<<g, kMgBlock, 0, s>>>(*mf, *mc, insts, list, lf, omega);
    else
      k_mg_restrict<1, false><<<g, kMgBlock, 0, s>>>(*mf, *mc, insts, list, lf, omega);
  } else {
    k_mg_restrict<6, false><<<g, kMgBlock, 0, s>>>(*mf, *mc, insts, list, lf, omega);
  }
  return (int)cudaGetLastError();
}

int mgb_launch_mg_prolong(const MeshDev *mf, const MeshDev *mc, const Inst *insts, const int *list, int nlist,
                          int nr, int lf, cudaStream_t s) {
  if (nlist <= 0) return 0;
  const dim3 g(cdiv(mf->nn, kMgBlock), nlist);
  if (nr == 1) {
    if (lf == 0)
      k_mg_prolong<1, true><<<g, kMgBlock, 0, s>>>(*mf, *mc, insts, list, lf);
    else
      k_mg_prolong<1, false><<<g, kMgBlock, 0, s>>>(*mf, *mc, insts, list, lf);
  } else {
    k_mg_prolong<6, false><<<g, kMgBlock, 0, s>>>(*mf, *mc, insts, list, lf);
  }
  return (int)cudaGetLastError();
}

int mgb_mg_init_attributes() {
  int e = (int)cudaFuncSetAttribute(k_mg_coarse_sweeps_smem<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kMgCoarseSmem);
  if (e) return e;
  return (int)cudaFuncSetAttribute(k_mg_coarse_sweeps_smem<6>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   kMgCoarseSmem);
}

int mgb_launch_mg_coarse_sweeps(const MeshDev *m, const Inst *insts, const int *list, int nlist, int nr, int l,
                                int pairs, float omega, cudaStream_t s) {
  if (nlist <= 0 || pairs <= 0) return 0;
  if (l < 1 || m->nn > kMgCoarseNodes) return (int)cudaErrorInvalidValue;
  const dim3 g(1, nlist);
  const size_t smem = coarse_smem_bytes(m->np, nr);
  if (smem <= (size_t)kMgCoarseSmem) {
    if (nr == 1)
      k_mg_coarse_sweeps_smem<1><<<g, kMgCoarseBlock, smem, s>>>(*m, insts, list, l, pairs, omega);
    else
      k_mg_coarse_sweeps_smem<6><<<g, kMgCoarseBlock, smem, s>>>(*m, insts, list, l, pairs, omega);
  } else if (nr == 1) {
    k_mg_coarse_sweeps<1><<<g, kMgCoarseBlock, 0, s>>>(*m, insts, list, l, pairs, omega);
  } else {
    k_mg_coarse_sweeps<6><<<g, kMgCoarseBlock, 0, s>>>(*m, insts, list, l, pairs, omega);
  }
  return (int)cudaGetLastError();
}

int mgb_launch_mg_jacobi(const MeshDev *m, const Inst *insts, const int *list, int nlist, int nr, int l, int src,
                         int dst, float omega, cudaStream_t s) {
  if (nlist <= 0) return 0;
  if (l < 1 || src < 0 || src > 2 || dst < 0 || dst > 2 || src == dst) return (int)cudaErrorInvalidValue;
  const dim3 g(cdiv(m->nn, kMgBlock), nlist);
  if (nr == 1)
    k_mg_jacobi<1><<<g, kMgBlock, 0, s>>>(*m, insts, list, l, src, dst, omega);
  else
    k_mg_jacobi<6><<<g, kMgBlock, 0, s>>>(*m, insts, list, l, src, dst, omega);
  return (int)cudaGetLastError();
}

int mgb_launch_mg_post0(const MeshDev *m, const Inst *insts, const int *list, int nlist, int nr, float omega,
                        int setup, int block, int half, cudaStream_t s) {
  if (nlist <= 0) return 0;
  if (nr == 6) {
    if (half)
      launch_post06<true>(m, insts, list, nlist, omega, setup, block, s);
    else
      launch_post06<false>(m, insts, list, nlist, omega, setup, block, s);
    return (int)cudaGetLastError();
  }
  const dim3 g(cdiv(m->nn, kMgBlock), nlist);
  if (half)
    k_mg_post0<1, true, true><<<g, kMgBlock, 0, s>>>(*m, insts, list, omega, setup);
  else
    k_mg_post0<1, true><<<g, kMgBlock, 0, s>>>(*m, insts, list, omega, setup);
  return (int)cudaGetLastError();
}

}  // extern "C"
