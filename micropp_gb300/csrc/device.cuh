// device.cuh -- data layout shared by the host engine and the sm_103a kernels.
//
// One RVE is a structured grid of nx*ny*nz nodes on the unit cube with 3 displacement unknowns per node
// (row = node*3 + d, node = (k*ny + j)*nx + i, as in the reference, ell.hpp:37-39) and nex*ney*nez hex8
// elements with 8 Gauss points each (element e = (ez*ney + ey)*nex + ex, params.hpp:37).
//
// HBM layout per RVE instance ("slot" of the batch):
//   vectors u, du, b, r, z, p, Ap, kinv      nndim doubles each, node-interleaved (the reference layout)
//   ELL values                               243 * np values: entry (s, fi, fj) of node n at
//                                            [(s*9 + fi*3 + fj) * np + n], s = stencil slot 0..26 ordered
//                                            (dz,dy,dx) in {-1,0,1}^3 (ell-common.cpp:95-134).  Columns are
//                                            implicit; boundary rows are identity rows and are not stored.
//   element residual blocks be               24 * nelem doubles, [(a*3+d) * nelem + e]
//   internal variables                       7 doubles per Gauss point, [(e*8 + g)*7 + v] (params.hpp:41)
// Mixed form: the same ELL layout in FP32 (vals32) with FP32 CG vectors.  When every phase is elastic or
// damage, vals32 is assembled by node gather and also holds the real rows of the boundary nodes (the CG still
// treats them as identity rows); they give the ctan from the boundary reactions.  The rest of the mixed form: the six tangent right-hand sides
// of the implicit ctan are stored component-major, [(i*3 + d) * np + n] (18 * np values), so that a warp
// reading one component of 32 consecutive nodes touches 128 contiguous bytes.
#pragma once

#include <stddef.h>
#include <stdint.h>

#ifdef __CUDACC__
#define MGB_HD __host__ __device__ __forceinline__
#else
#define MGB_HD inline
#endif

namespace mgb {

constexpr int kNvoi = 6;
constexpr int kNpe = 8;
constexpr int kNvarGp = 7;
constexpr int kEllPerNode = 243;  // 27 stencil nodes x 3 x 3

struct MeshDev {
  int nx, ny, nz, nxny, nn, np;  // np: padded node stride of the ELL arrays
  int nex, ney, nez, nelem;
  double lx, ly, lz, dx, dy, dz, wg, vol_tot;
};

// A material with the constants its laws need precomputed on the host by the same expressions the
// reference evaluates at every call (material.cpp:205-225, 110-147), so the values are identical.
struct MatDev {
  double E, nu, Ka, Sy, k, mu, lambda, Xt;
  double two_mu;       // 2 * mu
  double xt_thr;       // Xt / sqrt(E)
  double dmg_r0, dmg_q0, dmg_q1, dmg_r1;
  double pl_den;       // 2. * mu * (1. + Ka / (3. * mu))
  int type;            // 0 elastic, 1 plastic (J2), 2 damage
  int pad;
};

struct Mats {
  MatDev m[3];
};

// Per-instance CG scalars, read and written only on the device.
struct CgState {
  double rz, pnorm0, pnorm, alpha, beta, pAp;
  double min_err, rel_err;
  int its, max_its, done, pad;
};

// Per-instance scalars of the 6-RHS tangent CG (one independent CG per right-hand side).
struct Cg6State {
  double rz[6], pnorm0[6], pnorm[6], alpha[6], beta[6];
  double min_err, rel_err;
  int its, max_its, done[6], all_done, pad;
};

// Small per-instance outputs read back by the host.
struct InstOut {
  double norm;         // ||b||_2 of the last residual evaluation
  double sig[6];       // volume-averaged stress of the last residual evaluation
  double ctan[36];     // implicit ctan (row-major, column i = d sigma / d eps_i)
  double res6[6];      // ||f_i - K x_i|| of the last tangent refinement residual
  double f6[6];        // ||f_i|| of the tangent right-hand sides
  int cg_its;          // iterations of the last CG solve
  int nonlinear;       // OR of the evolute flags of the last update pass
  int nonfinite;       // a reduction produced NaN/Inf
  int cg_maxed;        // the last CG solve stopped at max_its
  int cg6_its;         // iterations of the last 6-RHS CG solve
  int pad;
};

// Geometric multigrid hierarchy of one instance (mixed form).  Level 0 is the fine grid (the instance's vals32,
// kinv32 and CG vectors); level l >= 1 coarsens every axis of level l-1 to ceil(elements / 2).  A level's
// operator is the Galerkin product P^T A P in the fine grid's stencil ELL layout; its vectors hold up to 6
// right-hand sides component-major, v[(r * 3 + d) * np_l + n], and are zero on boundary nodes.
constexpr int kMgMaxLevels = 8;
// A coarsest multigrid level of at most this many nodes runs its Jacobi sweeps in one block per instance.
constexpr int kMgCoarseNodes = 1024;

struct MgLevel {
  float *vals;             // 243 * np_l (level >= 1)
  float *kinv;             // 3 * nn_l, node-interleaved; 1 on boundary rows
  float *b, *x, *y, *t;    // right-hand side, iterate, Jacobi ping-pong partner, residual / prolonged iterate
};

struct MgInst {
  MgLevel lv[kMgMaxLevels];
  float *mid1, *mid2;      // the separable Galerkin product's intermediate operators (x, then x and y coarsened)
  unsigned short *vals16;  // FP16 bits of scale16 x the level-0 operator (MICROPP3_PRECOND_MG_HALF), else NULL
  float scale16, inv16;    // a power of two and its inverse
  int pad[2];
};

struct Inst {
  double *u, *du, *b, *r, *z, *p, *Ap, *kinv, *vals, *be;
  const double *vars_old;  // NULL: every law reads zeros (the reference's nullptr history)
  double *vars_new;
  double *red;             // reduction partials, kRedStride doubles per block
  unsigned int *ticket;    // last-block counter for the reductions
  CgState *cg;
  InstOut *out;
  // mixed form (FP32 Jacobian and CG vectors)
  float *vals32, *kinv32, *r32, *z32, *p32, *Ap32, *du32;
  // Gauss-point tangent descriptors of the damage law for the symmetric FP32 Jacobian, written by the mixed
  // form's residual kernel: [(q * 8 + g) * nelem + e], q = 0: a, 1: c, 2..7: s  (C_gp = a C_el + c s s^T)
  float *gpd;
  // implicit ctan: 6 right-hand sides; X6 (solutions) and F6 (right-hand sides) as double-float pairs hi + lo
  float *X6h, *X6l, *F6h, *F6l;
  float *R6, *Z6, *P6, *AP6, *D6;
  Cg6State *cg6;
  MgInst *mg;              // multigrid hierarchy (NULL: Jacobi-preconditioned CG)
  double strain[6];
  int has_vars_old;        // J2 evolute writes only when a history buffer exists (material.cpp:168-181)
  int pad;
};

struct Voigt6 {
  double v[6];
};

// Scalars of one BiCGSTAB solve (the adjoint system), resident on the device.
struct BicgState {
  double rho, rho_old, alpha, omega, beta, r0, rnorm, rel_tol;
  int its, max_its, done, converged;
};

// Vectors and scratch of the adjoint solve of one RVE (node-interleaved FP64, like u).
struct AdjDev {
  double *x, *r, *rh, *p, *v, *s, *t, *y, *z, *kinv;
  const double *b, *vals;
  double *red;
  unsigned int *ticket;
  BicgState *st;
};

// One load step of the adjoint of a path (per-Gauss-point arrays in the history layout [(e*8+g)*7 + k]).
struct AdjStep {
  double g[6];          // dL / d(average stress) of the step
  double wgv;           // Gauss weight / RVE volume
  const double *mu_in;  // dL / d(history after the step), NULL for the last step
  double *mu_out;       // dL / d(history before the step)
  const double *lam;    // adjoint solution, node-interleaved
  double *out;          // 21 sums: dL/dtheta of the 3 phases x 5, then dL/d(macro strain) (6)
};

constexpr int kRedStride = 40;
constexpr int kNodeBlock = 256;
constexpr int kElemBlock = 128;

// Offset of component (i, d) of a 6-RHS vector.
MGB_HD size_t c6(int i, int d, size_t np) { return (size_t)(i * 3 + d) * np; }

}  // namespace mgb
