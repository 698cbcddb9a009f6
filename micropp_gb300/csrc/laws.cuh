// laws.cuh -- Gauss-point material laws on the device (FP64).
//
// Elastic, J2 plasticity with linear isotropic hardening and the scalar damage law of the reference
// (material.cpp:48-307), evaluated per Gauss point with the history layout of params.hpp:41
// (J2: eps_p[6], alpha; damage: r, D).  A NULL history pointer reads as zeros, which is how the reference
// treats a Gauss point that has never been nonlinear.
#pragma once

#include "device.cuh"

namespace mgb {

#define MGB_SQRT_2DIV3 0.816496581  // truncated constant of material_base.h:30
#define MGB_D_EPS_CTAN 1.0e-8       // material_base.h:29

__device__ __forceinline__ void law_elastic(const MatDev &m, const double *eps, double *s) {
  const double tr = eps[0] + eps[1] + eps[2];
#pragma unroll
  for (int i = 0; i < 3; ++i) s[i] = m.lambda * tr + m.two_mu * eps[i];
#pragma unroll
  for (int i = 3; i < 6; ++i) s[i] = m.mu * eps[i];
}

// Trial state of the radial return (material.cpp:110-147).  Returns true when the trial stress is outside
// the yield surface; dl is the plastic multiplier and normal the flow direction.
__device__ __forceinline__ bool law_j2_trial(const MatDev &m, const double *eps, const double *vars, double *dl,
                                             double *normal, double *s_trial) {
  const double third = 1 / 3.0;
  const double alpha_old = vars ? vars[6] : 0.0;
  double ep[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) ep[i] = vars ? vars[i] : 0.0;
  const double tr_p = third * (ep[0] + ep[1] + ep[2]);
  const double tr_e = third * (eps[0] + eps[1] + eps[2]);
  double tmp = 0.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const double de = (i < 3) ? eps[i] - tr_e : eps[i];
    const double dp = (i < 3) ? ep[i] - tr_p : ep[i];
    s_trial[i] = (i < 3) ? m.two_mu * (de - dp) : m.mu * (de - dp);
    tmp += s_trial[i] * s_trial[i];
  }
  const double s_norm = sqrt(tmp);
  const double f = s_norm - MGB_SQRT_2DIV3 * (m.Sy + m.Ka * alpha_old);
  if (f > 0) {
#pragma unroll
    for (int i = 0; i < 6; ++i) normal[i] = s_trial[i] / s_norm;
    *dl = f / m.pl_den;
    return true;
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) normal[i] = 0.0;
  *dl = 0.0;
  return false;
}

__device__ __forceinline__ double law_damage_hardening(const MatDev &m, double r) {
  if (r < m.dmg_r0) return 0.0;
  if (r < m.dmg_r1) return m.dmg_q0 + 10.0 * (r - m.dmg_r0);
  return m.dmg_q1 + 5.0 * (r - m.dmg_r1);
}

// damage_law (material.cpp:227-268): writes the undamaged stress into s, returns the loading flag.
__device__ __forceinline__ bool law_damage(const MatDev &m, const double *eps, double r_old, double D_old,
                                           double *r_out, double *D_out, double *s) {
  law_elastic(m, eps, s);
  double product = 0.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) product += s[i] * eps[i];
  const double r = (product >= 0) ? sqrt(product) : 0.0;
  const double r_old_a = (r_old < m.xt_thr) ? m.xt_thr : r_old;
  if (r <= r_old_a) {
    *r_out = r_old_a;
    *D_out = D_old;
    return false;
  }
  const double q = law_damage_hardening(m, r);
  *r_out = r;
  *D_out = 1. - q / r;
  return true;
}

// Damage law for the residual with the terms of its consistent tangent (the damage branch of law_ctan_exact):
// s holds the undamaged stress C eps on return, the damaged stress is (1 - D) s, and
// d sigma / d eps = a C + c s (x) s.
__device__ __forceinline__ void law_damage_terms(const MatDev &m, const double *eps, const double *vars, double *s,
                                                 double *D, double *a, double *c) {
  const double r_old = vars ? vars[0] : 0.0;
  const double D_old = vars ? vars[1] : 0.0;
  double r;
  const bool loading = law_damage(m, eps, r_old, D_old, &r, D, s);
  if (!loading) {
    *a = 1 - D_old;
    *c = 0.0;
    return;
  }
  const double q = law_damage_hardening(m, r);
  const double qp = (r < m.dmg_r0) ? 0.0 : (r < m.dmg_r1 ? 10.0 : 5.0);
  *a = q / r;
  *c = (qp - *a) / (r * r);
}

// get_stress of the three laws (material.cpp:76-82, 149-162, 270-284).
__device__ __forceinline__ void law_stress(const MatDev &m, const double *eps, const double *vars, double *s) {
  if (m.type == 0) {
    law_elastic(m, eps, s);
  } else if (m.type == 1) {
    double dl, normal[6], st[6];
    law_j2_trial(m, eps, vars, &dl, normal, st);
    const double tr = eps[0] + eps[1] + eps[2];
    const double g = m.two_mu * dl;
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = ((i < 3) ? st[i] + m.k * tr : st[i]) - g * normal[i];
  } else {
    const double r_old = vars ? vars[0] : 0.0;
    const double D_old = vars ? vars[1] : 0.0;
    double r, D;
    law_damage(m, eps, r_old, D_old, &r, &D, s);
    const double f = 1 - D;
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] *= f;
  }
}

// get_ctan (material.cpp:84-95 closed form for the elastic law; forward differences of the stress with
// step 1e-8 for J2 and damage, apply_perturbation material.cpp:48-63).  C is row-major 6x6.
__device__ __forceinline__ void law_ctan(const MatDev &m, const double *eps, const double *vars, double *C) {
  if (m.type == 0) {
#pragma unroll
    for (int i = 0; i < 36; ++i) C[i] = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) C[i * 6 + j] = m.lambda;
#pragma unroll
    for (int i = 0; i < 3; ++i) C[i * 6 + i] += m.two_mu;
#pragma unroll
    for (int i = 3; i < 6; ++i) C[i * 6 + i] = m.mu;
    return;
  }
  double s0[6];
  law_stress(m, eps, vars, s0);
#pragma unroll 1
  for (int i = 0; i < 6; ++i) {
    double e1[6], s1[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) e1[j] = eps[j];
    e1[i] += MGB_D_EPS_CTAN;
    law_stress(m, e1, vars, s1);
#pragma unroll
    for (int j = 0; j < 6; ++j) C[j * 6 + i] = (s1[j] - s0[j]) / MGB_D_EPS_CTAN;
  }
}

// Consistent tangent d(sigma)/d(eps) of the three laws in closed form -- the derivative that the reference's
// forward differences (apply_perturbation, material.cpp:48-63) approximate.  Used by the mixed form's Jacobian
// and by the implicit ctan, where it is both exact and far cheaper than 7 stress evaluations in FP64.
//  damage, unloading (r <= r_old_a): (1 - D_old) C
//  damage, loading:                  (q/r) C + (q' - q/r) / r^2 * s (x) s,   s = C eps, r = sqrt(s . eps)
//  J2, plastic:  D + K 1(x)1 - 2 mu [ n (x) (D n) / den + (dl / |s|) (I - n (x) n) D ]
//                with D = d(s_trial)/d(eps), n = s_trial / |s_trial| (the reference's Voigt norm),
//                dl = f / den, den = 2 mu (1 + Ka / (3 mu))
__device__ __forceinline__ void law_ctan_exact(const MatDev &m, const double *eps, const double *vars, double *C) {
  // elastic C (material.cpp:84-95)
#pragma unroll
  for (int i = 0; i < 36; ++i) C[i] = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i * 6 + j] = m.lambda;
#pragma unroll
  for (int i = 0; i < 3; ++i) C[i * 6 + i] += m.two_mu;
#pragma unroll
  for (int i = 3; i < 6; ++i) C[i * 6 + i] = m.mu;
  if (m.type == 0) return;
  if (m.type == 2) {
    double s[6];
    law_elastic(m, eps, s);
    double product = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) product += s[i] * eps[i];
    const double r = (product >= 0) ? sqrt(product) : 0.0;
    const double r_old = vars ? vars[0] : 0.0;
    const double D_old = vars ? vars[1] : 0.0;
    const double r_old_a = (r_old < m.xt_thr) ? m.xt_thr : r_old;
    if (r <= r_old_a) {
      const double f = 1 - D_old;
#pragma unroll
      for (int i = 0; i < 36; ++i) C[i] *= f;
      return;
    }
    const double q = law_damage_hardening(m, r);
    const double qp = (r < m.dmg_r0) ? 0.0 : (r < m.dmg_r1 ? 10.0 : 5.0);
    const double a = q / r;
    const double b = (qp - a) / (r * r);
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) C[i * 6 + j] = a * C[i * 6 + j] + b * s[i] * s[j];
    return;
  }
  // J2
  double dl, n[6], st[6];
  const bool plastic = law_j2_trial(m, eps, vars, &dl, n, st);
  // D = d(s_trial)/d(eps): 2 mu (I - 1/3 1(x)1) on the normal block, mu on the shear diagonal
  double D[36];
#pragma unroll
  for (int i = 0; i < 36; ++i) D[i] = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) D[i * 6 + j] = m.two_mu * ((i == j ? 1.0 : 0.0) - 1.0 / 3.0);
#pragma unroll
  for (int i = 3; i < 6; ++i) D[i * 6 + i] = m.mu;
#pragma unroll
  for (int i = 0; i < 36; ++i) C[i] = D[i];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i * 6 + j] += m.k;
  if (!plastic) return;
  double snorm = 0.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) snorm += st[i] * st[i];
  snorm = sqrt(snorm);
  double Dn[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) t += n[i] * D[i * 6 + j];
    Dn[j] = t;
  }
  const double c1 = m.two_mu / m.pl_den;
  const double c2 = m.two_mu * dl / snorm;
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      // (I - n n^T) D row i, column j = D_ij - n_i (n^T D)_j
      const double proj = D[i * 6 + j] - n[i] * Dn[j];
      C[i * 6 + j] -= c1 * n[i] * Dn[j] + c2 * proj;
    }
}

// evolute (material.cpp:97-100, 168-181, 291-302): history update, returns the nonlinear flag.  J2 writes
// only when the old history exists; damage always writes (r, D).
__device__ __forceinline__ bool law_evolve(const MatDev &m, const double *eps, const double *vold, bool has_old,
                                           double *vnew) {
  if (m.type == 0) return false;
  if (m.type == 1) {
    double dl, normal[6], st[6];
    const bool nl = law_j2_trial(m, eps, has_old ? vold : nullptr, &dl, normal, st);
    if (has_old) {
#pragma unroll
      for (int i = 0; i < 6; ++i) vnew[i] = vold[i] + dl * normal[i];
      vnew[6] = vold[6] + MGB_SQRT_2DIV3 * dl + 0;
    }
    return nl;
  }
  const double r_old = has_old ? vold[0] : 0.0;
  const double D_old = has_old ? vold[1] : 0.0;
  double r, D, s[6];
  const bool nl = law_damage(m, eps, r_old, D_old, &r, &D, s);
  vnew[0] = r;
  vnew[1] = D;
  return nl;
}

}  // namespace mgb
