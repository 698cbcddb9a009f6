// adjoint_laws.h -- forward-mode derivatives of the Gauss-point laws, for the adjoint (VJP) of a load path.
//
// The laws of material.cpp:48-307 restated on a scalar type T that is either double or Dual (a value and
// one directional derivative), so one evaluation with one input seeded gives one column of the Jacobian of
// (stress, new history) with respect to (strain, old history, material parameters).  The operation order
// follows laws.cuh (the FP64 path); only the adjoint uses these copies, so the FP64 path keeps its own.
//
// Plain C++ templates usable from nvcc (device) and the host compiler (the CPU checks of the derivatives).
//
// Inputs of one Gauss point: eps[6] (Voigt, engineering shear), history h[7] (J2: eps_p[6], alpha;
// damage: r, D), parameters of its phase theta[5] = (E, nu, Xt, Sy, Ka).  Outputs: stress s[6] and the new
// history hn[7] (components a law does not update are copied from h).
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define MGB_ADJ_HD __host__ __device__ __forceinline__
#else
#define MGB_ADJ_HD inline
#endif

namespace mgb {
namespace adj {

constexpr int kNdir = 18;  // derivative directions: eps (6), history (7), parameters (5)
constexpr int kNpar = 5;   // E, nu, Xt, Sy, Ka

struct Dual {
  double v, d;
  MGB_ADJ_HD Dual() : v(0.0), d(0.0) {}
  MGB_ADJ_HD Dual(double a) : v(a), d(0.0) {}
  MGB_ADJ_HD Dual(double a, double b) : v(a), d(b) {}
};
MGB_ADJ_HD Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
MGB_ADJ_HD Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
MGB_ADJ_HD Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
MGB_ADJ_HD Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
MGB_ADJ_HD Dual operator/(Dual a, Dual b) { return Dual(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)); }
MGB_ADJ_HD Dual &operator+=(Dual &a, Dual b) { a = a + b; return a; }
MGB_ADJ_HD Dual &operator*=(Dual &a, Dual b) { a = a * b; return a; }
MGB_ADJ_HD Dual sqrt_(Dual a) {
  const double r = sqrt(a.v);
  return Dual(r, r > 0.0 ? a.d / (2.0 * r) : 0.0);
}
MGB_ADJ_HD double sqrt_(double a) { return sqrt(a); }
MGB_ADJ_HD double val(double a) { return a; }
MGB_ADJ_HD double val(Dual a) { return a.v; }

// Material constants derived from theta by the expressions of material.c:26-38 (k, mu, lambda) and
// material.cpp:110-147, 205-225 (the J2 denominator, the damage table with its hard-wired Ey = 1e5).
template <typename T>
struct Mat {
  T E, nu, Xt, Sy, Ka, k, mu, lambda, two_mu, xt_thr, r0, q0, q1, r1, pl_den;
  int type;
};

template <typename T>
MGB_ADJ_HD Mat<T> make_mat(int type, const T *theta) {
  Mat<T> m;
  m.type = type;
  m.E = theta[0];
  m.nu = theta[1];
  m.Xt = theta[2];
  m.Sy = theta[3];
  m.Ka = theta[4];
  m.k = m.E / (T(3.) * (T(1.) - T(2.) * m.nu));
  m.mu = m.E / (T(2.) * (T(1.) + m.nu));
  m.lambda = m.nu * m.E / ((T(1.) + m.nu) * (T(1.) - T(2.) * m.nu));
  m.two_mu = T(2.) * m.mu;
  const T sqE = sqrt_(m.E);
  m.xt_thr = m.Xt / sqE;
  const double Ey = 10.0e4, inf_Ey = 10. * Ey, H0 = 10.0;
  m.r0 = T(Ey) / sqE;
  m.q0 = m.r0;
  m.q1 = T(inf_Ey) / sqE;
  m.r1 = m.r0 + (m.q1 - m.q0) / T(H0);
  m.pl_den = T(2.) * m.mu * (T(1.) + m.Ka / (T(3.) * m.mu));
  return m;
}

template <typename T>
MGB_ADJ_HD void elastic(const Mat<T> &m, const T *eps, T *s) {
  const T tr = eps[0] + eps[1] + eps[2];
  for (int i = 0; i < 3; ++i) s[i] = m.lambda * tr + m.two_mu * eps[i];
  for (int i = 3; i < 6; ++i) s[i] = m.mu * eps[i];
}

// Stress and new history of one Gauss point (get_stress and evolute of the three laws, with the history
// always present, as after the point's first nonlinear step).
template <typename T>
MGB_ADJ_HD void law(const Mat<T> &m, const T *eps, const T *h, T *s, T *hn) {
  for (int i = 0; i < 7; ++i) hn[i] = h[i];
  if (m.type == 0) {
    elastic(m, eps, s);
    return;
  }
  if (m.type == 1) {
    // plastic_law (material.cpp:110-147), get_stress (149-162), evolute (168-181)
    const T third = T(1.0 / 3.0);
    const T tr_p = third * (h[0] + h[1] + h[2]);
    const T tr_e = third * (eps[0] + eps[1] + eps[2]);
    T st[6], tmp = T(0.0);
    for (int i = 0; i < 6; ++i) {
      const T de = (i < 3) ? eps[i] - tr_e : eps[i];
      const T dp = (i < 3) ? h[i] - tr_p : h[i];
      st[i] = (i < 3) ? m.two_mu * (de - dp) : m.mu * (de - dp);
      tmp += st[i] * st[i];
    }
    const T s_norm = sqrt_(tmp);
    const T f = s_norm - T(0.816496581) * (m.Sy + m.Ka * h[6]);
    T dl = T(0.0), normal[6];
    if (val(f) > 0) {
      for (int i = 0; i < 6; ++i) normal[i] = st[i] / s_norm;
      dl = f / m.pl_den;
    } else {
      for (int i = 0; i < 6; ++i) normal[i] = T(0.0);
    }
    const T tr = eps[0] + eps[1] + eps[2];
    const T g = m.two_mu * dl;
    for (int i = 0; i < 6; ++i) s[i] = ((i < 3) ? st[i] + m.k * tr : st[i]) - g * normal[i];
    for (int i = 0; i < 6; ++i) hn[i] = h[i] + dl * normal[i];
    hn[6] = h[6] + T(0.816496581) * dl;
    return;
  }
  // damage_law (material.cpp:227-268), get_stress (270-284), evolute (291-302)
  elastic(m, eps, s);
  T product = T(0.0);
  for (int i = 0; i < 6; ++i) product += s[i] * eps[i];
  const T r = (val(product) >= 0) ? sqrt_(product) : T(0.0);
  const T r_old_a = (val(h[0]) < val(m.xt_thr)) ? m.xt_thr : h[0];
  T D, rn;
  if (val(r) <= val(r_old_a)) {
    rn = r_old_a;
    D = h[1];
  } else {
    T q;
    if (val(r) < val(m.r0))
      q = T(0.0);
    else if (val(r) < val(m.r1))
      q = m.q0 + T(10.0) * (r - m.r0);
    else
      q = m.q1 + T(5.0) * (r - m.r1);
    rn = r;
    D = T(1.) - q / r;
  }
  const T fd = T(1.) - D;
  for (int i = 0; i < 6; ++i) s[i] *= fd;
  hn[0] = rn;
  hn[1] = D;
}

// One Jacobian column: direction j of (eps 0..5, history 6..12, theta 13..17).  ds[6], dhn[7] receive the
// derivatives of the stress and the new history along it.
MGB_ADJ_HD void law_column(int type, const double *theta, const double *eps, const double *h, int j, double *ds,
                           double *dhn) {
  Dual e[6], hh[7], th[kNpar], s[6], hn[7];
  for (int i = 0; i < 6; ++i) e[i] = Dual(eps[i], j == i ? 1.0 : 0.0);
  for (int i = 0; i < 7; ++i) hh[i] = Dual(h[i], j == 6 + i ? 1.0 : 0.0);
  for (int i = 0; i < kNpar; ++i) th[i] = Dual(theta[i], j == 13 + i ? 1.0 : 0.0);
  const Mat<Dual> m = make_mat<Dual>(type, th);
  law(m, e, hh, s, hn);
  for (int i = 0; i < 6; ++i) ds[i] = s[i].d;
  for (int i = 0; i < 7; ++i) dhn[i] = hn[i].d;
}

}  // namespace adj
}  // namespace mgb
