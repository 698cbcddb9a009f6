// elem_df.cuh -- the mixed form's element residual in double-float arithmetic (df.cuh), one element at a time,
// for elastic and damage phases: the body of k_elem_rhs_df (fe_kernels.cu).  It also compiles as plain C++,
// where the CPU test (tests/test_df_arithmetic.py) checks it against a long-double B-matrix evaluation.
//
// The residual block of an element is be = sum_g wg B_g^T sigma_g (assembly.cpp:123-138), evaluated by sum
// factorisation (hex_sumfact.h): the 36 nodal differences give the gradient at each Gauss point by bilinear
// interpolation, and the stresses times wg are summed per pair of points before the transposed weights.  The
// laws are the elastic law (material.cpp:76-82) and the damage law (material.cpp:227-268) with the terms of its
// consistent tangent, d sigma / d eps = a C + c s (x) s (s the undamaged stress).
#pragma once

#include "df.cuh"
#include "hex_sumfact.h"

#ifdef __CUDACC__
#define MGB_DF_UNROLL _Pragma("unroll")
#else
#define MGB_DF_UNROLL
#endif

namespace mgb {

// Constants of an elastic or damage phase as double-float values.
struct MatDf {
  dfl lambda, two_mu, mu, xt_thr, r0, r1, q0, q1;
};

// The residual's constants, split on the host: the phases, 1 - xg, 1 + xg, 1 / (4 h_d) and the Gauss weight.
struct ResDf {
  MatDf mat[3];
  dfl cm, cp, inv4h[3], wg;
};

// law_elastic (material.cpp:76-82)
MGB_DF void law_elastic_df(const MatDf &m, const dfl *eps, dfl *s) {
  const dfl lt = m.lambda * (eps[0] + eps[1] + eps[2]);
  MGB_DF_UNROLL
  for (int i = 0; i < 3; ++i) s[i] = lt + m.two_mu * eps[i];
  MGB_DF_UNROLL
  for (int i = 3; i < 6; ++i) s[i] = m.mu * eps[i];
}

// law_damage_hardening (material.cpp:213-225)
MGB_DF dfl hardening_df(const MatDf &m, dfl r) {
  if (r < m.r0) return dfl{0.f, 0.f};
  if (r < m.r1) return m.q0 + (r - m.r0) * 10.f;
  return m.q1 + (r - m.r1) * 5.f;
}

// One element: ue = its 24 FP64 nodal displacements (reference node order), mf = its phase, damage = the phase
// is the damage law, vars = its history (8 Gauss points x nvar values: r, D first) or null (zeros).  Returns the
// residual block be and sav = sum_g wg sigma_g; for a damage element, sink(g, a, c, s) receives each Gauss
// point's tangent terms (FP32, s the undamaged stress).
template <typename Sink>
MGB_DF void elem_rhs_df(const double (&ue)[24], const MatDf &mf, bool damage, const ResDf &cst, const double *vars,
                        int nvar, dfl (&be)[24], dfl (&sav)[6], Sink &&sink) {
  // D[d][c][k]: the 36 nodal differences of hex_sumfact.h (sf::diffs)
  dfl D[3][3][4];
  {
    dfl u[24];
    MGB_DF_UNROLL
    for (int i = 0; i < 24; ++i) u[i] = df_of(ue[i]);
    MGB_DF_UNROLL
    for (int d = 0; d < 3; ++d) {
      int p, q;
      sf::other_axes(d, p, q);
      MGB_DF_UNROLL
      for (int k = 0; k < 4; ++k) {
        int c1[3], c0[3];
        c1[d] = 1;
        c0[d] = 0;
        c1[p] = c0[p] = k >> 1;
        c1[q] = c0[q] = k & 1;
        const int a1 = sf::node_of(c1[0], c1[1], c1[2]), a0 = sf::node_of(c0[0], c0[1], c0[2]);
        MGB_DF_UNROLL
        for (int c = 0; c < 3; ++c) D[d][c][k] = u[a1 * 3 + c] - u[a0 * 3 + c];
      }
    }
  }
  const dfl cm = cst.cm, cp = cst.cp;  // 1 - xg, 1 + xg
  const dfl *inv4h = cst.inv4h;
  const dfl wg = cst.wg;
  dfl S[3][3][4];
  MGB_DF_UNROLL
  for (int d = 0; d < 3; ++d)
    MGB_DF_UNROLL
    for (int c = 0; c < 3; ++c)
      MGB_DF_UNROLL
      for (int k = 0; k < 4; ++k) S[d][c][k] = dfl{0.f, 0.f};
  MGB_DF_UNROLL
  for (int v = 0; v < 6; ++v) sav[v] = dfl{0.f, 0.f};
  MGB_DF_UNROLL
  for (int g = 0; g < 8; ++g) {
    const int gs[3] = {(g == 1 || g == 2 || g == 5 || g == 6) ? 1 : -1, (g == 2 || g == 3 || g == 6 || g == 7) ? 1 : -1,
                       g >= 4 ? 1 : -1};
    // gradient at the point (sf::grad_at): (1 - x_p)(1 - x_q) ... weights of the four differences
    dfl gr[3][3];
    MGB_DF_UNROLL
    for (int d = 0; d < 3; ++d) {
      int p, q;
      sf::other_axes(d, p, q);
      const dfl mp = gs[p] > 0 ? cm : cp, pp = gs[p] > 0 ? cp : cm;  // 1 - x_p, 1 + x_p
      const dfl mq = gs[q] > 0 ? cm : cp, pq = gs[q] > 0 ? cp : cm;  // 1 - x_q, 1 + x_q
      MGB_DF_UNROLL
      for (int c = 0; c < 3; ++c) {
        const dfl e0 = mq * D[d][c][0] + pq * D[d][c][1];
        const dfl e1 = mq * D[d][c][2] + pq * D[d][c][3];
        gr[d][c] = (mp * e0 + pp * e1) * inv4h[d];
      }
    }
    const dfl eps[6] = {gr[0][0], gr[1][1], gr[2][2], gr[1][0] + gr[0][1], gr[2][0] + gr[0][2], gr[2][1] + gr[1][2]};
    dfl sg[6];
    law_elastic_df(mf, eps, sg);
    if (damage) {
      // law_damage_terms (laws.cuh) on the undamaged stress sg
      const double *vg = vars ? vars + (size_t)g * nvar : nullptr;
      const dfl r_old = df_of(vg ? vg[0] : 0.0), D_old = df_of(vg ? vg[1] : 0.0);
      dfl prod = sg[0] * eps[0];
      MGB_DF_UNROLL
      for (int i = 1; i < 6; ++i) prod = prod + sg[i] * eps[i];
      const dfl r = df_nonneg(prod) ? df_sqrt(prod) : dfl{0.f, 0.f};
      const dfl r_old_a = (r_old < mf.xt_thr) ? mf.xt_thr : r_old;
      dfl Dm;
      float ta, tc;
      if (r <= r_old_a) {
        Dm = D_old;
        ta = (dfl{1.f, 0.f} - D_old).h;
        tc = 0.f;
      } else {
        const dfl q = hardening_df(mf, r);
        const dfl qr = q / r;
        Dm = dfl{1.f, 0.f} - qr;
        const float qp = (r < mf.r0) ? 0.f : (r < mf.r1 ? 10.f : 5.f);
        ta = qr.h;
        tc = (qp - ta) / (r.h * r.h);
      }
      float s6[6];
      MGB_DF_UNROLL
      for (int v = 0; v < 6; ++v) s6[v] = sg[v].h + sg[v].l;
      sink(g, ta, tc, s6);
      const dfl f = dfl{1.f, 0.f} - Dm;
      MGB_DF_UNROLL
      for (int v = 0; v < 6; ++v) sg[v] = sg[v] * f;
    }
    // S[d][c][gp * 2 + gq] += wg sigma_dc (sf::accumulate), and the stress average
    const dfl ws[6] = {sg[0] * wg, sg[1] * wg, sg[2] * wg, sg[3] * wg, sg[4] * wg, sg[5] * wg};
    const dfl t[3][3] = {{ws[0], ws[3], ws[4]}, {ws[3], ws[1], ws[5]}, {ws[4], ws[5], ws[2]}};
    MGB_DF_UNROLL
    for (int d = 0; d < 3; ++d) {
      int p, q;
      sf::other_axes(d, p, q);
      const int k = (gs[p] > 0 ? 2 : 0) + (gs[q] > 0 ? 1 : 0);
      MGB_DF_UNROLL
      for (int c = 0; c < 3; ++c) S[d][c][k] = S[d][c][k] + t[d][c];
    }
    MGB_DF_UNROLL
    for (int v = 0; v < 6; ++v) sav[v] = sav[v] + ws[v];
  }
  // be = the transpose (sf::finish)
  MGB_DF_UNROLL
  for (int i = 0; i < 24; ++i) be[i] = dfl{0.f, 0.f};
  MGB_DF_UNROLL
  for (int d = 0; d < 3; ++d) {
    int p, q;
    sf::other_axes(d, p, q);
    MGB_DF_UNROLL
    for (int c = 0; c < 3; ++c) {
      dfl f[2][2];  // f[gp][cq]
      MGB_DF_UNROLL
      for (int gp = 0; gp < 2; ++gp) {
        f[gp][0] = cp * S[d][c][gp * 2 + 0] + cm * S[d][c][gp * 2 + 1];
        f[gp][1] = cm * S[d][c][gp * 2 + 0] + cp * S[d][c][gp * 2 + 1];
      }
      MGB_DF_UNROLL
      for (int cpp = 0; cpp < 2; ++cpp)
        MGB_DF_UNROLL
        for (int cq = 0; cq < 2; ++cq) {
          const dfl w = (cpp ? cm * f[0][cq] + cp * f[1][cq] : cp * f[0][cq] + cm * f[1][cq]) * inv4h[d];
          int c1[3], c0[3];
          c1[d] = 1;
          c0[d] = 0;
          c1[p] = c0[p] = cpp;
          c1[q] = c0[q] = cq;
          const int a1 = sf::node_of(c1[0], c1[1], c1[2]) * 3 + c, a0 = sf::node_of(c0[0], c0[1], c0[2]) * 3 + c;
          be[a1] = be[a1] + w;
          be[a0] = be[a0] - w;
        }
    }
  }
}

}  // namespace mgb
