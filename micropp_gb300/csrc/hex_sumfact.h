// hex_sumfact.h -- sum-factorised gradients, and their transpose, on the trilinear hexahedron with 2x2x2 Gauss
// points (the element of calc_bmat, micro3D.cpp:80-120).
//
// With corner signs s = +-1 and Gauss coordinates xi = +-1/sqrt(3), the shape-function gradient is
//   dN_a/dx_d = s_a,d (1 + s_a,p xi_p) (1 + s_a,q xi_q) / (4 h_d),   p, q = the two other axes,
// which does not depend on xi_d.  So at every Gauss point
//   du_c/dx_d = 1/(4 h_d) sum_{cp, cq} (1 + s(cp) xi_p) (1 + s(cq) xi_q) D_dc(cp, cq),
// where D_dc(cp, cq) is u_c at the corner (c_d = 1, cp, cq) minus u_c at (c_d = 0, cp, cq): 36 differences per
// element and a bilinear interpolation per point, in place of the 8-node sums of B u.  The transpose,
// sum_g w sum_d dN_a/dx_d sigma_dc, sums each stress component over the two points that differ in xi_d only,
// then weights the four sums bilinearly per corner.  Plain templates for the device and the host (the CPU
// check against the B-matrix products).
#pragma once

#ifdef __CUDACC__
#define MGB_SF_HD __host__ __device__ __forceinline__
#define MGB_SF_UNROLL _Pragma("unroll")
#else
#define MGB_SF_HD inline
#define MGB_SF_UNROLL
#endif

namespace mgb {
namespace sf {

// Local node of corner (cx, cy, cz) in the reference numbering (common.cpp:28-40).
MGB_SF_HD int node_of(int cx, int cy, int cz) { return cz * 4 + (cy ? 3 - cx : cx); }

// The two axes other than d, in the order of calc_bmat's factors.
MGB_SF_HD void other_axes(int d, int &p, int &q) {
  p = (d == 0) ? 1 : 0;
  q = (d == 2) ? 1 : 2;
}

// D[d][c][cp * 2 + cq] = u_c(c_d = 1, c_p = cp, c_q = cq) - u_c(c_d = 0, c_p = cp, c_q = cq); ue node-major.
template <typename T>
MGB_SF_HD void diffs(const T *ue, T (&D)[3][3][4]) {
MGB_SF_UNROLL
  for (int d = 0; d < 3; ++d) {
    int p, q;
    other_axes(d, p, q);
MGB_SF_UNROLL
    for (int k = 0; k < 4; ++k) {
      int c1[3], c0[3];
      c1[d] = 1;
      c0[d] = 0;
      c1[p] = c0[p] = k >> 1;
      c1[q] = c0[q] = k & 1;
      const int a1 = node_of(c1[0], c1[1], c1[2]), a0 = node_of(c0[0], c0[1], c0[2]);
MGB_SF_UNROLL
      for (int c = 0; c < 3; ++c) D[d][c][k] = ue[a1 * 3 + c] - ue[a0 * 3 + c];
    }
  }
}

// grad[d][c] = du_c/dx_d at the Gauss point with coordinate signs gs (+-1 per axis); xg = 1/sqrt(3),
// inv4h[d] = 1 / (4 h_d).
template <typename T>
MGB_SF_HD void grad_at(const T (&D)[3][3][4], const int (&gs)[3], double xg, const double (&inv4h)[3],
                       T (&grad)[3][3]) {
MGB_SF_UNROLL
  for (int d = 0; d < 3; ++d) {
    int p, q;
    other_axes(d, p, q);
    const double xp = gs[p] * xg, xq = gs[q] * xg;
MGB_SF_UNROLL
    for (int c = 0; c < 3; ++c) {
      const T e0 = (1 - xq) * D[d][c][0] + (1 + xq) * D[d][c][1];
      const T e1 = (1 - xq) * D[d][c][2] + (1 + xq) * D[d][c][3];
      grad[d][c] = ((1 - xp) * e0 + (1 + xp) * e1) * inv4h[d];
    }
  }
}

// Voigt strain (engineering shear; xx, yy, zz, xy, xz, yz) of a gradient.
template <typename T>
MGB_SF_HD void strain_of(const T (&g)[3][3], T *eps) {
  eps[0] = g[0][0];
  eps[1] = g[1][1];
  eps[2] = g[2][2];
  eps[3] = g[1][0] + g[0][1];
  eps[4] = g[2][0] + g[0][2];
  eps[5] = g[2][1] + g[1][2];
}

// S[d][c][gp * 2 + gq] += w sigma_dc for a Gauss point with signs gs (gp, gq = 1 for the + sign along p, q).
template <typename T>
MGB_SF_HD void accumulate(T (&S)[3][3][4], const int (&gs)[3], const T *sig, T w) {
  const T t[3][3] = {{sig[0], sig[3], sig[4]}, {sig[3], sig[1], sig[5]}, {sig[4], sig[5], sig[2]}};
MGB_SF_UNROLL
  for (int d = 0; d < 3; ++d) {
    int p, q;
    other_axes(d, p, q);
    const int k = (gs[p] > 0 ? 2 : 0) + (gs[q] > 0 ? 1 : 0);
MGB_SF_UNROLL
    for (int c = 0; c < 3; ++c) S[d][c][k] += w * t[d][c];
  }
}

// be[a * 3 + c] = sum_d s(c_d(a)) W_dc(c_p(a), c_q(a)) / (4 h_d), with
// W_dc(cp, cq) = sum_{gp, gq} (1 + s(cp) xi(gp)) (1 + s(cq) xi(gq)) S[d][c][gp * 2 + gq].
template <typename T>
MGB_SF_HD void finish(const T (&S)[3][3][4], double xg, const double (&inv4h)[3], T *be) {
MGB_SF_UNROLL
  for (int i = 0; i < 24; ++i) be[i] = 0;
MGB_SF_UNROLL
  for (int d = 0; d < 3; ++d) {
    int p, q;
    other_axes(d, p, q);
MGB_SF_UNROLL
    for (int c = 0; c < 3; ++c) {
      T f[2][2];  // f[gp][cq]
MGB_SF_UNROLL
      for (int gp = 0; gp < 2; ++gp) {
        f[gp][0] = (1 + xg) * S[d][c][gp * 2 + 0] + (1 - xg) * S[d][c][gp * 2 + 1];
        f[gp][1] = (1 - xg) * S[d][c][gp * 2 + 0] + (1 + xg) * S[d][c][gp * 2 + 1];
      }
MGB_SF_UNROLL
      for (int cp = 0; cp < 2; ++cp)
MGB_SF_UNROLL
        for (int cq = 0; cq < 2; ++cq) {
          const T w = (cp ? (1 - xg) * f[0][cq] + (1 + xg) * f[1][cq] : (1 + xg) * f[0][cq] + (1 - xg) * f[1][cq]) *
                      inv4h[d];
          int c1[3], c0[3];
          c1[d] = 1;
          c0[d] = 0;
          c1[p] = c0[p] = cp;
          c1[q] = c0[q] = cq;
          be[node_of(c1[0], c1[1], c1[2]) * 3 + c] += w;
          be[node_of(c0[0], c0[1], c0[2]) * 3 + c] -= w;
        }
    }
  }
}

}  // namespace sf
}  // namespace mgb
