"""Double-float arithmetic of the fast form's FP64-accurate kernels (micropp_gb300/csrc/df.cuh and elem_df.cuh),
on the CPU.

The header compiles as plain C++ with the same sequence of correctly rounded FP32 operations that the GPU
kernels use (built here without floating-point contraction, which the device code forbids with its
explicit-rounding intrinsics).  A small harness checks every operator against long double on seeded random
operands over twelve decades, and the two composite steps of the kernels: the refinement residual's row
f - sum k x (df_sub_prod, FP32 k, double-float x and f) on rows that cancel to 1e-7 of their terms, and the
accumulation X += D (df_add).  Bars: 2^-44 relative for the operators, 1e-12 of sum |k x| for a row.  A second
harness runs the element residual of the mixed form (elem_rhs_df, the body of the GPU kernel k_elem_rhs_df)
against a long-double B-matrix evaluation.
"""
import pathlib
import shutil
import subprocess

import pytest

CSRC = pathlib.Path(__file__).resolve().parents[1] / "micropp_gb300" / "csrc"

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "df.cuh"
using namespace mgb;
typedef long double LD;
static LD ld(dfl a) { return (LD)a.h + (LD)a.l; }
static LD ldabs(LD x) { return x < 0 ? -x : x; }
int main() {
  std::mt19937_64 g(20241204);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::normal_distribution<double> N(0.0, 1.0);
  double e_add = 0, e_mul = 0, e_mulf = 0, e_div = 0, e_sqrt = 0, e_split = 0;
  for (int it = 0; it < 200000; ++it) {
    const double x = U(g) * std::pow(10.0, 6.0 * U(g)), y = U(g) * std::pow(10.0, 6.0 * U(g));
    const dfl a = df_of(x), b = df_of(y);
    const LD A = ld(a), B = ld(b);
    e_split = std::fmax(e_split, (double)(ldabs(A - (LD)x) / ldabs((LD)x)));
    e_add = std::fmax(e_add, (double)(ldabs(ld(a + b) - (A + B)) / (ldabs(A) + ldabs(B))));
    e_mul = std::fmax(e_mul, (double)(ldabs(ld(a * b) - A * B) / ldabs(A * B)));
    const float f = (float)y;
    e_mulf = std::fmax(e_mulf, (double)(ldabs(ld(a * f) - A * (LD)f) / ldabs(A * (LD)f)));
    e_div = std::fmax(e_div, (double)(ldabs(ld(a / b) - A / B) / ldabs(A / B)));
    const dfl p = df_of(std::fabs(x));
    const LD P = ld(p), R = std::sqrt((long double)P);
    e_sqrt = std::fmax(e_sqrt, (double)(ldabs(ld(df_sqrt(p)) - R) / R));
  }
  // refinement-residual rows: f - sum_j k_j x_j with 81 terms cancelling to ~1e-7 of their size
  double e_row = 0;
  for (int row = 0; row < 20000; ++row) {
    float k[81];
    double x[81];
    LD exact = 0;
    for (int j = 0; j < 81; ++j) {
      k[j] = (float)(N(g) * 2e5);
      x[j] = N(g) * 0.3;
      exact += (LD)k[j] * (LD)x[j];
    }
    float h, l;
    df_split((double)exact * (1.0 + 1e-7 * N(g)), h, l);
    LD ref = (LD)h + (LD)l, scale = 0;
    for (int j = 0; j < 81; ++j) {
      float xh, xl;
      df_split(x[j], xh, xl);
      df_sub_prod(h, l, k[j], xh, xl);
      ref -= (LD)k[j] * ((LD)xh + (LD)xl);
      scale += ldabs((LD)k[j] * (LD)x[j]);
    }
    e_row = std::fmax(e_row, (double)(ldabs((LD)h + (LD)l - ref) / scale));
  }
  // X += D over 50 FP32 corrections of decreasing size (the sweeps of a refined solve)
  double e_acc = 0;
  for (int it = 0; it < 20000; ++it) {
    float h = 0.f, l = 0.f;
    LD ref = 0, scale = 0;
    for (int s = 0; s < 50; ++s) {
      const float d = (float)(N(g) * std::pow(10.0, -0.2 * s));
      df_add(h, l, d);
      ref += (LD)d;
      scale += ldabs((LD)d);
    }
    e_acc = std::fmax(e_acc, (double)(ldabs((LD)h + (LD)l - ref) / scale));
  }
  std::printf("split %.3e add %.3e mul %.3e mulf %.3e div %.3e sqrt %.3e row %.3e acc %.3e\n", e_split, e_add, e_mul,
              e_mulf, e_div, e_sqrt, e_row, e_acc);
  return 0;
}
"""


def test_double_float_operators_and_kernel_steps(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    src = tmp_path / "df_check.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "df_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(CSRC), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    err = {out[i]: float(out[i + 1]) for i in range(0, len(out), 2)}
    print(err)
    bar = 2.0 ** -44
    for op in ("split", "add", "mul", "mulf", "div", "sqrt", "acc"):
        assert err[op] <= bar, (op, err[op])
    assert err["row"] <= 1e-12, err["row"]


ELEM_HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "elem_df.cuh"
using namespace mgb;
typedef long double LD;
static const LD kXg = 0.577350269189626L;
// corner (cx, cy, cz) of local node a, reference numbering (node_of = cz * 4 + (cy ? 3 - cx : cx))
static void corner(int a, int c[3]) {
  c[2] = a / 4;
  const int r = a % 4;
  c[1] = r >= 2;
  c[0] = (r == 1 || r == 2);
}
struct LMat { LD lam, mu, xt, r0, r1, q0, q1; };
static LD hard(const LMat &m, LD r) { return r < m.r0 ? 0 : (r < m.r1 ? m.q0 + 10 * (r - m.r0) : m.q1 + 5 * (r - m.r1)); }
int main() {
  std::mt19937_64 gen(77);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  std::normal_distribution<double> N(0.0, 1.0);
  double e_be = 0, e_sav = 0, e_a = 0, e_c = 0, e_s = 0;
  int n_load = 0, n_unload = 0, n_skip = 0;
  for (int it = 0; it < 4000; ++it) {
    const double h[3] = {0.01 + 0.04 * U(gen), 0.01 + 0.04 * U(gen), 0.01 + 0.04 * U(gen)};
    const double E = 1e7 * (1 + 9 * U(gen)), nu = 0.2 + 0.2 * U(gen);
    const double lam = E * nu / ((1 + nu) * (1 - 2 * nu)), mu = E / (2 * (1 + nu));
    const bool damage = it % 4 != 0;
    const double xt = 1e5 / std::sqrt(E) * (0.5 + U(gen)), r0 = 20 + 20 * U(gen), r1 = r0 + 20 + 20 * U(gen);
    const double q0 = 0.8 * r0, q1 = q0 + 10 * (r1 - r0);
    ResDf cst;
    cst.cm = df_of(1.0 - 0.577350269189626);
    cst.cp = df_of(1.0 + 0.577350269189626);
    for (int d = 0; d < 3; ++d) cst.inv4h[d] = df_of(0.25 / h[d]);
    const double wg = h[0] * h[1] * h[2] / 8.0;
    cst.wg = df_of(wg);
    const MatDf mf{df_of(lam), df_of(2 * mu), df_of(mu), df_of(xt), df_of(r0), df_of(r1), df_of(q0), df_of(q1)};
    cst.mat[0] = cst.mat[1] = cst.mat[2] = mf;
    const LMat lm{(LD)lam, (LD)mu, (LD)xt, (LD)r0, (LD)r1, (LD)q0, (LD)q1};
    // displacements: an affine field of strain ~3e-3 plus noise, offset by a rigid translation
    double ue[24], G[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) G[i][j] = 3e-3 * N(gen);
    const double t0[3] = {N(gen), N(gen), N(gen)};
    for (int a = 0; a < 8; ++a) {
      int c[3];
      corner(a, c);
      for (int i = 0; i < 3; ++i) {
        double v = 1e-3 * t0[i] + 2e-4 * N(gen) * h[i];
        for (int j = 0; j < 3; ++j) v += G[i][j] * c[j] * h[j];
        ue[a * 3 + i] = v;
      }
    }
    double vars[8 * 2];
    for (int g = 0; g < 8; ++g) {
      vars[g * 2] = (U(gen) < 0.5) ? 0.0 : 60 * U(gen);
      vars[g * 2 + 1] = vars[g * 2] > 0 ? 0.5 * U(gen) : 0.0;
    }
    // long-double reference by B-matrix products
    LD be_ref[24] = {0}, sav_ref[6] = {0}, a_ref[8], c_ref[8], c_scale[8], s_ref[8][6];
    bool skip = false;
    for (int g = 0; g < 8; ++g) {
      const int gs[3] = {(g == 1 || g == 2 || g == 5 || g == 6) ? 1 : -1, (g == 2 || g == 3 || g == 6 || g == 7) ? 1 : -1,
                         g >= 4 ? 1 : -1};
      LD dN[8][3];
      for (int a = 0; a < 8; ++a) {
        int c[3];
        corner(a, c);
        for (int d = 0; d < 3; ++d) {
          const int p = d == 0 ? 1 : 0, q = d == 2 ? 1 : 2;
          const LD sd = 2 * c[d] - 1, sp = 2 * c[p] - 1, sq = 2 * c[q] - 1;
          dN[a][d] = sd * (1 + sp * gs[p] * kXg) * (1 + sq * gs[q] * kXg) / (4 * (LD)h[d]);
        }
      }
      LD gr[3][3] = {{0}};  // gr[d][c] = du_c / dx_d
      for (int a = 0; a < 8; ++a)
        for (int d = 0; d < 3; ++d)
          for (int c = 0; c < 3; ++c) gr[d][c] += dN[a][d] * (LD)ue[a * 3 + c];
      const LD eps[6] = {gr[0][0], gr[1][1], gr[2][2], gr[1][0] + gr[0][1], gr[2][0] + gr[0][2], gr[2][1] + gr[1][2]};
      const LD tr = eps[0] + eps[1] + eps[2];
      LD s[6];
      for (int i = 0; i < 3; ++i) s[i] = lm.lam * tr + 2 * lm.mu * eps[i];
      for (int i = 3; i < 6; ++i) s[i] = lm.mu * eps[i];
      LD f = 1;
      if (damage) {
        LD prod = 0;
        for (int i = 0; i < 6; ++i) prod += s[i] * eps[i];
        const LD r = prod >= 0 ? std::sqrt(prod) : 0;
        const LD rold = vars[g * 2] < lm.xt ? lm.xt : (LD)vars[g * 2];
        // ties within 1e-9 of a branch switch may go either way in double-float: not a test of the arithmetic
        if (std::fabs((double)(r - rold)) < 1e-9 * (double)r || std::fabs((double)(r - lm.r0)) < 1e-9 * (double)r ||
            std::fabs((double)(r - lm.r1)) < 1e-9 * (double)r)
          skip = true;
        for (int i = 0; i < 6; ++i) s_ref[g][i] = s[i];
        if (r <= rold) {
          f = 1 - (LD)vars[g * 2 + 1];
          a_ref[g] = f;
          c_ref[g] = 0;
          c_scale[g] = 1;
          ++n_unload;
        } else {
          const LD q = hard(lm, r), qp = r < lm.r0 ? 0 : (r < lm.r1 ? 10 : 5);
          f = q / r;
          a_ref[g] = q / r;
          c_ref[g] = (qp - q / r) / (r * r);
          // c = (q' - a) / r^2 is formed in FP32 from the FP32 a: its error is relative to (|q'| + |a|) / r^2
          c_scale[g] = (std::fabs((double)qp) + std::fabs((double)(q / r))) / (r * r);
          ++n_load;
        }
      }
      for (int i = 0; i < 6; ++i) {
        s[i] *= f;
        sav_ref[i] += s[i] * wg;
      }
      for (int a = 0; a < 8; ++a) {
        be_ref[a * 3 + 0] += wg * (dN[a][0] * s[0] + dN[a][1] * s[3] + dN[a][2] * s[4]);
        be_ref[a * 3 + 1] += wg * (dN[a][1] * s[1] + dN[a][0] * s[3] + dN[a][2] * s[5]);
        be_ref[a * 3 + 2] += wg * (dN[a][2] * s[2] + dN[a][0] * s[4] + dN[a][1] * s[5]);
      }
    }
    if (skip) {
      ++n_skip;
      continue;
    }
    dfl be[24], sav[6];
    float ga[8] = {0}, gc[8] = {0}, gsv[8][6] = {{0}};
    auto sink = [&](int g, float a, float c, const float *s6) {
      ga[g] = a;
      gc[g] = c;
      for (int v = 0; v < 6; ++v) gsv[g][v] = s6[v];
    };
    elem_rhs_df(ue, mf, damage, cst, vars, 2, be, sav, sink);
    LD bmax = 0, smax = 0;
    for (int i = 0; i < 24; ++i) bmax = std::fmax((double)bmax, (double)std::fabs((double)be_ref[i]));
    for (int i = 0; i < 6; ++i) smax = std::fmax((double)smax, (double)std::fabs((double)sav_ref[i]));
    for (int i = 0; i < 24; ++i)
      e_be = std::fmax(e_be, (double)(std::fabs((double)(((LD)be[i].h + (LD)be[i].l) - be_ref[i])) / bmax));
    for (int i = 0; i < 6; ++i)
      e_sav = std::fmax(e_sav, (double)(std::fabs((double)(((LD)sav[i].h + (LD)sav[i].l) - sav_ref[i])) / smax));
    if (damage)
      for (int g = 0; g < 8; ++g) {
        e_a = std::fmax(e_a, std::fabs((double)((LD)ga[g] - a_ref[g])) / std::fabs((double)a_ref[g]));
        e_c = std::fmax(e_c, std::fabs((double)((LD)gc[g] - c_ref[g])) / (double)c_scale[g]);
        LD sm = 0;
        for (int v = 0; v < 6; ++v) sm = std::fmax((double)sm, std::fabs((double)s_ref[g][v]));
        for (int v = 0; v < 6; ++v) e_s = std::fmax(e_s, std::fabs((double)((LD)gsv[g][v] - s_ref[g][v])) / (double)sm);
      }
  }
  std::printf("be %.3e sav %.3e a %.3e c %.3e s %.3e load %d unload %d skip %d\n", e_be, e_sav, e_a, e_c, e_s, n_load,
              n_unload, n_skip);
  return 0;
}
"""


def test_double_float_element_residual_against_long_double(tmp_path):
    """elem_rhs_df (the body of k_elem_rhs_df) on random elements -- elastic, and damage on both branches of the
    law with random histories -- against a long-double evaluation by B-matrix products: the residual block and
    the average-stress sum within 1e-12 of their largest entry, the FP32 tangent terms within FP32 rounding (c,
    formed from the FP32 a, relative to (|q'| + |a|) / r^2)."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    src = tmp_path / "elem_check.cpp"
    src.write_text(ELEM_HARNESS)
    exe = tmp_path / "elem_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(CSRC), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    res = {out[i]: float(out[i + 1]) for i in range(0, len(out), 2)}
    print(res)
    assert res["load"] > 1000 and res["unload"] > 1000, res
    assert res["be"] <= 1e-12 and res["sav"] <= 1e-12, res
    assert res["a"] <= 1e-6 and res["s"] <= 1e-6, res
    assert res["c"] <= 1e-6, res
