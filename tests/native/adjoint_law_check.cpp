// Checks the forward-mode derivatives of adjoint_laws.h against central differences of the same laws on
// random Gauss-point states of every branch (elastic; J2 elastic and plastic; damage below threshold,
// unloading and loading).  Prints one line per case: the largest error of a Jacobian column relative to the
// largest entry of that column.  Test infrastructure (tests/test_adjoint_laws.py builds and runs it).
#include <cmath>
#include <cstdio>
#include <random>

#include "adjoint_laws.h"

using namespace mgb::adj;

static void eval(int type, const double *x, double *out) {  // x = eps(6), h(7), theta(5); out = s(6), hn(7)
  const Mat<double> m = make_mat<double>(type, x + 13);
  law(m, x, x + 6, out, out + 6);
}

int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  struct Case {
    const char *name;
    int type;
    double eps, hscale, r_old;
  } cases[] = {{"elastic", 0, 5e-3, 0.0, 0.0},        {"j2-elastic", 1, 2e-4, 1e-5, 0.0},
               {"j2-plastic", 1, 8e-3, 1e-3, 0.0},    {"damage-below", 2, 1e-3, 0.0, 0.0},
               {"damage-unload", 2, 1e-2, 0.0, 500.0}, {"damage-loading", 2, 2.5e-2, 0.0, 0.0}};
  int bad = 0;
  for (const Case &c : cases) {
    for (int trial = 0; trial < 5; ++trial) {
      double x[18];
      for (int i = 0; i < 6; ++i) x[i] = c.eps * U(rng);
      for (int i = 0; i < 7; ++i) x[6 + i] = c.hscale * U(rng);
      if (c.type == 2) {
        x[6] = c.r_old;  // r_old
        x[7] = (c.r_old > 0) ? 0.3 : 0.0;  // D_old
      }
      if (c.type == 1) x[12] = std::fabs(x[12]);  // alpha >= 0
      const double theta[5] = {1e7 * (1 + 0.1 * U(rng)), 0.25 + 0.02 * U(rng), 1e5 * (1 + 0.05 * U(rng)),
                               1e4 * (1 + 0.1 * U(rng)), 1e5 * (1 + 0.1 * U(rng))};
      for (int i = 0; i < 5; ++i) x[13 + i] = theta[i];
      double worst = 0.0;
      for (int j = 0; j < kNdir; ++j) {
        double ds[6], dh[7];
        law_column(c.type, x + 13, x, x + 6, j, ds, dh);
        const double step = 1e-6 * (std::fabs(x[j]) > 0 ? std::fabs(x[j]) : 1e-3);
        double xp[18], xm[18], op[13], om[13];
        for (int i = 0; i < 18; ++i) xp[i] = xm[i] = x[i];
        xp[j] += step;
        xm[j] -= step;
        eval(c.type, xp, op);
        eval(c.type, xm, om);
        double colmax = 0.0, err = 0.0;
        for (int i = 0; i < 13; ++i) {
          const double fd = (op[i] - om[i]) / (2 * step);
          const double ad = (i < 6) ? ds[i] : dh[i - 6];
          colmax = std::fmax(colmax, std::fabs(fd));
          err = std::fmax(err, std::fabs(fd - ad));
        }
        if (colmax > 0) worst = std::fmax(worst, err / colmax);
      }
      std::printf("%s %d %.3e\n", c.name, trial, worst);
      if (!(worst < 1e-5)) bad++;
    }
  }
  return bad ? 1 : 0;
}
