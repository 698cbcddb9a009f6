// Sum-factorised strain and element residual (hex_sumfact.h) against the direct B-matrix products on random
// displacements and stresses of a non-cubic element; prints the largest relative differences.
#include <cmath>
#include <cstdio>
#include <random>

#include "hex_sumfact.h"

static const int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

int main() {
  const double xg = 0.577350269189626;
  const double h[3] = {0.1, 0.125, 0.2};
  // shape-function gradients at the Gauss points, as calc_bmat forms them
  double dsh[8][24];
  for (int g = 0; g < 8; ++g)
    for (int a = 0; a < 8; ++a) {
      double s[3], x[3];
      for (int d = 0; d < 3; ++d) {
        s[d] = kCorner[a][d] ? 1.0 : -1.0;
        x[d] = kCorner[g][d] ? xg : -xg;
      }
      for (int d = 0; d < 3; ++d) {
        const int p = (d == 0) ? 1 : 0, q = (d == 2) ? 1 : 2;
        dsh[g][a * 3 + d] = s[d] * (1 + s[p] * x[p]) * (1 + s[q] * x[q]) / 8. * 2. / h[d];
      }
    }
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  double worst_eps = 0, worst_be = 0;
  for (int trial = 0; trial < 200; ++trial) {
    double ue[24], sig[8][6];
    for (double &v : ue) v = U(rng);
    for (auto &r : sig)
      for (double &v : r) v = 1e6 * U(rng);
    const double w = h[0] * h[1] * h[2] / 8;
    // direct
    double eps_d[8][6], be_d[24] = {0};
    for (int g = 0; g < 8; ++g) {
      double e[6] = {0, 0, 0, 0, 0, 0};
      for (int a = 0; a < 8; ++a) {
        const double gx = dsh[g][a * 3], gy = dsh[g][a * 3 + 1], gz = dsh[g][a * 3 + 2];
        const double ux = ue[a * 3], uy = ue[a * 3 + 1], uz = ue[a * 3 + 2];
        e[0] += gx * ux; e[1] += gy * uy; e[2] += gz * uz;
        e[3] += gy * ux + gx * uy; e[4] += gz * ux + gx * uz; e[5] += gz * uy + gy * uz;
        const double *s = sig[g];
        be_d[a * 3 + 0] += (gx * s[0] + gy * s[3] + gz * s[4]) * w;
        be_d[a * 3 + 1] += (gy * s[1] + gx * s[3] + gz * s[5]) * w;
        be_d[a * 3 + 2] += (gz * s[2] + gx * s[4] + gy * s[5]) * w;
      }
      for (int v = 0; v < 6; ++v) eps_d[g][v] = e[v];
    }
    // sum-factorised
    const double inv4h[3] = {1 / (4 * h[0]), 1 / (4 * h[1]), 1 / (4 * h[2])};
    double D[3][3][4], S[3][3][4] = {}, be_s[24];
    mgb::sf::diffs(ue, D);
    double emax = 0, bmax = 0, de = 0, db = 0;
    for (int g = 0; g < 8; ++g) {
      const int gs[3] = {kCorner[g][0] ? 1 : -1, kCorner[g][1] ? 1 : -1, kCorner[g][2] ? 1 : -1};
      double gr[3][3], eps[6];
      mgb::sf::grad_at(D, gs, xg, inv4h, gr);
      mgb::sf::strain_of(gr, eps);
      for (int v = 0; v < 6; ++v) {
        de = std::fmax(de, std::fabs(eps[v] - eps_d[g][v]));
        emax = std::fmax(emax, std::fabs(eps_d[g][v]));
      }
      mgb::sf::accumulate(S, gs, sig[g], w);
    }
    mgb::sf::finish(S, xg, inv4h, be_s);
    for (int i = 0; i < 24; ++i) {
      db = std::fmax(db, std::fabs(be_s[i] - be_d[i]));
      bmax = std::fmax(bmax, std::fabs(be_d[i]));
    }
    worst_eps = std::fmax(worst_eps, de / emax);
    worst_be = std::fmax(worst_be, db / bmax);
  }
  std::printf("strain %.3e\nresidual %.3e\n", worst_eps, worst_be);
  return 0;
}
