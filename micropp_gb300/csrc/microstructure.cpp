// microstructure.cpp -- element phases of the reference micro types (micropp.cpp:338-544).
//
// Compiled with -ffp-contract=off so that the centroid tests round as in the reference (a centroid that
// lies on an inclusion surface is classified identically).
#include "microstructure.hpp"

#include <cmath>

namespace mgb {

namespace {

double norm3(const double v[3]) {
  double t = 0;
  for (int i = 0; i < 3; ++i) t += v[i] * v[i];
  return std::sqrt(t);
}

// point_inside_sphere (util.hpp:101-111)
bool in_sphere(const double c[3], double rad, const double p[3]) {
  const double v[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
  return norm3(v) < rad;
}

// point_inside_cilinder_inf (util.hpp:113-128): distance from the axis through c along dir.
bool in_cylinder(const double dir[3], const double c[3], double rad, const double p[3]) {
  const double v[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
  double dv = 0;
  for (int i = 0; i < 3; ++i) dv += dir[i] * v[i];
  const double nd = norm3(dir), nv = norm3(v);
  const double cs = dv / (nd * nv);
  const double sn = std::sqrt(1 - cs * cs);
  return nv * sn <= rad;
}

// Centres and radii (x 0.1) of the 40 spheres of MIC3D_SPHERES (micropp.cpp:455-475), and the y/z
// direction components of the 20 fibres of MIC3D_FIBS_20_DISORDER (micropp.cpp:515-519), whose centres are
// the first 20 sphere centres.  These numbers define those microstructures and are kept as published.
const double kSphC[40][3] = {
    {.8663, .0689, .1568}, {.2305, .4008, .2093}, {.1987, .8423, .2126}, {.6465, .7095, .4446},
    {.6151, .9673, .2257}, {.1311, .9739, .4129}, {.8433, .0738, .2233}, {.5124, .2111, .0369},
    {.4094, .7030, .6241}, {.1215, .8289, .3812}, {.1125, .9266, .6872}, {.7422, .4030, .6000},
    {.0791, .3819, .9297}, {.1201, .7712, .0069}, {.9339, .2177, .1976}, {.3880, .1331, .9032},
    {.7319, .7146, .8150}, {.8796, .2858, .6701}, {.1427, .9309, .9830}, {.1388, .3126, .8054},
    {.0729, .4754, .4950}, {.5038, .7755, .7333}, {.0242, .2185, .9884}, {.5371, .5372, .8269},
    {.4564, .0039, .1715}, {.7410, .0799, .8775}, {.2627, .9047, .5681}, {.7894, .1908, .2993},
    {.1373, .5370, .9916}, {.0207, .8020, .9283}, {.6540, .2359, .0286}, {.7801, .3568, .5086},
    {.7322, .5706, .1114}, {.5479, .1493, .1267}, {.6722, .1530, .1003}, {.7659, .3426, .9181},
    {.4582, .4636, .6310}, {.1811, .9665, .4713}, {.0834, .6066, .6936}, {.4865, .7584, .3635}};
const double kSphR[40] = {.5741, .1735, .5065, .8565, .9735, .7087, .9585, .2843, .4029, .2574,
                          .1575, .3316, .1874, .6300, .7049, .7258, .8002, .8176, .9970, .4736,
                          .6351, .3140, .3440, .2444, .3894, .5234, .1658, .4020, .6813, .2060,
                          .1427, .9332, .5406, .9765, .0956, .6432, .9998, .4166, .6907, .0404};
const double kFibD[20][2] = {{.5741, .8515}, {.1735, .1103}, {.5065, .4600}, {.8565, .9045}, {.9735, .6313},
                             {.7087, .1547}, {.9585, .0220}, {.2843, .4062}, {.4029, .8095}, {.2574, .4742},
                             {.1575, .0768}, {.3316, .0320}, {.1874, .6364}, {.6300, .2688}, {.7049, .5137},
                             {.7258, .2799}, {.8002, .4794}, {.8176, .4142}, {.9970, .2189}, {.4736, .6202}};

}  // namespace

int micro_elem_type(int micro_type, const double g[4], int ex, int ey, int ez, double dx, double dy, double dz) {
  const double lx = 1.0, ly = 1.0, lz = 1.0;
  const double p[3] = {ex * dx + dx / 2., ey * dy + dy / 2., ez * dz + dz / 2.};
  const double ax[3] = {1, 0, 0}, az[3] = {0, 0, 1};
  switch (micro_type) {
    case 0:  // MIC_HOMOGENEOUS
      return 0;
    case 1: {  // MIC_SPHERE
      const double c[3] = {lx / 2, ly / 2, lz / 2};
      return in_sphere(c, g[0], p) ? 1 : 0;
    }
    case 2:  // MIC_LAYER_Y
      return p[1] < g[0] ? 1 : 0;
    case 3: {  // MIC_CILI_FIB_X
      const double c[3] = {lx / 2, ly / 2, lz / 2};
      return in_cylinder(ax, c, g[0], p) ? 1 : 0;
    }
    case 4: {  // MIC_CILI_FIB_Z
      const double c[3] = {lx / 2, ly / 2, lz / 2};
      return in_cylinder(az, c, g[0], p) ? 1 : 0;
    }
    case 5: {  // MIC_CILI_FIB_XZ
      const double c1[3] = {lx / 2., ly * .75, lz / 2.}, c2[3] = {lx / 2., ly * .25, lz / 2.};
      return (in_cylinder(az, c1, g[0], p) || in_cylinder(ax, c2, g[0], p)) ? 1 : 0;
    }
    case 6:    // MIC_QUAD_FIB_XYZ
    case 7:    // MIC_QUAD_FIB_XZ
    case 8: {  // MIC_QUAD_FIB_XZ_BROKEN_X
      const double w = g[0];
      const double c[3] = {lx / 2., ly / 2., lz / 2.};
      const bool xy = std::fabs(p[0] - c[0]) < w && std::fabs(p[1] - c[1]) < w;
      const bool xz = std::fabs(p[0] - c[0]) < w && std::fabs(p[2] - c[2]) < w;
      const bool yz = std::fabs(p[1] - c[1]) < w && std::fabs(p[2] - c[2]) < w;
      if (micro_type == 6) return (xy || xz || yz) ? 1 : 0;
      if (micro_type == 7) return (xy || yz) ? 1 : 0;
      if (xy) return 1;
      return (yz && (p[0] < lx * .8 || p[0] > lx * .9)) ? 1 : 0;
    }
    case 9:  // MIC3D_SPHERES
      for (int i = 0; i < 40; ++i)
        if (in_sphere(kSphC[i], 0.1 * kSphR[i], p)) return 1;
      return 0;
    case 10: {  // MIC3D_8: cylinders (1), their coats and a flat layer (2), matrix (0)
      const double rc = 0.1, wf = 0.02, wc = 0.01;
      const double c1[3] = {lx * .25, ly * .75, 0.0}, c2[3] = {lx * .75, ly * .75, 0.0};
      const double c3[3] = {0.0, ly * .25, lz * .25}, c4[3] = {0.0, ly * .25, lz * .75};
      if (in_cylinder(az, c1, rc, p) || in_cylinder(az, c2, rc, p) || in_cylinder(ax, c3, rc, p) ||
          in_cylinder(ax, c4, rc, p))
        return 1;
      if (in_cylinder(az, c1, rc + wc, p) || in_cylinder(az, c2, rc + wc, p) || in_cylinder(ax, c3, rc + wc, p) ||
          in_cylinder(ax, c4, rc + wc, p) || std::fabs(p[1] - ly / 2) < wf)
        return 2;
      return 0;
    }
    case 11: {  // MIC3D_FIBS_20_ORDER: a 5 x 4 array of x-fibres
      const double dzf = 1.0 / (5 + 1), dyf = 1.0 / (4 + 1);
      for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 4; ++j) {
          const double c[3] = {0.0, (j + 1) * dyf, (i + 1) * dzf};
          if (in_cylinder(ax, c, 0.05, p)) return 1;
        }
      return 0;
    }
    case 12:  // MIC3D_FIBS_20_DISORDER
      for (int i = 0; i < 20; ++i) {
        const double d[3] = {1, kFibD[i][0], kFibD[i][1]};
        if (in_cylinder(d, kSphC[i], 0.05, p)) return 1;
      }
      return 0;
    default:
      return -1;
  }
}

}  // namespace mgb
