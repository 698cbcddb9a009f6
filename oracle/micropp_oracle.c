/*
 * micropp_oracle.c -- CPU restatement of Micropp's RVE homogenization path (FP64).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the GPU library is checked against.  Only tests/, the smoke check
 * and the benchmark's CPU-baseline leg load it; the product library never does.
 *
 * Every routine restates the reference CPU code in the same floating-point operation order (compiled with
 * -ffp-contract=off so that no multiply-add is fused), so that on identical inputs it reproduces the
 * reference bit for bit.  Citations are file:line in gagiuntoli/Micropp.
 */
#include "micropp_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Compile-time constants of the reference (params.hpp:26-41, material_base.h:29-30, ell.hpp:33-35). */
#define NVOI 6
#define NPE 8
#define DIM 3
#define NPEDIM 24
#define NVAR_GP 7
#define NNZ 81
#define D_EPS_CTAN_AVE 1.0e-8
#define D_EPS_CTAN 1.0e-8
#define CONSTXG 0.577350269189626
#define SQRT_2DIV3 0.816496581

enum { MAT_ELASTIC = 0, MAT_PLASTIC = 1, MAT_DAMAGE = 2 };
enum { FE_LINEAR = 0, FE_ONE_WAY = 1, FE_FULL = 2, MIX_RULE_CHAMIS = 3 };
enum {
  MIC_HOMOGENEOUS, MIC_SPHERE, MIC_LAYER_Y, MIC_CILI_FIB_X, MIC_CILI_FIB_Z, MIC_CILI_FIB_XZ, MIC_QUAD_FIB_XYZ,
  MIC_QUAD_FIB_XZ, MIC_QUAD_FIB_XZ_BROKEN_X, MIC3D_SPHERES, MIC3D_8, MIC3D_FIBS_20_ORDER, MIC3D_FIBS_20_DISORDER
};

typedef struct {
  double strain_old[NVOI], strain[NVOI], stress[NVOI], ctan[NVOI * NVOI];
  int allocated;
  double *vars_n, *vars_k, *u_n, *u_k;
  long cost;
  int converged, subiterated, coupling;
  int nr_its, nr_solver_its, nr_converged;
  double op_count[ORC_NOPS], op_sec[ORC_NOPS]; /* instrumentation only (orc_get_ops) */
} orc_gp;

/* Operation record of the Gauss point whose homogenization runs on this thread (NULL: not recorded).  It
 * only counts and times operations; no result depends on it. */
static __thread orc_gp *t_ops;

static double wtime(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return (double)clock() / CLOCKS_PER_SEC;
#endif
}

static void op_add(int op, double count, double t0) {
  if (t_ops) {
    t_ops->op_count[op] += count;
    t_ops->op_sec[op] += wtime() - t0;
  }
}

typedef struct {
  int n[3], nn, nrow;
  int *cols;
  double *vals;
  int max_its;
  double min_err, rel_err;
  double *k, *r, *z, *p, *Ap;
} orc_ell;

struct orc_rve {
  int ngp, nx, ny, nz, nn, nndim, nex, ney, nez, nelem, nvars;
  double lx, ly, lz, dx, dy, dz, wg, vol_tot, ivol, evol;
  int micro_type;
  double geo_params[4];
  double bmat[NPE][NVOI][NPEDIM];
  int *elem_type;
  struct orc_material mats[3];
  int nr_max_its, cg_max_its;
  double nr_max_tol, nr_rel_tol, cg_abs_tol, cg_rel_tol;
  int lin_stress, subiterations, nsubiterations;
  double ctan_lin[NVOI * NVOI];
  double Vm, Vf;
  orc_gp *gp;
  int use_A0, its_with_A0, nA0;
  orc_ell *A0; /* micropp.cpp:128-143: the Jacobian at u = 0, one per OpenMP thread (it holds CG work vectors) */
};

/* ------------------------------------------------------------------------------------------------ */
/* Configuration                                                                                      */

/* Defaults of micropp_params_t (types.hpp:43-63, params.hpp:32-35, ell.hpp:33-35). */
void orc_config_default(struct orc_config *c) {
  memset(c, 0, sizeof(*c));
  c->ngp = 1;
  c->geo_params[0] = c->geo_params[1] = c->geo_params[2] = c->geo_params[3] = 0.1;
  c->subiterations = 0;
  c->nsubiterations = 10;
  c->nr_max_its = 4;
  c->nr_max_tol = 1.0e-10;
  c->nr_rel_tol = 1.0e-3;
  c->cg_max_its = 1000;
  c->cg_abs_tol = 1.0e-50;
  c->cg_rel_tol = 1.0e-5;
  c->calc_ctan_lin = 1;
  c->its_with_A0 = 1;
  c->lin_stress = 1;
}

/* material_set (material.c:26-38). */
void orc_material_set(struct orc_material *m, int type, double E, double nu, double Ka, double Sy, double Xt) {
  m->E = E;
  m->nu = nu;
  m->Ka = Ka;
  m->Sy = Sy;
  m->Xt = Xt;
  m->type = type;
  m->k = E / (3. * (1. - 2. * nu));
  m->mu = E / (2. * (1. + nu));
  m->lambda = nu * E / ((1. + nu) * (1. - 2. * nu));
}

/* ------------------------------------------------------------------------------------------------ */
/* Material laws (material.cpp:48-307)                                                                */

static void mat_get_stress(const struct orc_material *m, const double *eps, double *stress, const double *vars);

/* get_dev_tensor (material.cpp:65-69). */
static void dev_tensor(const double t[6], double d[6]) {
  memcpy(d, t, 6 * sizeof(double));
  for (int i = 0; i < 3; i++) d[i] -= (1 / 3.0) * (t[0] + t[1] + t[2]);
}

/* material_elastic::get_stress (material.cpp:76-82). */
static void elastic_stress(const struct orc_material *m, const double *eps, double *s) {
  for (int i = 0; i < 3; ++i) s[i] = m->lambda * (eps[0] + eps[1] + eps[2]) + 2 * m->mu * eps[i];
  for (int i = 3; i < 6; ++i) s[i] = m->mu * eps[i];
}

/* material_plastic::plastic_law (material.cpp:110-147). */
static int plastic_law(const struct orc_material *m, const double eps[6], const double *eps_p_old,
                       const double *alpha_old_p, double *dl, double normal[6], double s_trial[6]) {
  const double zeros[6] = {0.0};
  const double alpha_old = alpha_old_p ? *alpha_old_p : 0;
  const double *ep = eps_p_old ? eps_p_old : zeros;
  double eps_dev[6], ep_dev[6];
  dev_tensor(ep, ep_dev);
  dev_tensor(eps, eps_dev);
  for (int i = 0; i < 3; ++i) s_trial[i] = 2 * m->mu * (eps_dev[i] - ep_dev[i]);
  for (int i = 3; i < 6; ++i) s_trial[i] = m->mu * (eps_dev[i] - ep_dev[i]);
  double tmp = 0.0;
  for (int i = 0; i < 6; ++i) tmp += s_trial[i] * s_trial[i];
  const double s_norm = sqrt(tmp);
  const double f_trial = s_norm - SQRT_2DIV3 * (m->Sy + m->Ka * alpha_old);
  if (f_trial > 0) {
    for (int i = 0; i < 6; ++i) normal[i] = s_trial[i] / s_norm;
    *dl = f_trial / (2. * m->mu * (1. + m->Ka / (3. * m->mu)));
    return 1;
  }
  memset(normal, 0, 6 * sizeof(double));
  *dl = 0;
  return 0;
}

/* material_damage::hardening_law (material.cpp:205-225). */
static double damage_hardening(const struct orc_material *m, double r) {
  const double Ey = 10.0e4;
  const double inf_Ey = 10. * Ey;
  const double H0 = 10.0, H1 = 5.0;
  const double r0 = Ey / sqrt(m->E);
  const double q0 = r0;
  const double q1 = inf_Ey / sqrt(m->E);
  const double r1 = r0 + (q1 - q0) / H0;
  if (r < r0) return 0.0;
  if (r >= r0 && r < r1) return q0 + H0 * (r - r0);
  return q1 + H1 * (r - r1);
}

/* material_damage::damage_law (material.cpp:227-268). */
static int damage_law(const struct orc_material *m, const double *eps, double r_old, double D_old, double *r_out,
                      double *D_out, double *stress) {
  double local[6] = {0.0};
  double *s = stress ? stress : local;
  elastic_stress(m, eps, s);
  double product = 0.0;
  for (int i = 0; i < 6; ++i) product += s[i] * eps[i];
  const double r = (product >= 0) ? sqrt(product) : 0;
  const double r_old_a = (r_old < m->Xt / sqrt(m->E)) ? m->Xt / sqrt(m->E) : r_old;
  if (r <= r_old_a) {
    *r_out = r_old_a;
    *D_out = D_old;
    return 0;
  }
  const double q = damage_hardening(m, r);
  *r_out = r;
  *D_out = 1. - q / r;
  return 1;
}

/* get_stress of the three laws (material.cpp:76-82, 149-162, 270-284). `vars` may be NULL. */
static void mat_get_stress(const struct orc_material *m, const double *eps, double *stress, const double *vars) {
  if (m->type == MAT_ELASTIC) {
    elastic_stress(m, eps, stress);
  } else if (m->type == MAT_PLASTIC) {
    double dl, normal[6], s_trial[6];
    plastic_law(m, eps, vars ? &vars[0] : NULL, vars ? &vars[6] : NULL, &dl, normal, s_trial);
    memcpy(stress, s_trial, 6 * sizeof(double));
    for (int i = 0; i < 3; ++i) stress[i] += m->k * (eps[0] + eps[1] + eps[2]);
    for (int i = 0; i < 6; ++i) stress[i] -= 2 * m->mu * dl * normal[i];
  } else {
    const double r_old = vars ? vars[0] : 0.0;
    const double D_old = vars ? vars[1] : 0.0;
    double D, r;
    damage_law(m, eps, r_old, D_old, &r, &D, stress);
    for (int i = 0; i < 6; ++i) stress[i] *= (1 - D);
  }
}

/* get_ctan: elastic closed form (material.cpp:84-95); plastic and damage by forward differences of the
 * stress, apply_perturbation (material.cpp:48-63). */
static void mat_get_ctan(const struct orc_material *m, const double *eps, double *ctan, const double *vars) {
  if (m->type == MAT_ELASTIC) {
    memset(ctan, 0, 36 * sizeof(double));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) ctan[i * 6 + j] += m->lambda;
    for (int i = 0; i < 3; ++i) ctan[i * 6 + i] += 2 * m->mu;
    for (int i = 3; i < 6; ++i) ctan[i * 6 + i] = m->mu;
    return;
  }
  double s0[6];
  mat_get_stress(m, eps, s0, vars);
  for (int i = 0; i < 6; ++i) {
    double e1[6], s1[6];
    memcpy(e1, eps, 6 * sizeof(double));
    e1[i] += D_EPS_CTAN;
    mat_get_stress(m, e1, s1, vars);
    for (int j = 0; j < 6; ++j) ctan[j * 6 + i] = (s1[j] - s0[j]) / D_EPS_CTAN;
  }
}

/* evolute of the three laws (material.cpp:97-100, 168-181, 291-302).  Returns the nonlinear flag. */
static int mat_evolute(const struct orc_material *m, const double *eps, const double *vars_old, double *vars_new) {
  if (m->type == MAT_ELASTIC) return 0;
  if (m->type == MAT_PLASTIC) {
    const double *ep_old = vars_old ? &vars_old[0] : NULL;
    const double *al_old = vars_old ? &vars_old[6] : NULL;
    double *ep_new = vars_new ? &vars_new[0] : NULL;
    double *al_new = vars_new ? &vars_new[6] : NULL;
    double dl, normal[6], s_trial[6];
    const int nl = plastic_law(m, eps, ep_old, al_old, &dl, normal, s_trial);
    if (ep_old && ep_new)
      for (int i = 0; i < 6; ++i) ep_new[i] = ep_old[i] + dl * normal[i];
    if (al_old && al_new) *al_new = *al_old + SQRT_2DIV3 * dl + 0;
    return nl;
  }
  const double r_old = vars_old ? vars_old[0] : 0;
  const double D_old = vars_old ? vars_old[1] : 0;
  return damage_law(m, eps, r_old, D_old, &vars_new[0], &vars_new[1], NULL);
}

/* ------------------------------------------------------------------------------------------------ */
/* Geometry                                                                                           */

/* Hex8 local node corners in the reference's numbering (common.cpp:28-40): 0..3 counter-clockwise on
 * z=0, 4..7 the same on z=1.  Gauss points use the same corner pattern scaled by CONSTXG
 * (micropp.hpp:93-96). */
static const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                 {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

/* calc_bmat (micro3D.cpp:80-120): trilinear shape-function gradients at Gauss point `gp`.  The product is
 * formed as (s_a*(1+s_b*xi_b))*(1+s_c*xi_c)/8*2/h, which equals the reference expression bit for bit
 * (multiplying by -1 only flips the sign). */
void orc_calc_bmat(double dx, double dy, double dz, int gp, double bmat[6][24]) {
  double xg[3];
  for (int d = 0; d < 3; ++d) xg[d] = corner[gp][d] ? +CONSTXG : -CONSTXG;
  const double h[3] = {dx, dy, dz};
  for (int i = 0; i < 8; ++i) {
    double s[3], dsh[3];
    for (int d = 0; d < 3; ++d) s[d] = corner[i][d] ? 1.0 : -1.0;
    for (int d = 0; d < 3; ++d) {
      /* d=0 uses (y, z); d=1 uses (x, z); d=2 uses (x, y) */
      const int p = (d == 0) ? 1 : 0;
      const int q = (d == 2) ? 1 : 2;
      const double f1 = 1 + s[p] * xg[p];
      const double f2 = 1 + s[q] * xg[q];
      dsh[d] = s[d] * f1 * f2 / 8. * 2. / h[d];
    }
    bmat[0][i * 3 + 0] = dsh[0]; bmat[0][i * 3 + 1] = 0;      bmat[0][i * 3 + 2] = 0;
    bmat[1][i * 3 + 0] = 0;      bmat[1][i * 3 + 1] = dsh[1]; bmat[1][i * 3 + 2] = 0;
    bmat[2][i * 3 + 0] = 0;      bmat[2][i * 3 + 1] = 0;      bmat[2][i * 3 + 2] = dsh[2];
    bmat[3][i * 3 + 0] = dsh[1]; bmat[3][i * 3 + 1] = dsh[0]; bmat[3][i * 3 + 2] = 0;
    bmat[4][i * 3 + 0] = dsh[2]; bmat[4][i * 3 + 1] = 0;      bmat[4][i * 3 + 2] = dsh[0];
    bmat[5][i * 3 + 0] = 0;      bmat[5][i * 3 + 1] = dsh[2]; bmat[5][i * 3 + 2] = dsh[1];
  }
}

/* util.hpp:58-128 predicates used by get_elem_type. */
static double norm3(const double v[3]) {
  double t = 0;
  for (int i = 0; i < 3; ++i) t += v[i] * v[i];
  return sqrt(t);
}
static int in_sphere(const double c[3], double rad, const double p[3]) {
  const double v[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
  return norm3(v) < rad;
}
static int in_cylinder(const double dir[3], const double c[3], double rad, const double p[3]) {
  const double v[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
  double dv = 0;
  for (int i = 0; i < 3; ++i) dv += dir[i] * v[i];
  const double nd = norm3(dir), nv = norm3(v);
  const double cs = dv / (nd * nv);
  const double sn = sqrt(1 - cs * cs);
  return nv * sn <= rad;
}

/* Sphere and fibre tables of MIC3D_SPHERES and MIC3D_FIBS_20_DISORDER (micropp.cpp:455-480, 515-530):
 * data that defines those microstructures, kept identical for a drop-in. */
static const double sph_c[40][3] = {
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
static const double sph_r[40] = {.5741, .1735, .5065, .8565, .9735, .7087, .9585, .2843, .4029, .2574,
                                 .1575, .3316, .1874, .6300, .7049, .7258, .8002, .8176, .9970, .4736,
                                 .6351, .3140, .3440, .2444, .3894, .5234, .1658, .4020, .6813, .2060,
                                 .1427, .9332, .5406, .9765, .0956, .6432, .9998, .4166, .6907, .0404};
static const double fib_d[20][2] = {{.5741, .8515}, {.1735, .1103}, {.5065, .4600}, {.8565, .9045},
                                    {.9735, .6313}, {.7087, .1547}, {.9585, .0220}, {.2843, .4062},
                                    {.4029, .8095}, {.2574, .4742}, {.1575, .0768}, {.3316, .0320},
                                    {.1874, .6364}, {.6300, .2688}, {.7049, .5137}, {.7258, .2799},
                                    {.8002, .4794}, {.8176, .4142}, {.9970, .2189}, {.4736, .6202}};

/* get_elem_type (micropp.cpp:338-544): phase of element (ex,ey,ez) from its centroid. */
static int elem_type_of(const orc_rve *h, int ex, int ey, int ez) {
  const double lx = h->lx, ly = h->ly, lz = h->lz;
  const double coor[3] = {ex * h->dx + h->dx / 2., ey * h->dy + h->dy / 2., ez * h->dz + h->dz / 2.};
  const double *g = h->geo_params;
  const double dir_x[3] = {1, 0, 0}, dir_z[3] = {0, 0, 1};
  switch (h->micro_type) {
    case MIC_HOMOGENEOUS:
      return 0;
    case MIC_SPHERE: {
      const double c[3] = {lx / 2, ly / 2, lz / 2};
      return in_sphere(c, g[0], coor);
    }
    case MIC_LAYER_Y:
      return coor[1] < g[0];
    case MIC_CILI_FIB_X: {
      const double c[3] = {lx / 2, ly / 2, lz / 2};
      return in_cylinder(dir_x, c, g[0], coor);
    }
    case MIC_CILI_FIB_Z: {
      const double c[3] = {lx / 2, ly / 2, lz / 2};
      return in_cylinder(dir_z, c, g[0], coor);
    }
    case MIC_CILI_FIB_XZ: {
      const double c1[3] = {lx / 2., ly * .75, lz / 2.}, c2[3] = {lx / 2., ly * .25, lz / 2.};
      return (in_cylinder(dir_z, c1, g[0], coor) || in_cylinder(dir_x, c2, g[0], coor)) ? 1 : 0;
    }
    case MIC_QUAD_FIB_XYZ:
    case MIC_QUAD_FIB_XZ:
    case MIC_QUAD_FIB_XZ_BROKEN_X: {
      const double w = g[0];
      const double c[3] = {lx / 2., ly / 2., lz / 2.};
      const int xy = fabs(coor[0] - c[0]) < w && fabs(coor[1] - c[1]) < w;
      const int xz = fabs(coor[0] - c[0]) < w && fabs(coor[2] - c[2]) < w;
      const int yz = fabs(coor[1] - c[1]) < w && fabs(coor[2] - c[2]) < w;
      if (h->micro_type == MIC_QUAD_FIB_XYZ) return (xy || xz || yz) ? 1 : 0;
      if (h->micro_type == MIC_QUAD_FIB_XZ) return (xy || yz) ? 1 : 0;
      if (xy) return 1;
      return (yz && (coor[0] < lx * .8 || coor[0] > lx * .9)) ? 1 : 0;
    }
    case MIC3D_SPHERES:
      for (int i = 0; i < 40; ++i)
        if (in_sphere(sph_c[i], 0.1 * sph_r[i], coor)) return 1;
      return 0;
    case MIC3D_8: {
      const double rc = 0.1, wf = 0.02, wc = 0.01;
      const double c1[3] = {lx * .25, ly * .75, 0.0}, c2[3] = {lx * .75, ly * .75, 0.0};
      const double c3[3] = {0.0, ly * .25, lz * .25}, c4[3] = {0.0, ly * .25, lz * .75};
      if (in_cylinder(dir_z, c1, rc, coor) || in_cylinder(dir_z, c2, rc, coor) || in_cylinder(dir_x, c3, rc, coor) ||
          in_cylinder(dir_x, c4, rc, coor))
        return 1;
      if (in_cylinder(dir_z, c1, rc + wc, coor) || in_cylinder(dir_z, c2, rc + wc, coor) ||
          in_cylinder(dir_x, c3, rc + wc, coor) || in_cylinder(dir_x, c4, rc + wc, coor) || fabs(coor[1] - ly / 2) < wf)
        return 2;
      return 0;
    }
    case MIC3D_FIBS_20_ORDER: {
      const double dzf = 1.0 / (5 + 1), dyf = 1.0 / (4 + 1);
      for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 4; ++j) {
          const double c[3] = {0.0, (j + 1) * dyf, (i + 1) * dzf};
          if (in_cylinder(dir_x, c, 0.05, coor)) return 1;
        }
      return 0;
    }
    case MIC3D_FIBS_20_DISORDER:
      for (int i = 0; i < 20; ++i) {
        const double d[3] = {1, fib_d[i][0], fib_d[i][1]};
        if (in_cylinder(d, sph_c[i], 0.05, coor)) return 1;
      }
      return 0;
    default:
      fprintf(stderr, "Invalid micro_type = %d\n", h->micro_type);
      return -1;
  }
}

/* ------------------------------------------------------------------------------------------------ */
/* ELL matrix and DPCG (ell-common.cpp:34-139,166-198,200,238-297; ell.cpp:35-122)                   */

static void ell_init(orc_ell *m, const int ns[3], double min_err, double rel_err, int max_its) {
  const int nx = ns[0], ny = ns[1], nz = ns[2];
  const int nxny = nx * ny;
  memcpy(m->n, ns, sizeof(m->n));
  m->nn = nx * ny * nz;
  m->nrow = m->nn * 3;
  m->cols = (int *)malloc((size_t)NNZ * m->nrow * sizeof(int));
  m->vals = (double *)malloc((size_t)NNZ * m->nrow * sizeof(double));
  m->max_its = max_its;
  m->min_err = min_err;
  m->rel_err = rel_err;
  m->k = (double *)malloc(m->nrow * sizeof(double));
  m->r = (double *)malloc(m->nrow * sizeof(double));
  m->z = (double *)malloc(m->nrow * sizeof(double));
  m->p = (double *)malloc(m->nrow * sizeof(double));
  m->Ap = (double *)malloc(m->nrow * sizeof(double));
  /* 27-point stencil columns ordered (dz,dy,dx) in {-1,0,1}^3; a neighbour outside the grid points at
   * node 0 (ell-common.cpp:95-134). */
  for (int zi = 0; zi < nz; ++zi)
    for (int yi = 0; yi < ny; ++yi)
      for (int xi = 0; xi < nx; ++xi) {
        const int ni = zi * nxny + yi * nx + xi;
        int ix[27];
        for (int s = 0; s < 27; ++s) {
          const int ddz = s / 9 - 1, ddy = (s / 3) % 3 - 1, ddx = s % 3 - 1;
          const int x = xi + ddx, y = yi + ddy, z = zi + ddz;
          const int out = x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz;
          ix[s] = out ? 0 : ni + ddz * nxny + ddy * nx + ddx;
        }
        for (int fi = 0; fi < 3; ++fi) {
          int *c = &m->cols[(size_t)ni * 3 * NNZ + fi * NNZ];
          for (int s = 0; s < 27; ++s)
            for (int fj = 0; fj < 3; ++fj) c[s * 3 + fj] = ix[s] * 3 + fj;
        }
      }
}

static void ell_free(orc_ell *m) {
  free(m->cols);
  free(m->vals);
  free(m->k);
  free(m->r);
  free(m->z);
  free(m->p);
  free(m->Ap);
}

/* Stencil slot of local node j seen from local node i (the cols_row table of ell_add_3D,
 * ell-common.cpp:172-175), derived from the corner offsets. */
static int slot_of(int i, int j) {
  const int ddx = corner[j][0] - corner[i][0], ddy = corner[j][1] - corner[i][1], ddz = corner[j][2] - corner[i][2];
  return (ddz + 1) * 9 + (ddy + 1) * 3 + (ddx + 1);
}

/* ell_add_3D (ell-common.cpp:166-198). */
static void ell_add_3d(orc_ell *m, int ex, int ey, int ez, const double *Ae) {
  const int nx = m->n[0], ny = m->n[1];
  const int nxny = nx * ny;
  const int n0 = ez * nxny + ey * nx + ex;
  int glo[8];
  for (int i = 0; i < 8; ++i) glo[i] = n0 + corner[i][2] * nxny + corner[i][1] * nx + corner[i][0];
  for (int fi = 0; fi < 3; ++fi)
    for (int fj = 0; fj < 3; ++fj)
      for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j)
          m->vals[(size_t)glo[i] * 3 * NNZ + slot_of(i, j) * 3 + fi * NNZ + fj] += Ae[i * 72 + fi * 24 + j * 3 + fj];
}

static int on_boundary(int i, int j, int k, int nx, int ny, int nz) {
  return i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1;
}

/* ell_set_bc_3D (ell-common.cpp:238-297): every boundary row becomes an identity row. */
static void ell_set_bc_3d(orc_ell *m) {
  const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (!on_boundary(i, j, k, nx, ny, nz)) continue;
        const int n = (k * ny + j) * nx + i;
        for (int d = 0; d < 3; ++d) {
          double *row = &m->vals[(size_t)n * 3 * NNZ + d * NNZ];
          memset(row, 0, NNZ * sizeof(double));
          row[13 * 3 + d] = 1;
        }
      }
}

/* ell_mvp (ell.cpp:35-45). */
static void ell_mvp(const orc_ell *m, const double *x, double *y) {
  for (int i = 0; i < m->nrow; i++) {
    double tmp = 0;
    const size_t ix = (size_t)i * NNZ;
    for (int j = 0; j < NNZ; j++) tmp += m->vals[ix + j] * x[m->cols[ix + j]];
    y[i] = tmp;
  }
}

/* get_dot (ell.cpp:53-57).  With -DORC_BLOCKED_DOTS the sum is taken in blocks of 768 terms whose partial
 * sums are added last, the association of a GPU grid reduction; that build only serves to measure how much
 * a different summation order moves the results (tests/test_rounding_floor.py). */
__attribute__((unused)) static double get_dot(const double *a, const double *b, int n) {
#ifdef ORC_BLOCKED_DOTS
  double total = 0.0;
  for (int i0 = 0; i0 < n; i0 += 768) {
    double s = 0.0;
    const int i1 = (i0 + 768 < n) ? i0 + 768 : n;
    for (int i = i0; i < i1; ++i) s += a[i] * b[i];
    total += s;
  }
  return total;
#else
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
#endif
}

#ifdef ORC_GPU_ORDER
/* With -DORC_GPU_ORDER the CG's dot products are summed in the order of the GB300 library's FP64 CG kernels:
 * per-thread partials (one node of 3 rows per thread in the set-up and the SpMV, 4 rows strided by the grid
 * per thread in the update), 256-thread blocks, shuffle-down warp trees, a tree over the 8 warp sums, and the
 * last block adding the block partials strided by its 256 threads before one more block tree.  That build only
 * serves to measure how much a different summation order moves the results (tests/test_rounding_floor.py). */
#define GPU_BLOCK 256
#define GPU_UPD_ROWS 4

static double warp_tree(double w[32]) {
  for (int o = 16; o > 0; o >>= 1)
    for (int l = 0; l < 32; ++l) w[l] = w[l] + (l + o < 32 ? w[l + o] : w[l]);
  return w[0];
}

static double block_tree(const double *t, long n) {
  double sh[32];
  for (int wi = 0; wi < 32; ++wi) sh[wi] = 0.0;
  for (int wi = 0; wi < GPU_BLOCK / 32; ++wi) {
    double w[32];
    for (int l = 0; l < 32; ++l) w[l] = (wi * 32 + l < n) ? t[wi * 32 + l] : 0.0;
    sh[wi] = warp_tree(w);
  }
  return warp_tree(sh);
}

/* Sum of per-thread partials part[0..nthreads) by the grid tree. */
static double grid_tree(const double *part, long nthreads) {
  const long nb = (nthreads + GPU_BLOCK - 1) / GPU_BLOCK;
  double *red = (double *)malloc(nb * sizeof(double));
  for (long b = 0; b < nb; ++b) {
    const long rem = nthreads - b * GPU_BLOCK;
    red[b] = block_tree(part + b * GPU_BLOCK, rem < GPU_BLOCK ? rem : GPU_BLOCK);
  }
  double acc[GPU_BLOCK];
  for (int t = 0; t < GPU_BLOCK; ++t) {
    acc[t] = 0.0;
    for (long b = t; b < nb; b += GPU_BLOCK) acc[t] += red[b];
  }
  free(red);
  return block_tree(acc, GPU_BLOCK);
}

static int node_on_boundary(const orc_ell *m, int n) {
  const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
  return on_boundary(n % nx, (n / nx) % ny, n / (nx * ny), nx, ny, nz);
}

/* r.z and z.z of the CG set-up, one node per thread. */
static void gpu_setup_dots(const orc_ell *m, const double *r, const double *z, double *rz, double *zz) {
  const long nt = (long)((m->nn + GPU_BLOCK - 1) / GPU_BLOCK) * GPU_BLOCK;
  double *a = (double *)calloc(nt, sizeof(double)), *b = (double *)calloc(nt, sizeof(double));
  for (int n = 0; n < m->nn; ++n)
    for (int d = 0; d < 3; ++d) {
      a[n] += r[n * 3 + d] * z[n * 3 + d];
      b[n] += z[n * 3 + d] * z[n * 3 + d];
    }
  *rz = grid_tree(a, nt);
  *zz = grid_tree(b, nt);
  free(a);
  free(b);
}

/* p.Ap of the SpMV, one node per thread: p0 y0 + p1 y1 + p2 y2 inside, p.p on boundary nodes. */
static double gpu_spmv_dot(const orc_ell *m, const double *p, const double *y) {
  const long nt = (long)((m->nn + GPU_BLOCK - 1) / GPU_BLOCK) * GPU_BLOCK;
  double *a = (double *)calloc(nt, sizeof(double));
  for (int n = 0; n < m->nn; ++n) {
    const double *q = p + n * 3, *w = y + n * 3;
    if (node_on_boundary(m, n)) {
      for (int d = 0; d < 3; ++d) a[n] += q[d] * q[d];
    } else {
      a[n] = q[0] * w[0] + q[1] * w[1] + q[2] * w[2];
    }
  }
  const double s = grid_tree(a, nt);
  free(a);
  return s;
}

/* z.z and r.z of the update: GPU_UPD_ROWS rows per thread, strided by the grid. */
static void gpu_update_dots(const orc_ell *m, const double *r, const double *z, double *zz, double *rz) {
  const long per = (long)GPU_UPD_ROWS * GPU_BLOCK;
  const long nb = (m->nrow + per - 1) / per, nt = nb * GPU_BLOCK, stride = nt;
  double *a = (double *)calloc(nt, sizeof(double)), *b = (double *)calloc(nt, sizeof(double));
  for (long t = 0; t < nt; ++t)
    for (long row0 = t; row0 < m->nrow; row0 += GPU_UPD_ROWS * stride)
      for (int q = 0; q < GPU_UPD_ROWS; ++q) {
        const long row = row0 + q * stride;
        if (row < m->nrow) {
          a[t] += z[row] * z[row];
          b[t] += r[row] * z[row];
        }
      }
  *zz = grid_tree(a, nt);
  *rz = grid_tree(b, nt);
  free(a);
  free(b);
}
#endif

/* ell_solve_cgpd (ell.cpp:66-122): Jacobi-preconditioned CG from x0 = 0, stopping on ||z||. */
static int ell_solve_cgpd(orc_ell *m, const double *b, double *x, double *err) {
  double t0 = wtime();
  for (int i = 0; i < m->nn; i++)
    for (int d = 0; d < 3; d++) m->k[i * 3 + d] = 1 / m->vals[(size_t)i * 3 * NNZ + 13 * 3 + d * NNZ + d];
  for (int i = 0; i < m->nrow; ++i) x[i] = 0.0;
  ell_mvp(m, x, m->r);
  for (int i = 0; i < m->nrow; ++i) m->r[i] = b[i] - m->r[i];
  for (int i = 0; i < m->nrow; ++i) m->z[i] = m->k[i] * m->r[i];
  for (int i = 0; i < m->nrow; ++i) m->p[i] = m->z[i];
#ifdef ORC_GPU_ORDER
  double rz, zz0;
  gpu_setup_dots(m, m->r, m->z, &rz, &zz0);
  const double pnorm_0 = sqrt(zz0);
#else
  double rz = get_dot(m->r, m->z, m->nrow);
  const double pnorm_0 = sqrt(get_dot(m->z, m->z, m->nrow));
#endif
  double pnorm = pnorm_0;
  int its = 0;
  op_add(ORC_OP_CG_SETUP, 1, t0);
  t0 = wtime();
  while (its < m->max_its) {
    if (pnorm < m->min_err || pnorm < pnorm_0 * m->rel_err) break;
    ell_mvp(m, m->p, m->Ap);
#ifdef ORC_GPU_ORDER
    const double pAp = gpu_spmv_dot(m, m->p, m->Ap);
#else
    const double pAp = get_dot(m->p, m->Ap, m->nrow);
#endif
    const double alpha = rz / pAp;
    for (int i = 0; i < m->nrow; ++i) x[i] += alpha * m->p[i];
    for (int i = 0; i < m->nrow; ++i) m->r[i] -= alpha * m->Ap[i];
    for (int i = 0; i < m->nrow; ++i) m->z[i] = m->k[i] * m->r[i];
#ifdef ORC_GPU_ORDER
    double zz, rz_n;
    gpu_update_dots(m, m->r, m->z, &zz, &rz_n);
    pnorm = sqrt(zz);
#else
    pnorm = sqrt(get_dot(m->z, m->z, m->nrow));
    const double rz_n = get_dot(m->r, m->z, m->nrow);
#endif
    const double beta = rz_n / rz;
    for (int i = 0; i < m->nrow; ++i) m->p[i] = m->z[i] + beta * m->p[i];
    rz = rz_n;
    its++;
  }
  op_add(ORC_OP_CG_ITER, its, t0);
  *err = rz;
  return its;
}

/* ------------------------------------------------------------------------------------------------ */
/* FE kernels                                                                                         */

static const struct orc_material *elem_mat(const orc_rve *h, int e) { return &h->mats[h->elem_type[e]]; }

/* get_elem_nodes + get_elem_displ + get_strain (common.cpp:28-72). */
static void get_strain(const orc_rve *h, const double *u, int gp, double *strain, int ex, int ey, int ez) {
  const int nxny = h->nx * h->ny;
  const int n0 = ez * nxny + ey * h->nx + ex;
  double ue[NPEDIM];
  for (int i = 0; i < NPE; ++i) {
    const int n = n0 + corner[i][2] * nxny + corner[i][1] * h->nx + corner[i][0];
    for (int d = 0; d < DIM; ++d) ue[i * DIM + d] = u[n * DIM + d];
  }
  for (int i = 0; i < NVOI; ++i) strain[i] = 0;
  for (int v = 0; v < NVOI; ++v)
    for (int i = 0; i < NPEDIM; ++i) strain[v] += h->bmat[gp][v][i] * ue[i];
}

static const double *gp_vars(const orc_rve *h, const double *vars, int e, int gp) {
  (void)h;
  return vars ? &vars[(size_t)e * NPE * NVAR_GP + gp * NVAR_GP] : NULL;
}

/* set_displ_bc (micro3D.cpp:26-78): u = eps_t * x on the six faces.  The faces are written in the order
 * z=0, z=lz, y=0, y=ly, x=0, x=lx, so an edge or corner node keeps the coordinates of the last face that
 * contains it. */
static void set_displ_bc(const orc_rve *h, const double eps[6], double *u) {
  const double et[3][3] = {{eps[0], 0.5 * eps[3], 0.5 * eps[4]},
                           {0.5 * eps[3], eps[1], 0.5 * eps[5]},
                           {0.5 * eps[4], 0.5 * eps[5], eps[2]}};
  const int nx = h->nx, ny = h->ny, nz = h->nz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double c[3];
        if (i == nx - 1) {
          c[0] = h->lx; c[1] = j * h->dy; c[2] = k * h->dz;
        } else if (i == 0) {
          c[0] = 0; c[1] = j * h->dy; c[2] = k * h->dz;
        } else if (j == ny - 1) {
          c[0] = i * h->dx; c[1] = h->ly; c[2] = k * h->dz;
        } else if (j == 0) {
          c[0] = i * h->dx; c[1] = 0; c[2] = k * h->dz;
        } else if (k == nz - 1) {
          c[0] = i * h->dx; c[1] = j * h->dy; c[2] = h->lz;
        } else if (k == 0) {
          c[0] = i * h->dx; c[1] = j * h->dy; c[2] = 0;
        } else {
          continue;
        }
        const int n = (k * ny + j) * nx + i;
        for (int a = 0; a < 3; ++a) {
          double t = 0.0;
          for (int b = 0; b < 3; ++b) t += et[a][b] * c[b];
          u[n * 3 + a] = t;
        }
      }
}

/* get_elem_rhs (assembly.cpp:123-138). */
static void get_elem_rhs(const orc_rve *h, const double *u, const double *vars, double be[NPEDIM], int ex, int ey,
                         int ez) {
  const int e = (ez * h->ney + ey) * h->nex + ex;
  const struct orc_material *m = elem_mat(h, e);
  memset(be, 0, NPEDIM * sizeof(double));
  for (int gp = 0; gp < NPE; ++gp) {
    double strain[6], stress[6];
    get_strain(h, u, gp, strain, ex, ey, ez);
    mat_get_stress(m, strain, stress, gp_vars(h, vars, e, gp));
    for (int i = 0; i < NPEDIM; ++i)
      for (int j = 0; j < NVOI; ++j) be[i] += h->bmat[gp][j][i] * stress[j] * h->wg;
  }
}

/* assembly_rhs (assembly.cpp:27-103): b = -(sum_e be) with Dirichlet rows zeroed; returns ||b||_2. */
static double assembly_rhs(const orc_rve *h, const double *u, const double *vars, double *b) {
  const double t0 = wtime();
  const int nx = h->nx, ny = h->ny, nz = h->nz, nxny = nx * ny;
  memset(b, 0, h->nndim * sizeof(double));
  for (int ez = 0; ez < h->nez; ++ez)
    for (int ey = 0; ey < h->ney; ++ey)
      for (int ex = 0; ex < h->nex; ++ex) {
        double be[NPEDIM];
        get_elem_rhs(h, u, vars, be, ex, ey, ez);
        const int n0 = ez * nxny + ey * nx + ex;
        for (int i = 0; i < NPE; ++i) {
          const int n = n0 + corner[i][2] * nxny + corner[i][1] * nx + corner[i][0];
          for (int d = 0; d < DIM; ++d) b[n * DIM + d] += be[i * DIM + d];
        }
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        if (on_boundary(i, j, k, nx, ny, nz)) memset(&b[((k * ny + j) * nx + i) * 3], 0, 3 * sizeof(double));
  for (int i = 0; i < h->nndim; ++i) b[i] = -b[i];
  double norm = 0.0;
  for (int i = 0; i < h->nndim; ++i) norm += b[i] * b[i];
  op_add(ORC_OP_RESIDUAL, 1, t0);
  return sqrt(norm);
}

/* get_elem_mat (assembly.cpp:140-178). */
static void get_elem_mat(const orc_rve *h, const double *u, const double *vars, double *Ae, int ex, int ey, int ez) {
  const int e = (ez * h->ney + ey) * h->nex + ex;
  const struct orc_material *m = elem_mat(h, e);
  double TAe[NPEDIM * NPEDIM];
  memset(TAe, 0, sizeof(TAe));
  for (int gp = 0; gp < NPE; ++gp) {
    double eps[6], ctan[36], cxb[NVOI][NPEDIM];
    get_strain(h, u, gp, eps, ex, ey, ez);
    mat_get_ctan(m, eps, ctan, gp_vars(h, vars, e, gp));
    for (int i = 0; i < NVOI; ++i)
      for (int j = 0; j < NPEDIM; ++j) {
        double tmp = 0.0;
        for (int k = 0; k < NVOI; ++k) tmp += ctan[i * 6 + k] * h->bmat[gp][k][j];
        cxb[i][j] = tmp * h->wg;
      }
    for (int mm = 0; mm < NVOI; ++mm)
      for (int i = 0; i < NPEDIM; ++i) {
        const double bmi = h->bmat[gp][mm][i];
        for (int j = 0; j < NPEDIM; ++j) TAe[i * NPEDIM + j] += bmi * cxb[mm][j];
      }
  }
  memcpy(Ae, TAe, sizeof(TAe));
}

/* assembly_mat (assembly.cpp:105-121); note the ex-outer loop order. */
static void assembly_mat(const orc_rve *h, orc_ell *A, const double *u, const double *vars) {
  const double t0 = wtime();
  memset(A->vals, 0, (size_t)A->nrow * NNZ * sizeof(double));
  double Ae[NPEDIM * NPEDIM];
#ifdef ORC_GPU_ORDER
  /* the GB300 library's order: 8 colours by the parity of (ex, ey, ez), colour c = cx + 2 cy + 4 cz */
  for (int c = 0; c < 8; ++c)
    for (int ez = (c >> 2) & 1; ez < h->nez; ez += 2)
      for (int ey = (c >> 1) & 1; ey < h->ney; ey += 2)
        for (int ex = c & 1; ex < h->nex; ex += 2) {
          get_elem_mat(h, u, vars, Ae, ex, ey, ez);
          ell_add_3d(A, ex, ey, ez, Ae);
        }
#else
  for (int ex = 0; ex < h->nex; ++ex)
    for (int ey = 0; ey < h->ney; ++ey)
      for (int ez = 0; ez < h->nez; ++ez) {
        get_elem_mat(h, u, vars, Ae, ex, ey, ez);
        ell_add_3d(A, ex, ey, ez, Ae);
      }
#endif
  ell_set_bc_3d(A);
  op_add(ORC_OP_ASSEMBLY, 1, t0);
}

/* calc_ave_stress (average.cpp:57-82). */
static void calc_ave_stress(const orc_rve *h, const double *u, double ave[6], const double *vars) {
  const double t0 = wtime();
  memset(ave, 0, 6 * sizeof(double));
  for (int ez = 0; ez < h->nez; ++ez)
    for (int ey = 0; ey < h->ney; ++ey)
      for (int ex = 0; ex < h->nex; ++ex) {
        const int e = (ez * h->ney + ey) * h->nex + ex;
        double aux[6] = {0.0};
        for (int gp = 0; gp < NPE; ++gp) {
          double strain[6], stress[6];
          get_strain(h, u, gp, strain, ex, ey, ez);
          mat_get_stress(elem_mat(h, e), strain, stress, gp_vars(h, vars, e, gp));
          for (int v = 0; v < 6; ++v) aux[v] += stress[v] * h->wg;
        }
        for (int v = 0; v < 6; ++v) ave[v] += aux[v];
      }
  for (int v = 0; v < 6; ++v) ave[v] /= h->vol_tot;
  op_add(ORC_OP_AVE_STRESS, 1, t0);
}

/* calc_vars_new (update.cpp:32-56). */
static int calc_vars_new(const orc_rve *h, const double *u, const double *vold, double *vnew) {
  const double t0 = wtime();
  int nl = 0;
  for (int ez = 0; ez < h->nez; ++ez)
    for (int ey = 0; ey < h->ney; ++ey)
      for (int ex = 0; ex < h->nex; ++ex) {
        const int e = (ez * h->ney + ey) * h->nex + ex;
        for (int gp = 0; gp < NPE; ++gp) {
          double eps[6];
          get_strain(h, u, gp, eps, ex, ey, ez);
          nl |= mat_evolute(elem_mat(h, e), eps, gp_vars(h, vold, e, gp),
                            &vnew[(size_t)e * NPE * NVAR_GP + gp * NVAR_GP]);
        }
      }
  op_add(ORC_OP_VARS, 1, t0);
  return nl;
}

/* newton_raphson (solve.cpp:28-82); with use_A0 the first its_with_A0 iterations solve with A0
 * (solve.cpp:55-66). */
static void newton_raphson(const orc_rve *h, orc_ell *A, double *b, double *u, double *du, const double strain[6],
                           const double *vars, int *its_out, int *solver_its_out, int *conv_out) {
  int its = 0, solver_its = 0, converged = 0;
  set_displ_bc(h, strain, u);
  double norm = assembly_rhs(h, u, vars, b);
  const double norm_0 = norm;
  while (its < h->nr_max_its) {
    if (norm < h->nr_max_tol || norm < norm_0 * h->nr_rel_tol) {
      converged = 1;
      break;
    }
    orc_ell *A_ptr;
    if (!h->use_A0 || its > (h->its_with_A0 - 1)) {
      assembly_mat(h, A, u, vars);
      A_ptr = A;
    } else {
#ifdef _OPENMP
      A_ptr = &h->A0[omp_get_thread_num()];
#else
      A_ptr = &h->A0[0];
#endif
    }
    double cg_err;
    solver_its += ell_solve_cgpd(A_ptr, b, du, &cg_err);
    for (int i = 0; i < h->nndim; ++i) u[i] += du[i];
    norm = assembly_rhs(h, u, vars, b);
    its++;
  }
  *its_out = its;
  *solver_its_out = solver_its;
  *conv_out = converged;
}

/* ------------------------------------------------------------------------------------------------ */
/* Homogenization drivers                                                                             */

static void gp_allocate(const orc_rve *h, orc_gp *g) {
  g->vars_n = (double *)calloc(h->nvars, sizeof(double));
  g->vars_k = (double *)calloc(h->nvars, sizeof(double));
  g->allocated = 1;
}

/* homogenize_linear(gp) (homogenize.cpp:101-109). */
static void homogenize_linear_gp(orc_gp *g) {
  memset(g->stress, 0, sizeof(g->stress));
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) g->stress[i] += g->ctan[i * 6 + j] * g->strain[j];
}

/* homogenize_fe_one_way / homogenize_fe_full (homogenize.cpp:111-282).  They differ only in the final
 * ctan block, which runs for FE_FULL. */
static void homogenize_fe(const orc_rve *h, orc_gp *g, int full) {
  const double t_start = wtime();
  t_ops = g;
  orc_ell A;
  const int ns[3] = {h->nx, h->ny, h->nz};
  ell_init(&A, ns, h->cg_abs_tol, h->cg_rel_tol, h->cg_max_its);
  double *b = (double *)calloc(h->nndim, sizeof(double));
  double *du = (double *)calloc(h->nndim, sizeof(double));
  double *u = (double *)calloc(h->nndim, sizeof(double));
  double *vars_new_aux = (double *)calloc(h->nvars, sizeof(double));
  double *vars_new = g->allocated ? g->vars_k : vars_new_aux;
  const double *vars_n = g->allocated ? g->vars_n : NULL;
  int its, sits, conv;

  g->cost = 0;
  g->subiterated = 0;
  memcpy(u, g->u_n, h->nndim * sizeof(double));
  newton_raphson(h, &A, b, u, du, g->strain, vars_n, &its, &sits, &conv);
  g->nr_its = its;
  g->nr_solver_its = sits;
  g->nr_converged = conv;
  memcpy(g->u_k, u, h->nndim * sizeof(double));
  g->cost += sits;
  g->converged = conv;

  if (!g->converged && h->subiterations) {
    double eps_sub[6], deps_sub[6];
    memcpy(u, g->u_n, h->nndim * sizeof(double));
    memcpy(eps_sub, g->strain_old, sizeof(eps_sub));
    g->subiterated = 1;
    for (int i = 0; i < 6; ++i) deps_sub[i] = (g->strain[i] - g->strain_old[i]) / h->nsubiterations;
    for (int s = 0; s < h->nsubiterations; ++s) {
      for (int j = 0; j < 6; ++j) eps_sub[j] += deps_sub[j];
      newton_raphson(h, &A, b, u, du, eps_sub, vars_n, &its, &sits, &conv);
      g->cost += sits;
    }
    g->converged = conv;
    memcpy(g->u_k, u, h->nndim * sizeof(double));
  }

  if (h->lin_stress)
    homogenize_linear_gp(g);
  else
    calc_ave_stress(h, g->u_k, g->stress, vars_n);

  const int nl = calc_vars_new(h, g->u_k, vars_n, vars_new);
  if (nl && !g->allocated) {
    gp_allocate(h, g);
    memcpy(g->vars_k, vars_new, h->nvars * sizeof(double));
  }

  if (full && g->allocated) {
    /* 6 perturbed nonlinear solves from u_k, u carried across them; the cost adds the first solve's CG
     * count again each time (homogenize.cpp:256-275). */
    double eps_1[6], sig_0[6], sig_1[6];
    memcpy(u, g->u_k, h->nndim * sizeof(double));
    memcpy(sig_0, g->stress, sizeof(sig_0));
    const int first_sits = sits;
    for (int i = 0; i < 6; ++i) {
      int its2, sits2, conv2;
      memcpy(eps_1, g->strain, sizeof(eps_1));
      eps_1[i] += D_EPS_CTAN_AVE;
      newton_raphson(h, &A, b, u, du, eps_1, g->vars_n, &its2, &sits2, &conv2);
      g->cost += first_sits;
      calc_ave_stress(h, u, sig_1, g->vars_n);
      for (int v = 0; v < 6; ++v) g->ctan[v * 6 + i] = (sig_1[v] - sig_0[v]) / D_EPS_CTAN_AVE;
    }
  }
  ell_free(&A);
  free(b);
  free(u);
  free(du);
  free(vars_new_aux);
  op_add(ORC_OP_HOMOGENIZE, 1, t_start);
  t_ops = NULL;
}

/* calc_ctan_lin_fe_models (micropp.cpp:255-284). */
static void calc_ctan_lin_fe(orc_rve *h) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < 6; ++i) {
    orc_ell A;
    const int ns[3] = {h->nx, h->ny, h->nz};
    ell_init(&A, ns, h->cg_abs_tol, h->cg_rel_tol, h->cg_max_its);
    double *b = (double *)calloc(h->nndim, sizeof(double));
    double *du = (double *)calloc(h->nndim, sizeof(double));
    double *u = (double *)calloc(h->nndim, sizeof(double));
    double sig[6], eps[6] = {0.0};
    int its, sits, conv;
    eps[i] += D_EPS_CTAN_AVE;
    newton_raphson(h, &A, b, u, du, eps, NULL, &its, &sits, &conv);
    calc_ave_stress(h, u, sig, NULL);
    for (int v = 0; v < 6; ++v) h->ctan_lin[v * 6 + i] = sig[v] / D_EPS_CTAN_AVE;
    ell_free(&A);
    free(b);
    free(u);
    free(du);
  }
}

/* calc_ctan_lin_mix_rule_Chamis (micropp.cpp:286-331). */
static void ctan_mix_rule_chamis(const orc_rve *h, double ctan[36]) {
  const double Em = h->mats[0].E, nu_m = h->mats[0].nu, Gm = Em / (2 * (1 + nu_m));
  const double Ef = h->mats[1].E, nu_f = h->mats[1].nu, Gf = Ef / (2 * (1 + nu_f));
  const double E11 = h->Vf * Ef + h->Vm * Em;
  const double E22 = Em / (1 - sqrt(h->Vf) * (1 - Em / Ef));
  const double nu12 = h->Vf * nu_f + h->Vm * nu_m;
  const double G12 = Gm / (1 - sqrt(h->Vf) * (1 - Gm / Gf));
  const double nu23 = nu12;
  const double S[3][3] = {{1 / E11, -nu12 / E11, -nu12 / E11},
                          {-nu12 / E11, 1 / E22, -nu23 / E22},
                          {-nu12 / E11, -nu23 / E22, 1 / E22}};
  /* invert_3x3 (util.hpp:130-151) */
  const double det = S[0][0] * (S[1][1] * S[2][2] - S[2][1] * S[1][2]) -
                     S[0][1] * (S[1][0] * S[2][2] - S[2][0] * S[1][2]) +
                     S[0][2] * (S[1][0] * S[2][1] - S[2][0] * S[1][1]);
  double Si[3][3];
  Si[0][0] = +(S[1][1] * S[2][2] - S[2][1] * S[1][2]) / det;
  Si[0][1] = -(S[1][0] * S[2][2] - S[2][0] * S[1][2]) / det;
  Si[0][2] = +(S[1][0] * S[2][1] - S[2][0] * S[1][1]) / det;
  Si[1][0] = -(S[0][1] * S[2][2] - S[2][1] * S[0][2]) / det;
  Si[1][1] = +(S[0][0] * S[2][2] - S[2][0] * S[0][2]) / det;
  Si[1][2] = -(S[0][0] * S[2][1] - S[2][0] * S[0][1]) / det;
  Si[2][0] = +(S[0][1] * S[1][2] - S[1][1] * S[0][2]) / det;
  Si[2][1] = -(S[0][0] * S[1][2] - S[1][0] * S[0][2]) / det;
  Si[2][2] = +(S[0][0] * S[1][1] - S[1][0] * S[0][1]) / det;
  memset(ctan, 0, 36 * sizeof(double));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) ctan[i * 6 + j] = Si[i][j];
  ctan[3 * 6 + 3] = G12;
  ctan[4 * 6 + 4] = G12;
  ctan[5 * 6 + 5] = G12;
}

/* ------------------------------------------------------------------------------------------------ */
/* Public API                                                                                         */

/* micropp<3>::micropp (micropp.cpp:29-171). */
orc_rve *orc_new(const struct orc_config *c) {
  orc_rve *h = (orc_rve *)calloc(1, sizeof(orc_rve));
  h->ngp = c->ngp;
  h->nx = c->size[0];
  h->ny = c->size[1];
  h->nz = c->size[2];
  h->nn = h->nx * h->ny * h->nz;
  h->nndim = h->nn * 3;
  h->nex = h->nx - 1;
  h->ney = h->ny - 1;
  h->nez = h->nz - 1;
  h->nelem = h->nex * h->ney * h->nez;
  h->lx = h->ly = h->lz = 1.0;
  h->dx = h->lx / h->nex;
  h->dy = h->ly / h->ney;
  h->dz = h->lz / h->nez;
  h->wg = h->dx * h->dy * h->dz / NPE;
  h->vol_tot = h->lx * h->ly * h->lz;
  h->ivol = 1.0 / (h->wg * NPE);
  h->evol = h->dx * h->dy * h->dz;
  h->micro_type = c->micro_type;
  h->nvars = h->nelem * NPE * NVAR_GP;
  memcpy(h->geo_params, c->geo_params, sizeof(h->geo_params));
  for (int i = 0; i < 3; ++i) h->mats[i] = c->materials[i];
  h->nr_max_its = c->nr_max_its;
  h->nr_max_tol = c->nr_max_tol;
  h->nr_rel_tol = c->nr_rel_tol;
  h->cg_max_its = c->cg_max_its;
  h->cg_abs_tol = c->cg_abs_tol;
  h->cg_rel_tol = c->cg_rel_tol;
  h->lin_stress = c->lin_stress;
  h->subiterations = c->subiterations;
  h->nsubiterations = c->nsubiterations;

  for (int gp = 0; gp < NPE; ++gp) orc_calc_bmat(h->dx, h->dy, h->dz, gp, h->bmat[gp]);

  h->gp = (orc_gp *)calloc(h->ngp, sizeof(orc_gp));
  int n_fe = 0;
  for (int i = 0; i < h->ngp; ++i) {
    orc_gp *g = &h->gp[i];
    g->coupling = c->coupling ? c->coupling[i] : FE_ONE_WAY;
    g->converged = 1;
    if (!c->coupling || g->coupling == FE_ONE_WAY || g->coupling == FE_FULL) {
      g->u_n = (double *)calloc(h->nndim, sizeof(double));
      g->u_k = (double *)calloc(h->nndim, sizeof(double));
    }
    if (g->coupling == FE_LINEAR || g->coupling == FE_ONE_WAY || g->coupling == FE_FULL) n_fe++;
  }

  h->elem_type = (int *)calloc(h->nelem, sizeof(int));
  for (int ez = 0; ez < h->nez; ++ez)
    for (int ey = 0; ey < h->ney; ++ey)
      for (int ex = 0; ex < h->nex; ++ex) {
        const int e = (ez * h->ney + ey) * h->nex + ex;
        h->elem_type[e] = c->elem_type ? c->elem_type[e] : elem_type_of(h, ex, ey, ez);
      }

  /* calc_volume_fractions (micropp.cpp:609-627) */
  h->Vm = h->Vf = 0.0;
  for (int e = 0; e < h->nelem; ++e) {
    if (h->elem_type[e] == 0)
      h->Vm += h->evol;
    else if (h->elem_type[e] >= 1)
      h->Vf += h->evol;
  }
  h->Vm /= h->vol_tot;
  h->Vf /= h->vol_tot;

  /* A0 (micropp.cpp:128-143), before the linear ctan whose solves use it */
  h->use_A0 = c->use_A0;
  h->its_with_A0 = c->its_with_A0;
  if (h->use_A0) {
#ifdef _OPENMP
    h->nA0 = omp_get_max_threads();
#else
    h->nA0 = 1;
#endif
    h->A0 = (orc_ell *)calloc(h->nA0, sizeof(orc_ell));
    const int ns[3] = {h->nx, h->ny, h->nz};
    double *u0 = (double *)calloc(h->nndim, sizeof(double));
    for (int i = 0; i < h->nA0; ++i) {
      ell_init(&h->A0[i], ns, h->cg_abs_tol, h->cg_rel_tol, h->cg_max_its);
      assembly_mat(h, &h->A0[i], u0, NULL);
    }
    free(u0);
  }

  memset(h->ctan_lin, 0, sizeof(h->ctan_lin));
  if (c->calc_ctan_lin && n_fe > 0) calc_ctan_lin_fe(h);

  for (int i = 0; i < h->ngp; ++i) {
    orc_gp *g = &h->gp[i];
    if (g->coupling == FE_LINEAR || g->coupling == FE_ONE_WAY || g->coupling == FE_FULL)
      memcpy(g->ctan, h->ctan_lin, sizeof(g->ctan));
    else if (g->coupling == MIX_RULE_CHAMIS)
      ctan_mix_rule_chamis(h, g->ctan);
  }
  return h;
}

void orc_free(orc_rve *h) {
  if (!h) return;
  for (int i = 0; i < h->ngp; ++i) {
    free(h->gp[i].u_n);
    free(h->gp[i].u_k);
    if (h->gp[i].allocated) {
      free(h->gp[i].vars_n);
      free(h->gp[i].vars_k);
    }
  }
  free(h->gp);
  free(h->elem_type);
  for (int i = 0; i < h->nA0; ++i) ell_free(&h->A0[i]);
  free(h->A0);
  free(h);
}

void orc_set_strain(orc_rve *h, int gp, const double *strain) { memcpy(h->gp[gp].strain, strain, 6 * sizeof(double)); }
void orc_get_stress(const orc_rve *h, int gp, double *stress) { memcpy(stress, h->gp[gp].stress, 6 * sizeof(double)); }
void orc_get_ctan(const orc_rve *h, int gp, double *ctan) { memcpy(ctan, h->gp[gp].ctan, 36 * sizeof(double)); }

/* homogenize (homogenize.cpp:68-99): OpenMP over Gauss points, as in the reference. */
void orc_homogenize(orc_rve *h) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < h->ngp; ++i) {
    orc_gp *g = &h->gp[i];
    if (g->coupling == FE_LINEAR || g->coupling == MIX_RULE_CHAMIS)
      homogenize_linear_gp(g);
    else if (g->coupling == FE_ONE_WAY)
      homogenize_fe(h, g, 0);
    else if (g->coupling == FE_FULL)
      homogenize_fe(h, g, 1);
  }
}

void orc_homogenize_linear(orc_rve *h) {
  for (int i = 0; i < h->ngp; ++i) homogenize_linear_gp(&h->gp[i]);
}

/* update_vars (homogenize.cpp:284-287, gp.hpp:95-105). */
void orc_update_vars(orc_rve *h) {
  for (int i = 0; i < h->ngp; ++i) {
    orc_gp *g = &h->gp[i];
    double *t = g->vars_n;
    g->vars_n = g->vars_k;
    g->vars_k = t;
    t = g->u_n;
    g->u_n = g->u_k;
    g->u_k = t;
    memcpy(g->strain_old, g->strain, sizeof(g->strain));
  }
}

int orc_is_non_linear(const orc_rve *h, int gp) { return h->gp[gp].allocated; }
int orc_get_non_linear_gps(const orc_rve *h) {
  int c = 0;
  for (int i = 0; i < h->ngp; ++i) c += h->gp[i].allocated ? 1 : 0;
  return c;
}
long orc_get_cost(const orc_rve *h, int gp) { return h->gp[gp].cost; }
int orc_has_converged(const orc_rve *h, int gp) { return h->gp[gp].converged; }
int orc_has_subiterated(const orc_rve *h, int gp) { return h->gp[gp].subiterated; }
int orc_nelem(const orc_rve *h) { return h->nelem; }
int orc_nndim(const orc_rve *h) { return h->nndim; }
void orc_get_elem_type(const orc_rve *h, int *out) { memcpy(out, h->elem_type, h->nelem * sizeof(int)); }
void orc_get_ctan_lin(const orc_rve *h, double *out) { memcpy(out, h->ctan_lin, 36 * sizeof(double)); }
void orc_get_vol_fractions(const orc_rve *h, double *out) {
  out[0] = h->Vm;
  out[1] = h->Vf;
}
void orc_get_vars(const orc_rve *h, int gp, int which, double *out) {
  const orc_gp *g = &h->gp[gp];
  const double *src = g->allocated ? (which ? g->vars_k : g->vars_n) : NULL;
  if (src)
    memcpy(out, src, h->nvars * sizeof(double));
  else
    memset(out, 0, h->nvars * sizeof(double));
}
void orc_get_u(const orc_rve *h, int gp, int which, double *out) {
  const orc_gp *g = &h->gp[gp];
  const double *src = which ? g->u_k : g->u_n;
  if (src)
    memcpy(out, src, h->nndim * sizeof(double));
  else
    memset(out, 0, h->nndim * sizeof(double));
}
void orc_get_ops(const orc_rve *h, int gp, double *count, double *sec) {
  memcpy(count, h->gp[gp].op_count, sizeof(h->gp[gp].op_count));
  memcpy(sec, h->gp[gp].op_sec, sizeof(h->gp[gp].op_sec));
}
void orc_reset_ops(orc_rve *h) {
  for (int i = 0; i < h->ngp; ++i) {
    memset(h->gp[i].op_count, 0, sizeof(h->gp[i].op_count));
    memset(h->gp[i].op_sec, 0, sizeof(h->gp[i].op_sec));
  }
}
void orc_get_newton(const orc_rve *h, int gp, int *its, int *sits, int *conv) {
  *its = h->gp[gp].nr_its;
  *sits = h->gp[gp].nr_solver_its;
  *conv = h->gp[gp].nr_converged;
}

/* gp_t::write_restart / read_restart (gp.hpp:107-124): per GP a one-byte `allocated`, then vars_n and u_n
 * when allocated. */
int orc_write_restart(const orc_rve *h, const char *path) {
  FILE *f = fopen(path, "wb");
  if (!f) return 1;
  for (int i = 0; i < h->ngp; ++i) {
    const orc_gp *g = &h->gp[i];
    const unsigned char a = g->allocated ? 1 : 0;
    fwrite(&a, 1, 1, f);
    if (a) {
      fwrite(g->vars_n, sizeof(double), h->nvars, f);
      fwrite(g->u_n, sizeof(double), h->nndim, f);
    }
  }
  fclose(f);
  return 0;
}

int orc_read_restart(orc_rve *h, const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) return 1;
  for (int i = 0; i < h->ngp; ++i) {
    orc_gp *g = &h->gp[i];
    unsigned char a = 0;
    if (fread(&a, 1, 1, f) != 1) break;
    if (a) {
      if (!g->allocated) gp_allocate(h, g);
      if (fread(g->vars_n, sizeof(double), h->nvars, f) != (size_t)h->nvars) break;
      if (fread(g->u_n, sizeof(double), h->nndim, f) != (size_t)h->nndim) break;
    } else if (g->allocated) {
      free(g->vars_n);
      free(g->vars_k);
      g->vars_n = g->vars_k = NULL;
      g->allocated = 0;
    }
  }
  fclose(f);
  return 0;
}
