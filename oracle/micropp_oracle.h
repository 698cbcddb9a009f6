/*
 * micropp_oracle.h -- CPU restatement of Micropp's RVE homogenization path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the GPU library is checked against: only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it.  The product library
 * (micropp_gb300) never links, loads or calls it.
 *
 * It restates, in plain C and in the same floating-point operation order, the reference's CPU path
 * (gagiuntoli/Micropp, src/{micropp,homogenize,solve,assembly,ell,ell-common,material,average,update,
 * micro3D,common}.cpp).  Each function cites the file:line it follows.  It is pinned against the
 * compiled reference (oracle/build_ref.sh + oracle/ref_driver.cpp) and the reference's own golden tables
 * (test/benchmark-{elastic,plastic,damage}.cpp) by tests/test_oracle_pin.py.
 */
#ifndef MICROPP_ORACLE_H
#define MICROPP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Same layout as `struct material_base` (include/material_base.h in the reference, material_base.h:40-45). */
struct orc_material {
  double E, nu, Ka, Sy;
  double k, mu, lambda;
  double Xt;
  int type;
};

/* Construction parameters.  Field meaning and defaults follow micropp_params_t (types.hpp:43-63); the
 * layout is identical to `struct micropp3_config` of the product (include/micropp_gb300.h) so one ctypes
 * structure drives both. */
struct orc_config {
  int ngp;
  int size[3];
  int micro_type;
  double geo_params[4];
  struct orc_material materials[3];
  const int *coupling;   /* ngp entries or NULL (=> FE_ONE_WAY for every GP, micropp.cpp:88-96) */
  int subiterations;
  int nsubiterations;
  int mpi_rank;
  int nr_max_its;
  double nr_max_tol;
  double nr_rel_tol;
  int cg_max_its;
  double cg_abs_tol;
  double cg_rel_tol;
  int calc_ctan_lin;
  int use_A0;
  int its_with_A0;
  int lin_stress;
  int write_log;
  const int *elem_type;  /* optional override of the element phase map (nelem entries) */
  int precision;         /* ignored by the oracle (always FP64) */
  int ctan_mode;         /* ignored by the oracle (always the reference's 6 perturbed solves) */
  int reserved[4];
};

typedef struct orc_rve orc_rve;

void orc_config_default(struct orc_config *cfg);
void orc_material_set(struct orc_material *m, int type, double E, double nu, double Ka, double Sy, double Xt);

orc_rve *orc_new(const struct orc_config *cfg);
void orc_free(orc_rve *h);

void orc_set_strain(orc_rve *h, int gp, const double *strain);
void orc_get_stress(const orc_rve *h, int gp, double *stress);
void orc_get_ctan(const orc_rve *h, int gp, double *ctan);
void orc_homogenize(orc_rve *h);
void orc_homogenize_linear(orc_rve *h);
void orc_update_vars(orc_rve *h);
int orc_is_non_linear(const orc_rve *h, int gp);
int orc_get_non_linear_gps(const orc_rve *h);
long orc_get_cost(const orc_rve *h, int gp);
int orc_has_converged(const orc_rve *h, int gp);
int orc_has_subiterated(const orc_rve *h, int gp);

/* Inspection (test only). */
int orc_nelem(const orc_rve *h);
int orc_nndim(const orc_rve *h);
void orc_get_elem_type(const orc_rve *h, int *out);
void orc_get_ctan_lin(const orc_rve *h, double *out36);
void orc_get_vol_fractions(const orc_rve *h, double *vm_vf);
/* which = 0: vars_n, 1: vars_k (nelem*8*7 doubles; zeros when not allocated). */
void orc_get_vars(const orc_rve *h, int gp, int which, double *out);
/* which = 0: u_n, 1: u_k (nndim doubles). */
void orc_get_u(const orc_rve *h, int gp, int which, double *out);
/* Newton statistics of the most recent main solve of `gp`: its, solver_its, converged. */
void orc_get_newton(const orc_rve *h, int gp, int *its, int *solver_its, int *converged);
/* Operation counts and host seconds of every FE homogenization of `gp` since construction or the last
 * orc_reset_ops, indexed by ORC_OP_*: residual assemblies (assembly_rhs), Jacobian assemblies (assembly_mat),
 * CG set-ups (one per solve), CG iterations, average stresses, internal-variable updates, and whole
 * homogenize_fe calls (whose seconds include everything, also allocation and copies).  Instrumentation for
 * the CPU baseline's cost model; no result depends on it. */
enum { ORC_OP_RESIDUAL, ORC_OP_ASSEMBLY, ORC_OP_CG_SETUP, ORC_OP_CG_ITER, ORC_OP_AVE_STRESS, ORC_OP_VARS,
       ORC_OP_HOMOGENIZE, ORC_NOPS };
void orc_get_ops(const orc_rve *h, int gp, double *count, double *sec);
void orc_reset_ops(orc_rve *h);
/* Restart files in the reference's binary format (gp.hpp:107-124, output.cpp:216-262). */
int orc_write_restart(const orc_rve *h, const char *path);
int orc_read_restart(orc_rve *h, const char *path);

/* Low-level pieces exposed for unit tests. */
void orc_calc_bmat(double dx, double dy, double dz, int gp, double bmat[6][24]);

#ifdef __cplusplus
}
#endif
#endif
