/*
 * ref_driver.cpp -- C entry points over the compiled reference CPU library (oracle/_ref).
 *
 * TEST INFRASTRUCTURE ONLY.  Linked against the object files that oracle/build_ref.sh compiles from the
 * reference's own sources; used here to pin the C restatement (micropp_oracle.c) and to generate the
 * golden fixtures under tests/golden/.  The reference headers come from the reference tree at build time.
 *
 * `ref_rve` subclasses micropp<3> (micropp.hpp:54-218) only to reach protected state: an element-phase
 * override (micropp.hpp:82, recomputing calc_volume_fractions and calc_ctan_lin_fe_models as the
 * constructor does, micropp.cpp:117-165) and read access to gp_list for internal variables and
 * displacements.
 */
#include <cstring>

#include "micropp.hpp"
#include "micropp_oracle.h"

class ref_rve : public micropp<3> {
 public:
  ref_rve(const micropp_params_t &p, const int *et, bool want_lin) : micropp<3>(p) {
    if (et) {
      memcpy(elem_type, et, nelem * sizeof(int));
      calc_volume_fractions();
    }
    if (want_lin && !p.calc_ctan_lin) {
      calc_ctan_lin_fe_models();
      for (int gp = 0; gp < ngp; ++gp) {
        const int c = gp_list[gp].coupling;
        if (c == FE_LINEAR || c == FE_ONE_WAY || c == FE_FULL) memcpy(gp_list[gp].ctan, ctan_lin_fe, sizeof(ctan_lin_fe));
      }
    }
  }
  int n_elem() const { return nelem; }
  int n_dim() const { return nndim; }
  void elem_types(int *out) const { memcpy(out, elem_type, nelem * sizeof(int)); }
  void ctan_lin(double *out) const { memcpy(out, ctan_lin_fe, sizeof(ctan_lin_fe)); }
  void vol_fr(double *out) const {
    out[0] = Vm;
    out[1] = Vf;
  }
  void vars(int gp, int which, double *out) const {
    const gp_t<3> &g = gp_list[gp];
    const double *src = g.allocated ? (which ? g.vars_k : g.vars_n) : nullptr;
    if (src)
      memcpy(out, src, nvars * sizeof(double));
    else
      memset(out, 0, nvars * sizeof(double));
  }
  void u(int gp, int which, double *out) const {
    const gp_t<3> &g = gp_list[gp];
    const double *src = which ? g.u_k : g.u_n;
    if (src)
      memcpy(out, src, nndim * sizeof(double));
    else
      memset(out, 0, nndim * sizeof(double));
  }
};

extern "C" {

void *ref_new(const struct orc_config *c) {
  micropp_params_t p;
  p.ngp = c->ngp;
  memcpy(p.size, c->size, sizeof(p.size));
  p.type = c->micro_type;
  memcpy(p.geo_params, c->geo_params, sizeof(p.geo_params));
  for (int i = 0; i < 3; ++i) memcpy(&p.materials[i], &c->materials[i], sizeof(struct material_base));
  p.coupling = const_cast<int *>(c->coupling);
  p.subiterations = c->subiterations != 0;
  p.nsubiterations = c->nsubiterations;
  p.mpi_rank = c->mpi_rank;
  p.nr_max_its = c->nr_max_its;
  p.nr_max_tol = c->nr_max_tol;
  p.nr_rel_tol = c->nr_rel_tol;
  p.cg_max_its = c->cg_max_its;
  p.cg_abs_tol = c->cg_abs_tol;
  p.cg_rel_tol = c->cg_rel_tol;
  /* With a phase override the linear ctan is computed once, after the override. */
  p.calc_ctan_lin = c->elem_type ? false : (c->calc_ctan_lin != 0);
  p.use_A0 = c->use_A0 != 0;
  p.its_with_A0 = c->its_with_A0;
  p.lin_stress = c->lin_stress != 0;
  p.write_log = false;
  return new ref_rve(p, c->elem_type, c->elem_type && c->calc_ctan_lin);
}

void ref_free(void *h) { delete (ref_rve *)h; }
void ref_set_strain(void *h, int gp, const double *e) { ((ref_rve *)h)->set_strain(gp, e); }
void ref_get_stress(void *h, int gp, double *s) { ((ref_rve *)h)->get_stress(gp, s); }
void ref_get_ctan(void *h, int gp, double *c) { ((ref_rve *)h)->get_ctan(gp, c); }
void ref_homogenize(void *h) { ((ref_rve *)h)->homogenize(); }
void ref_homogenize_linear(void *h) { ((ref_rve *)h)->homogenize_linear(); }
void ref_update_vars(void *h) { ((ref_rve *)h)->update_vars(); }
int ref_is_non_linear(void *h, int gp) { return ((ref_rve *)h)->is_non_linear(gp); }
int ref_get_non_linear_gps(void *h) { return ((ref_rve *)h)->get_non_linear_gps(); }
long ref_get_cost(void *h, int gp) { return ((ref_rve *)h)->get_cost(gp); }
int ref_has_converged(void *h, int gp) { return ((ref_rve *)h)->has_converged(gp) ? 1 : 0; }
int ref_has_subiterated(void *h, int gp) { return ((ref_rve *)h)->has_subiterated(gp) ? 1 : 0; }
int ref_nelem(void *h) { return ((ref_rve *)h)->n_elem(); }
int ref_nndim(void *h) { return ((ref_rve *)h)->n_dim(); }
void ref_get_elem_type(void *h, int *out) { ((ref_rve *)h)->elem_types(out); }
void ref_get_ctan_lin(void *h, double *out) { ((ref_rve *)h)->ctan_lin(out); }
void ref_get_vol_fractions(void *h, double *out) { ((ref_rve *)h)->vol_fr(out); }
void ref_get_vars(void *h, int gp, int which, double *out) { ((ref_rve *)h)->vars(gp, which, out); }
void ref_get_u(void *h, int gp, int which, double *out) { ((ref_rve *)h)->u(gp, which, out); }
void ref_write_restart(void *h, int id) { ((ref_rve *)h)->write_restart(id); }
void ref_read_restart(void *h, int id) { ((ref_rve *)h)->read_restart(id); }
void ref_output(void *h, int gp, const char *filename) { ((ref_rve *)h)->output(gp, filename); }
}
