/*
 * micropp.hpp -- the micropp<3> C++ API, served by the GB300 library (libmicropp_gb300.so).
 *
 * Drop-in for the public part of the reference's include/micropp.hpp:54-218 and the parameter record of
 * include/types.hpp:43-83: same class name and template, same constructor parameters with the same
 * defaults, same member functions with the same meaning.  Three fields are appended to micropp_params_t
 * (elem_type, precision, ctan_mode); code written for the reference compiles unchanged.  Only tdim = 3 is
 * provided, as in the reference (which instantiates micropp<3> only).
 */
#pragma once

#include "material_base.h"
#include "micropp_gb300.h"

/* Micro-structure types (types.hpp:85-99). */
enum {
  MIC_HOMOGENEOUS,
  MIC_SPHERE,
  MIC_LAYER_Y,
  MIC_CILI_FIB_X,
  MIC_CILI_FIB_Z,
  MIC_CILI_FIB_XZ,
  MIC_QUAD_FIB_XYZ,
  MIC_QUAD_FIB_XZ,
  MIC_QUAD_FIB_XZ_BROKEN_X,
  MIC3D_SPHERES,
  MIC3D_8,
  MIC3D_FIBS_20_ORDER,
  MIC3D_FIBS_20_DISORDER
};

/* Coupling of a macro Gauss point (types.hpp:110). */
enum { FE_LINEAR, FE_ONE_WAY, FE_FULL, MIX_RULE_CHAMIS };

/* Construction parameters (types.hpp:43-83) with the reference's defaults (params.hpp:32-35, ell.hpp:33-35). */
struct micropp_params_t {
  int ngp = 1;
  int size[3];
  int type = 0;
  double geo_params[4] = {0.1, 0.1, 0.1, 0.1};
  struct material_base materials[4];
  int *coupling = nullptr;
  bool subiterations = false;
  int nsubiterations = 10;
  int mpi_rank = 0;
  int nr_max_its = 4;
  double nr_max_tol = 1.0e-10;
  double nr_rel_tol = 1.0e-3;
  int cg_max_its = 1000;
  double cg_abs_tol = 1.0e-50;
  double cg_rel_tol = 1.0e-5;
  bool calc_ctan_lin = true;
  bool use_A0 = false;
  int its_with_A0 = 1;
  bool lin_stress = true;
  bool write_log = false;
  /* GB300 additions */
  const int *elem_type = nullptr; /* optional element phase map, nelem entries */
  int precision = MICROPP3_FP64;
  int ctan_mode = MICROPP3_CTAN_PERTURB;

  void print() const;
};

template <int tdim>
class micropp;

template <>
class micropp<3> {
 public:
  micropp() = delete;
  micropp(const micropp_params_t &params);
  ~micropp();
  micropp(const micropp &) = delete;
  micropp &operator=(const micropp &) = delete;

  void set_strain(const int gp_id, const double *strain);
  void get_stress(const int gp_id, double *stress) const;
  void get_ctan(const int gp_id, double *ctan) const;
  void homogenize();
  void homogenize_linear();

  int is_non_linear(const int gp_id) const;
  int get_non_linear_gps(void) const;
  int get_cost(int gp_id) const;
  bool has_converged(int gp_id) const;
  bool has_subiterated(int gp_id) const;
  void output(int gp_id, const char *filename);
  void output2(const int gp_id, const int elem_global, const int time_step);
  void update_vars();
  void write_restart(const int restart_id) const;
  void read_restart(const int restart_id) const;
  void print_info() const;

  /* The C handle behind this object (for the micropp3_* extension entry points). */
  struct micropp3 *c_handle() { return &handle_; }

 private:
  struct micropp3 handle_;
};
