// micropp.cpp -- the micropp<3> C++ class (include/micropp.hpp) over the C ABI of the GB300 library.
//
// The class is a thin owner of a micropp3 handle: every member function is the C entry of the same name.
// Unlike the C ABI, a failure here throws std::runtime_error, the C++ way of the reference's asserts.
#include "micropp.hpp"

#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>

namespace {

void raise_if_failed(const char *where) {
  const char *msg = micropp3_last_error();
  if (msg && msg[0]) throw std::runtime_error(std::string(where) + ": " + msg);
}

}  // namespace

void micropp_params_t::print() const {
  std::cout << "ngp  : " << ngp << "\nsize : " << size[0] << "\ntype  : " << type << "\ngeo_params : "
            << geo_params[0] << "\nsubiterations : " << subiterations << "\nnsubiterations : " << nsubiterations
            << "\nmpi_rank : " << mpi_rank << "\nnr_max_its : " << nr_max_its << "\nnr_max_tol : " << nr_max_tol
            << "\nnr_rel_tol : " << nr_rel_tol << "\ncalc_ctan_lin : " << calc_ctan_lin << "\nuse_A0 : " << use_A0
            << "\nits_with_A0 : " << its_with_A0 << "\nlin_stress : " << lin_stress << "\nwrite_log : " << write_log
            << std::endl;
}

micropp<3>::micropp(const micropp_params_t &p) {
  micropp3_config c;
  micropp3_config_default(&c);
  c.ngp = p.ngp;
  std::memcpy(c.size, p.size, sizeof(c.size));
  c.micro_type = p.type;
  std::memcpy(c.geo_params, p.geo_params, sizeof(c.geo_params));
  for (int i = 0; i < 3; ++i) c.materials[i] = p.materials[i];
  c.coupling = p.coupling;
  c.subiterations = p.subiterations;
  c.nsubiterations = p.nsubiterations;
  c.mpi_rank = p.mpi_rank;
  c.nr_max_its = p.nr_max_its;
  c.nr_max_tol = p.nr_max_tol;
  c.nr_rel_tol = p.nr_rel_tol;
  c.cg_max_its = p.cg_max_its;
  c.cg_abs_tol = p.cg_abs_tol;
  c.cg_rel_tol = p.cg_rel_tol;
  c.calc_ctan_lin = p.calc_ctan_lin;
  c.use_A0 = p.use_A0;
  c.its_with_A0 = p.its_with_A0;
  c.lin_stress = p.lin_stress;
  c.write_log = p.write_log;
  c.elem_type = p.elem_type;
  c.precision = p.precision;
  c.ctan_mode = p.ctan_mode;
  micropp3_new_ext(&handle_, &c);
  if (!handle_.ptr) raise_if_failed("micropp<3>::micropp");
}

micropp<3>::~micropp() { micropp3_free(&handle_); }

#define MICROPP_FORWARD(call, name) \
  do {                              \
    micropp3_clear_error();         \
    call;                           \
    raise_if_failed(name);          \
  } while (0)

void micropp<3>::set_strain(const int gp, const double *strain) {
  MICROPP_FORWARD(micropp3_set_strain(&handle_, gp, strain), "set_strain");
}
void micropp<3>::get_stress(const int gp, double *stress) const {
  MICROPP_FORWARD(micropp3_get_stress(&handle_, gp, stress), "get_stress");
}
void micropp<3>::get_ctan(const int gp, double *ctan) const {
  MICROPP_FORWARD(micropp3_get_ctan(&handle_, gp, ctan), "get_ctan");
}
void micropp<3>::homogenize() { MICROPP_FORWARD(micropp3_homogenize(&handle_), "homogenize"); }
void micropp<3>::homogenize_linear() { MICROPP_FORWARD(micropp3_homogenize_linear(&handle_), "homogenize_linear"); }
int micropp<3>::is_non_linear(const int gp) const {
  int r = 0;
  MICROPP_FORWARD(r = micropp3_is_non_linear(&handle_, gp) ? 1 : 0, "is_non_linear");
  return r;
}
int micropp<3>::get_non_linear_gps(void) const {
  int r = 0;
  MICROPP_FORWARD(r = micropp3_get_non_linear_gps(&handle_), "get_non_linear_gps");
  return r;
}
int micropp<3>::get_cost(int gp) const {
  int r = 0;
  MICROPP_FORWARD(r = micropp3_get_cost(&handle_, gp), "get_cost");
  return r;
}
bool micropp<3>::has_converged(int gp) const {
  bool r = false;
  MICROPP_FORWARD(r = micropp3_has_converged(&handle_, gp), "has_converged");
  return r;
}
bool micropp<3>::has_subiterated(int gp) const {
  bool r = false;
  MICROPP_FORWARD(r = micropp3_has_subiterated(&handle_, gp), "has_subiterated");
  return r;
}
void micropp<3>::output(int gp, const char *filename) {
  MICROPP_FORWARD(micropp3_output(&handle_, gp, filename), "output");
}
void micropp<3>::output2(const int gp, const int elem_global, const int time_step) {
  MICROPP_FORWARD(micropp3_output2(&handle_, gp, elem_global, time_step), "output2");
}
void micropp<3>::update_vars() { MICROPP_FORWARD(micropp3_update_vars(&handle_), "update_vars"); }
void micropp<3>::write_restart(const int id) const {
  MICROPP_FORWARD(micropp3_write_restart(&handle_, id), "write_restart");
}
void micropp<3>::read_restart(const int id) const {
  MICROPP_FORWARD(micropp3_read_restart(&handle_, id), "read_restart");
}
void micropp<3>::print_info() const { MICROPP_FORWARD(micropp3_print_info(const_cast<micropp3 *>(&handle_)), "print_info"); }
