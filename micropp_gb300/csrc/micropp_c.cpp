// micropp_c.cpp -- the micropp3 C ABI (include/micropp_c.h, include/micropp_gb300.h) over the Engine.
//
// Each entry forwards to the handle's Engine like the reference wrapper (micropp_c.cpp:29-142).  Failures
// (a bad argument, a CUDA error) cannot surface through the reference's void signatures, so they are
// printed on stderr and kept for micropp3_last_error(); a failed micropp3_new leaves self->ptr NULL.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include "engine.hpp"
#include "micropp_c.h"
#include "micropp_gb300.h"

using mgb::Engine;

namespace {

thread_local std::string g_last_error;

void fail(const char *where, const char *what) {
  g_last_error = std::string(where) + ": " + what;
  std::fprintf(stderr, "micropp3 error: %s\n", g_last_error.c_str());
}

template <typename F>
void guard(const char *where, F f) {
  try {
    f();
  } catch (const std::exception &e) {
    fail(where, e.what());
  }
}

Engine *eng(const micropp3 *self, const char *where) {
  if (!self || !self->ptr) {
    fail(where, "invalid handle (construction failed or the handle was freed)");
    return nullptr;
  }
  return (Engine *)self->ptr;
}

}  // namespace

extern "C" {

void micropp3_config_default(struct micropp3_config *c) {
  std::memset(c, 0, sizeof(*c));
  c->ngp = 1;
  for (double &g : c->geo_params) g = 0.1;
  c->coupling = nullptr;
  c->subiterations = 0;
  c->nsubiterations = 10;
  c->mpi_rank = 0;
  c->nr_max_its = 4;
  c->nr_max_tol = 1.0e-10;
  c->nr_rel_tol = 1.0e-3;
  c->cg_max_its = 1000;
  c->cg_abs_tol = 1.0e-50;
  c->cg_rel_tol = 1.0e-5;
  c->calc_ctan_lin = 1;
  c->use_A0 = 0;
  c->its_with_A0 = 1;
  c->lin_stress = 1;
  c->write_log = 0;
  c->elem_type = nullptr;
  c->precision = MICROPP3_FP64;
  c->ctan_mode = MICROPP3_CTAN_PERTURB;
}

const char *micropp3_last_error(void) { return g_last_error.c_str(); }

void micropp3_clear_error(void) { g_last_error.clear(); }

void micropp3_new_ext(struct micropp3 *self, const struct micropp3_config *cfg) {
  if (!self) return;
  self->ptr = nullptr;
  g_last_error.clear();
  if (!cfg) {
    fail("micropp3_new_ext", "NULL configuration");
    return;
  }
  guard("micropp3_new_ext", [&] { self->ptr = new Engine(*cfg); });
}

void micropp3_new(struct micropp3 *self, int ngp, const int size[3], const int micro_type, const double *micro_params,
                  const struct material_base *materials, const int *coupling, const int nsubiterations,
                  const int mpi_rank) {
  if (!self) return;
  micropp3_config c;
  micropp3_config_default(&c);
  c.ngp = ngp;
  std::memcpy(c.size, size, 3 * sizeof(int));
  c.micro_type = micro_type;
  std::memcpy(c.geo_params, micro_params, 4 * sizeof(double));
  for (int i = 0; i < 3; ++i) c.materials[i] = materials[i];
  c.coupling = coupling;
  c.subiterations = 1;  // forced on by the reference wrapper (micropp_c.cpp:46)
  c.nsubiterations = nsubiterations;
  c.mpi_rank = mpi_rank;
  c.use_A0 = 0;
  c.its_with_A0 = 1;
  c.write_log = 0;
  micropp3_new_ext(self, &c);
}

void micropp3_free(struct micropp3 *self) {
  if (!self || !self->ptr) return;
  guard("micropp3_free", [&] { delete (Engine *)self->ptr; });
  self->ptr = nullptr;
}

void micropp3_set_strain(struct micropp3 *self, const int gp_id, const double *strain) {
  if (Engine *e = eng(self, "micropp3_set_strain")) guard("micropp3_set_strain", [&] { e->set_strain(gp_id, strain); });
}

void micropp3_get_stress(const struct micropp3 *self, const int gp_id, double *stress) {
  if (Engine *e = eng(self, "micropp3_get_stress")) guard("micropp3_get_stress", [&] { e->get_stress(gp_id, stress); });
}

void micropp3_get_ctan(const struct micropp3 *self, const int gp_id, double *ctan) {
  if (Engine *e = eng(self, "micropp3_get_ctan")) guard("micropp3_get_ctan", [&] { e->get_ctan(gp_id, ctan); });
}

void micropp3_homogenize(struct micropp3 *self) {
  if (Engine *e = eng(self, "micropp3_homogenize")) guard("micropp3_homogenize", [&] { e->homogenize(); });
}

void micropp3_homogenize_linear(struct micropp3 *self) {
  if (Engine *e = eng(self, "micropp3_homogenize_linear"))
    guard("micropp3_homogenize_linear", [&] { e->homogenize_linear(); });
}

void micropp3_update_vars(struct micropp3 *self) {
  if (Engine *e = eng(self, "micropp3_update_vars")) guard("micropp3_update_vars", [&] { e->update_vars(); });
}

bool micropp3_is_non_linear(const struct micropp3 *self, const int gp_id) {
  bool r = false;
  if (Engine *e = eng(self, "micropp3_is_non_linear"))
    guard("micropp3_is_non_linear", [&] { r = e->is_non_linear(gp_id) != 0; });
  return r;
}

int micropp3_get_cost(const struct micropp3 *self, int gp_id) {
  int r = 0;
  if (Engine *e = eng(self, "micropp3_get_cost")) guard("micropp3_get_cost", [&] { r = (int)e->get_cost(gp_id); });
  return r;
}

bool micropp3_has_converged(const struct micropp3 *self, int gp_id) {
  bool r = false;
  if (Engine *e = eng(self, "micropp3_has_converged"))
    guard("micropp3_has_converged", [&] { r = e->has_converged(gp_id); });
  return r;
}

bool micropp3_has_subiterated(const struct micropp3 *self, int gp_id) {
  bool r = false;
  if (Engine *e = eng(self, "micropp3_has_subiterated"))
    guard("micropp3_has_subiterated", [&] { r = e->has_subiterated(gp_id); });
  return r;
}

void micropp3_output(struct micropp3 *self, const int gp_id, const char *filename) {
  if (Engine *e = eng(self, "micropp3_output")) guard("micropp3_output", [&] { e->output_vtu(gp_id, filename); });
}

void micropp3_output2(struct micropp3 *self, const int gp_id, const int elem_global, const int time_step) {
  if (Engine *e = eng(self, "micropp3_output2"))
    guard("micropp3_output2", [&] {
      const std::string name = "micropp-" + std::to_string(elem_global) + "-" + std::to_string(time_step);
      e->output_vtu(gp_id, name.c_str());
    });
}

void micropp3_print_info(struct micropp3 *self) {
  if (Engine *e = eng(self, "micropp3_print_info")) guard("micropp3_print_info", [&] { e->print_info(); });
}

int micropp3_get_non_linear_gps(const struct micropp3 *self) {
  int r = 0;
  if (Engine *e = eng(self, "micropp3_get_non_linear_gps"))
    guard("micropp3_get_non_linear_gps", [&] { r = e->get_non_linear_gps(); });
  return r;
}

void micropp3_write_restart(const struct micropp3 *self, const int restart_id) {
  if (Engine *e = eng(self, "micropp3_write_restart"))
    guard("micropp3_write_restart", [&] { e->write_restart(restart_id); });
}

void micropp3_read_restart(const struct micropp3 *self, const int restart_id) {
  if (Engine *e = eng(self, "micropp3_read_restart"))
    guard("micropp3_read_restart", [&] { e->read_restart(restart_id); });
}

// ---- extensions -------------------------------------------------------------------------------------

int micropp3_path_forward(struct micropp3 *self, int nsteps, const double *strains, const double *params,
                          int checkpoint_every, double *sigma) {
  int rc = -2;
  if (Engine *e = eng(self, "micropp3_path_forward"))
    guard("micropp3_path_forward", [&] { rc = e->path_forward(nsteps, strains, params, checkpoint_every, sigma); });
  return rc;
}

int micropp3_path_vjp(struct micropp3 *self, const double *gsigma, double *grad_params, double *grad_strains) {
  int rc = -2;
  if (Engine *e = eng(self, "micropp3_path_vjp"))
    guard("micropp3_path_vjp", [&] { rc = e->path_vjp(gsigma, grad_params, grad_strains); });
  return rc;
}

void micropp3_path_newton(const struct micropp3 *self, int step, int *its, int *cg_its, int *status,
                          double *rel_norm) {
  if (Engine *e = eng(self, "micropp3_path_newton"))
    guard("micropp3_path_newton", [&] { e->path_newton(step, its, cg_its, status, rel_norm); });
}

void micropp3_set_cuda_graphs(struct micropp3 *self, int enable) {
  if (Engine *e = eng(self, "micropp3_set_cuda_graphs")) guard("micropp3_set_cuda_graphs", [&] { e->set_graphs(enable != 0); });
}

void micropp3_homogenize_many(struct micropp3 *const *handles, int n) {
  if (n <= 0) return;
  if (!handles) {
    fail("micropp3_homogenize_many", "handles is NULL");
    return;
  }
  std::vector<Engine *> engines(n);
  for (int i = 0; i < n; ++i)
    if (!(engines[i] = eng(handles[i], "micropp3_homogenize_many"))) return;
  // Every handle has its own stream: homogenize them from worker threads so that their batches (RVEs of
  // different sizes or materials) run on the GPU at the same time.
  std::vector<std::string> errors(n);
  std::atomic<int> next(0);
  auto work = [&] {
    for (int i; (i = next.fetch_add(1)) < n;) {
      try {
        engines[i]->homogenize();
      } catch (const std::exception &e) {
        errors[i] = e.what();
      }
    }
  };
  const int nthreads = std::min(n, 16);
  std::vector<std::thread> pool;
  for (int t = 1; t < nthreads; ++t) pool.emplace_back(work);
  work();
  for (auto &t : pool) t.join();
  for (int i = 0; i < n; ++i)
    if (!errors[i].empty()) fail("micropp3_homogenize_many", ("handle " + std::to_string(i) + ": " + errors[i]).c_str());
}

int micropp3_get_status(const struct micropp3 *self, int gp_id) {
  int r = 0;
  if (Engine *e = eng(self, "micropp3_get_status")) guard("micropp3_get_status", [&] { r = e->get_status(gp_id); });
  return r;
}

void micropp3_get_newton(const struct micropp3 *self, int gp_id, int *its, int *solver_its, int *converged) {
  if (Engine *e = eng(self, "micropp3_get_newton"))
    guard("micropp3_get_newton", [&] { e->get_newton(gp_id, its, solver_its, converged); });
}

int micropp3_get_nelem(const struct micropp3 *self) {
  Engine *e = eng(self, "micropp3_get_nelem");
  return e ? e->nelem() : 0;
}

int micropp3_get_nndim(const struct micropp3 *self) {
  Engine *e = eng(self, "micropp3_get_nndim");
  return e ? e->nndim() : 0;
}

void micropp3_get_vars(const struct micropp3 *self, int gp_id, int which, double *out) {
  if (Engine *e = eng(self, "micropp3_get_vars")) guard("micropp3_get_vars", [&] { e->get_vars(gp_id, which, out); });
}

void micropp3_get_u(const struct micropp3 *self, int gp_id, int which, double *out) {
  if (Engine *e = eng(self, "micropp3_get_u")) guard("micropp3_get_u", [&] { e->get_u(gp_id, which, out); });
}

void micropp3_get_elem_type(const struct micropp3 *self, int *out) {
  if (Engine *e = eng(self, "micropp3_get_elem_type")) guard("micropp3_get_elem_type", [&] { e->get_elem_type(out); });
}

void micropp3_get_ctan_lin(const struct micropp3 *self, double *out36) {
  if (Engine *e = eng(self, "micropp3_get_ctan_lin")) guard("micropp3_get_ctan_lin", [&] { e->get_ctan_lin(out36); });
}

int micropp3_get_mg_levels(const struct micropp3 *self) {
  Engine *e = eng(self, "micropp3_get_mg_levels");
  return e ? e->mg_levels() : 0;
}

double micropp3_last_homogenize_ms(const struct micropp3 *self) {
  Engine *e = eng(self, "micropp3_last_homogenize_ms");
  return e ? e->last_homogenize_ms() : 0.0;
}

void micropp3_set_kernel_timing(struct micropp3 *self, int enable) {
  if (Engine *e = eng(self, "micropp3_set_kernel_timing"))
    guard("micropp3_set_kernel_timing", [&] { e->set_kernel_timing(enable != 0); });
}

int micropp3_kernel_stats(const struct micropp3 *self, const char *family, long *launches, double *ms, double *bytes) {
  int ok = 0;
  if (Engine *e = eng(self, "micropp3_kernel_stats"))
    guard("micropp3_kernel_stats", [&] { ok = e->kernel_stats(family ? family : "", launches, ms, bytes) ? 1 : 0; });
  return ok;
}

long micropp3_kernel_launches(const struct micropp3 *self) {
  Engine *e = eng(self, "micropp3_kernel_launches");
  return e ? e->kernel_launches() : 0;
}

long micropp3_total_cg_its(const struct micropp3 *self) {
  Engine *e = eng(self, "micropp3_total_cg_its");
  return e ? e->total_cg_its() : 0;
}

}  // extern "C"
