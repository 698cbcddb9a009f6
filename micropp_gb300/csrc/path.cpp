// path.cpp -- load paths of one RVE and their reverse-mode gradients (the adjoint pass, adjoint_kernels.cu).
//
// A path runs the FP64 Newton of the plain form from the undeformed state through nsteps macro strains, with
// the exact consistent tangent of the adjoint in place of the reference's forward differences and BiCGSTAB
// in place of CG for the corrections (the reference's J2 tangent is not symmetric), and the previous solution
// moved with the affine field of the strain increment as the start of each step's Newton,
// accepting every step (history h_n = H(u_n, h_{n-1}) at every Gauss point, the history present from the
// first step on), with per-phase parameters theta = (E, nu, Xt, Sy, Ka) that replace the handle's for the
// path only.  The forward pass keeps the state before every `every`-th step; the reverse pass recomputes each
// segment from its checkpoint and runs the adjoint steps backwards (the recomputation is bitwise identical:
// every reduction of the solver has a fixed order).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "cuda_util.hpp"
#include "engine.hpp"
#include "launch.h"

namespace mgb {

namespace {

constexpr double kAdjTol = 1.0e-14;  // BiCGSTAB: ||r|| <= max(cg_rel_tol, kAdjTol) ||b||
constexpr int kAdjMaxIts = 20000;

}  // namespace

// Slot 0 with the FP64 buffers of the plain form (a mixed-precision handle does not allocate them).
void Engine::ensure_fp64_slot0() {
  ensure_slots(1);
  Slot &w = slots_[0];
  const size_t nd = nndim();
  if (!w.r) w.r = dalloc<double>(nd, "r");
  if (!w.z) w.z = dalloc<double>(nd, "z");
  if (!w.p) w.p = dalloc<double>(nd, "p");
  if (!w.Ap) w.Ap = dalloc<double>(nd, "Ap");
  if (!w.kinv) w.kinv = dalloc<double>(nd, "kinv");
  if (!w.vals) w.vals = dalloc<double>((size_t)kEllPerNode * mesh_.np, "ELL values");
  Inst &I = h_insts_[0];
  I.r = w.r; I.z = w.z; I.p = w.p; I.Ap = w.Ap; I.kinv = w.kinv; I.vals = w.vals;
}

void Engine::path_free() {
  PathState &P = path_;
  for (double *p : P.ck_u) dfree(p);
  for (double *p : P.ck_h) dfree(p);
  for (double *p : P.seg_u) dfree(p);
  for (double *p : P.seg_h) dfree(p);
  P.ck_u.clear(); P.ck_h.clear(); P.seg_u.clear(); P.seg_h.clear();
  for (double *p : {P.d_ke, P.h_a, P.h_b, P.mu_a, P.mu_b, P.adj.x, P.adj.r, P.adj.rh, P.adj.p, P.adj.v, P.adj.s,
                    P.adj.t, P.adj.y, P.adj.z, P.adj.kinv, P.d_out})
    dfree(p);
  dfree(P.d_st);
  P = PathState{};
}

// One accepted step of the path on slot 0: Newton at strain n from the slot's current u with history h_prev,
// then h_next = H(u, h_prev).  The stress of the step goes to sigma[6].
bool Engine::path_step(int n, double *h_prev, double *h_next, double *sigma, bool record) {
  PathState &P = path_;
  Inst &I = h_insts_[0];
  I.vars_old = h_prev;
  I.has_vars_old = 1;
  I.vars_new = h_next;
  std::array<double, 6> e;
  std::memcpy(e.data(), &P.strains[(size_t)n * 6], sizeof(e));
  double de[6];
  for (int q = 0; q < 6; ++q) de[q] = e[q] - (n > 0 ? P.strains[(size_t)(n - 1) * 6 + q] : 0.0);
  launches_ += 1;
  check_launch(mgb_launch_affine_add(&mesh_, slots_[0].u, de, stream_), "path predictor");
  const std::vector<NewtonResult> r = newton({0}, {e});
  std::memcpy(sigma, h_out_[0].sig, 6 * sizeof(double));
  // converged also when the last allowed iteration reached the tolerance (the reference's loop tests before
  // each iteration only)
  const bool conv = r[0].converged || r[0].rel_norm < nr_rel_tol_ || h_out_[0].norm < nr_max_tol_;
  if (record) {
    P.nr_its[n] = r[0].its;
    P.cg_its[n] = r[0].solver_its;
    P.nr_conv[n] = conv ? 1 : 0;
    P.cg_maxed[n] = r[0].cg_maxed ? 1 : 0;
    P.nr_norm[n] = r[0].rel_norm;
  }
  check(cudaMemcpyAsync(h_next, h_prev, nvars() * sizeof(double), cudaMemcpyDeviceToDevice, stream_), "history copy");
  upload_insts();
  upload_list({0});
  launches_ += 1;
  check_launch(mgb_launch_evolve(&mesh_, &mats_, d_etype_, d_dsh_, d_insts_, d_list_, 1, stream_), "path evolve");
  return conv;
}

namespace {

// The handle's materials, precision, tangent and elastic element matrices swapped for the path's while a path
// runs (the path's Newton is FP64 with the exact consistent tangent).
struct PathScope {
  Mats &mats;
  double *&ke;
  int &precision;
  bool &exact;
  Mats saved_mats;
  double *saved_ke;
  int saved_precision;
  bool saved_exact;
  PathScope(Mats &m, double *&k, int &p, bool &x, const Mats &pm, double *pk)
      : mats(m), ke(k), precision(p), exact(x), saved_mats(m), saved_ke(k), saved_precision(p), saved_exact(x) {
    mats = pm;
    ke = pk;
    precision = MICROPP3_FP64;
    exact = true;
  }
  ~PathScope() {
    mats = saved_mats;
    ke = saved_ke;
    precision = saved_precision;
    exact = saved_exact;
  }
};

}  // namespace

int Engine::path_forward(int nsteps, const double *strains, const double *params, int every, double *sigma) {
  if (nsteps <= 0 || !strains || !params || !sigma || every <= 0)
    throw std::invalid_argument("path: nsteps > 0, strains, params, sigma and checkpoint_every > 0 are required");
  path_free();
  PathState &P = path_;
  P.nsteps = nsteps;
  P.every = every;
  P.strains.assign(strains, strains + (size_t)nsteps * 6);
  for (int ph = 0; ph < 3; ++ph) {
    const double *t = params + ph * 5;  // E, nu, Xt, Sy, Ka
    P.mats.m[ph] = make_matdev(mats_.m[ph].type, t[0], t[1], t[4], t[3], t[2]);
  }
  phase_stiffness(P.mats, P.ke, nullptr);
  P.d_ke = dalloc<double>(3 * 576, "path ke");
  check(cudaMemcpy(P.d_ke, P.ke, sizeof(P.ke), cudaMemcpyHostToDevice), "path ke upload");
  ensure_fp64_slot0();
  path_alloc_adj();
  const size_t nd = nndim(), nv = nvars();
  P.h_a = dalloc<double>(nv, "path history");
  P.h_b = dalloc<double>(nv, "path history");
  check(cudaMemsetAsync(P.h_a, 0, nv * sizeof(double), stream_), "history zero");
  check(cudaMemsetAsync(slots_[0].u, 0, nd * sizeof(double), stream_), "u zero");
  const int nck = (nsteps + every - 1) / every;
  for (int c = 0; c < nck; ++c) {
    P.ck_u.push_back(dalloc<double>(nd, "checkpoint u"));
    P.ck_h.push_back(dalloc<double>(nv, "checkpoint history"));
  }
  P.nr_its.assign(nsteps, 0);
  P.cg_its.assign(nsteps, 0);
  P.nr_conv.assign(nsteps, 0);
  P.cg_maxed.assign(nsteps, 0);
  P.nr_norm.assign(nsteps, 0.0);
  PathScope scope(mats_, d_ke_, precision_, exact_tangent_, P.mats, P.d_ke);
  bool ok = true;
  double *hp = P.h_a, *hn = P.h_b;
  for (int n = 0; n < nsteps; ++n) {
    if (n % every == 0) {
      check(cudaMemcpyAsync(P.ck_u[n / every], slots_[0].u, nd * sizeof(double), cudaMemcpyDeviceToDevice, stream_),
            "checkpoint");
      check(cudaMemcpyAsync(P.ck_h[n / every], hp, nv * sizeof(double), cudaMemcpyDeviceToDevice, stream_),
            "checkpoint");
    }
    ok &= path_step(n, hp, hn, sigma + (size_t)n * 6, true);
    std::swap(hp, hn);
  }
  sync();
  P.ready = true;
  return ok ? 0 : 1;
}

void Engine::path_newton(int step, int *its, int *cg_its, int *converged, double *rel_norm) const {
  const PathState &P = path_;
  if (step < 0 || step >= (int)P.nr_its.size()) throw std::out_of_range("path_newton: no such step of the last path");
  if (its) *its = P.nr_its[step];
  if (cg_its) *cg_its = P.cg_its[step];
  if (converged) *converged = P.nr_conv[step] + 2 * P.cg_maxed[step];
  if (rel_norm) *rel_norm = P.nr_norm[step];
}

void Engine::path_alloc_adj() {
  PathState &P = path_;
  if (P.mu_a) return;
  const size_t nd = nndim(), nv = nvars();
  P.mu_a = dalloc<double>(nv, "history adjoint");
  P.mu_b = dalloc<double>(nv, "history adjoint");
  for (double **v : {&P.adj.x, &P.adj.r, &P.adj.rh, &P.adj.p, &P.adj.v, &P.adj.s, &P.adj.t, &P.adj.y, &P.adj.z,
                     &P.adj.kinv})
    *v = dalloc<double>(nd, "BiCGSTAB vector");
  P.d_st = dalloc<BicgState>(1, "bicg state");
  P.adj.st = P.d_st;
  P.d_out = dalloc<double>(21, "adjoint sums");
}

// K x = b (transpose: K^T x = b) on slot 0's FP64 ELL and right-hand side, to the handle's CG tolerance.
// Returns the iterations; last_bicg_converged_ tells whether the tolerance was met.
int Engine::bicg_solve(bool transpose, double *x) {
  PathState &P = path_;
  Slot &w = slots_[0];
  double *x_buf = P.adj.x;
  P.adj.x = x;
  P.adj.b = w.b;
  P.adj.vals = w.vals;
  P.adj.red = w.red;
  P.adj.ticket = w.ticket;
  BicgState st{};
  st.rel_tol = std::max(cg_rel_tol_, kAdjTol);
  st.max_its = std::min(std::max(cg_max_its_, 1), kAdjMaxIts);
  check(cudaMemcpyAsync(P.d_st, &st, sizeof(st), cudaMemcpyHostToDevice, stream_), "bicg state");
  launches_ += 1;
  check_launch(mgb_launch_bicg_init(&mesh_, &P.adj, stream_), "bicg init");
  const int chunk = 16;
  for (int done = 0; done <= kAdjMaxIts; done += chunk) {
    check(cudaMemsetAsync(d_count_, 0, sizeof(unsigned int), stream_), "count reset");
    for (int it = 0; it < chunk; ++it) {
      launches_ += 5;
      check_launch(mgb_launch_bicg_iter(&mesh_, &P.adj, d_count_, transpose ? 1 : 0, stream_), "bicg iteration");
    }
    check(cudaMemcpyAsync(h_count_, d_count_, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream_), "count");
    sync();
    if (*h_count_ == 0) break;
  }
  check(cudaMemcpyAsync(&st, P.d_st, sizeof(st), cudaMemcpyDeviceToHost, stream_), "bicg state");
  sync();
  P.adj.x = x_buf;
  last_bicg_converged_ = st.converged != 0;
  return st.its;
}

int Engine::path_vjp(const double *gsigma, double *grad_params, double *grad_strains) {
  PathState &P = path_;
  if (!P.ready) throw std::runtime_error("path_vjp: no path (call micropp3_path_forward first)");
  if (!gsigma || !grad_params) throw std::invalid_argument("path_vjp: gsigma and grad_params are required");
  const size_t nd = nndim(), nv = nvars();
  ensure_fp64_slot0();
  if (P.seg_u.empty())
    for (int k = 0; k < P.every; ++k) {
      P.seg_u.push_back(dalloc<double>(nd, "segment u"));
      P.seg_h.push_back(dalloc<double>(nv, "segment history"));
    }
  path_alloc_adj();
  std::fill(grad_params, grad_params + 15, 0.0);
  if (grad_strains) std::fill(grad_strains, grad_strains + (size_t)P.nsteps * 6, 0.0);
  P.bicg_its = 0;
  P.bicg_converged = true;
  PathScope scope(mats_, d_ke_, precision_, exact_tangent_, P.mats, P.d_ke);
  const double wgv = mesh_.wg / mesh_.vol_tot;
  const double *mu_in = nullptr;  // dL/dh after the last step: nothing depends on it
  double *mu_out = P.mu_a;
  std::vector<double> sig(6);
  const int nseg = (P.nsteps + P.every - 1) / P.every;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int s0 = seg * P.every, s1 = std::min(s0 + P.every, P.nsteps);
    // recompute the segment from its checkpoint
    check(cudaMemcpyAsync(slots_[0].u, P.ck_u[seg], nd * sizeof(double), cudaMemcpyDeviceToDevice, stream_), "restore");
    check(cudaMemcpyAsync(P.h_a, P.ck_h[seg], nv * sizeof(double), cudaMemcpyDeviceToDevice, stream_), "restore");
    double *hp = P.h_a, *hn = P.h_b;
    for (int n = s0; n < s1; ++n) {
      check(cudaMemcpyAsync(P.seg_h[n - s0], hp, nv * sizeof(double), cudaMemcpyDeviceToDevice, stream_), "segment");
      path_step(n, hp, hn, sig.data(), false);
      check(cudaMemcpyAsync(P.seg_u[n - s0], slots_[0].u, nd * sizeof(double), cudaMemcpyDeviceToDevice, stream_),
            "segment");
      std::swap(hp, hn);
    }
    // adjoint steps, last to first
    for (int n = s1 - 1; n >= s0; --n) {
      check(cudaMemcpyAsync(slots_[0].u, P.seg_u[n - s0], nd * sizeof(double), cudaMemcpyDeviceToDevice, stream_),
            "adjoint state");
      Inst &I = h_insts_[0];
      I.vars_old = P.seg_h[n - s0];
      I.has_vars_old = 1;
      upload_insts();
      upload_list({0});
      launches_ += 9;
      check_launch(mgb_launch_assembly_dual(&mesh_, &mats_, d_etype_, d_dsh_, d_ke_, d_insts_, d_list_, 1, stream_),
                   "adjoint tangent");
      AdjStep st{};
      std::memcpy(st.g, gsigma + (size_t)n * 6, sizeof(st.g));
      st.wgv = wgv;
      st.mu_in = mu_in;
      st.mu_out = mu_out;
      st.lam = P.adj.x;
      st.out = P.d_out;
      launches_ += 2;
      check_launch(mgb_launch_adj_rhs(&mesh_, &mats_, d_etype_, d_dsh_, d_insts_, d_list_, &st, stream_), "adjoint rhs");
      check_launch(mgb_launch_node_gather(&mesh_, d_insts_, d_list_, 1, stream_), "adjoint rhs gather");
      P.bicg_its += bicg_solve(true, P.adj.x);
      if (!last_bicg_converged_) P.bicg_converged = false;
      launches_ += 1;
      check_launch(mgb_launch_adj_back(&mesh_, &mats_, d_etype_, d_dsh_, d_insts_, d_list_, &st, stream_),
                   "adjoint step");
      double out[21];
      check(cudaMemcpyAsync(out, P.d_out, sizeof(out), cudaMemcpyDeviceToHost, stream_), "adjoint sums");
      sync();
      for (int q = 0; q < 15; ++q) grad_params[q] += out[q];
      if (grad_strains)
        for (int i = 0; i < 6; ++i) grad_strains[(size_t)n * 6 + i] = out[15 + i];
      mu_in = mu_out;
      mu_out = (mu_out == P.mu_a) ? P.mu_b : P.mu_a;
    }
  }
  return P.bicg_converged ? 0 : 1;
}

}  // namespace mgb
