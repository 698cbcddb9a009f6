// engine.cpp -- host orchestration of the GB300 homogenization (see engine.hpp).
//
// This file is compiled with -ffp-contract=off: the few FP64 quantities formed on the host (shape
// function gradients, the elastic phase stiffness, material constants, the mixture-rule tangent) are then
// rounded exactly as the reference rounds them.
#include "engine.hpp"

#include <algorithm>
#include <functional>
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>

#include "cuda_util.hpp"
#include "launch.h"
#include "microstructure.hpp"

namespace mgb {

namespace {

constexpr double kConstXg = 0.577350269189626;  // params.hpp:34
constexpr double kDepsCtanAve = 1.0e-8;        // params.hpp:32

// Tangent solve of the implicit ctan: FP32 CG sweeps to this relative tolerance, refined with FP64-accurate
// (double-float) residuals until ||f_i - K x_i|| <= kTangentTol ||f_i|| for all six right-hand sides (at most
// kTangentSweeps sweeps).
constexpr double kTangentSweepRel = 1.0e-5;
constexpr double kTangentTol = 1.0e-9;
// With a symmetric tangent (every phase elastic or damage) ctan takes the energy form from element energies,
// whose error is quadratic in the solve's: the sweeps go to 2e-6 and the refinement stops at 3e-6 ||f_i||.
constexpr double kTangentSweepRelEnergy = 2.0e-6;
constexpr double kTangentTolEnergy = 3.0e-6;
constexpr int kTangentSweeps = 4;

// Lowest relative tolerance asked of the mixed form's FP32 Newton CG.
constexpr double kFp32CgFloor = 1.0e-6;

// Multigrid preconditioner of the FP32 solves: the smoother diagonal max(a_ii / kMgOmega, kMgSafe sum_j |a_ij|),
// pairs of Jacobi sweeps on the coarsest level after the first one (9 sweeps), CG iterations between polls of
// the active count, and the iteration cap of a multigrid solve: one that reaches it is redone with Jacobi.
constexpr float kMgOmega = 0.6f;
constexpr float kMgSafe = 0.55f;
constexpr int kMgCoarsePairs = 4;
constexpr int kMgChunk = 4;
constexpr int kMgMaxIts = 100;

// A structured grid of nx x ny x nz nodes (the multigrid levels and the separable product's intermediates).
static MeshDev grid_of(int nx, int ny, int nz) {
  MeshDev g{};
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.nex = nx - 1;
  g.ney = ny - 1;
  g.nez = nz - 1;
  g.nelem = g.nex * g.ney * g.nez;
  g.nxny = nx * ny;
  g.nn = g.nxny * nz;
  g.np = (g.nn + 31) / 32 * 32;
  return g;
}

const int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

}  // namespace

// ------------------------------------------------------------------------------------------------
// Construction (micropp.cpp:29-171)

Engine::Engine(const micropp3_config &cfg) {
  if (cfg.ngp <= 0) throw std::invalid_argument("ngp must be positive");
  for (int d = 0; d < 3; ++d)
    if (cfg.size[d] < 2) throw std::invalid_argument("size[] must be at least 2 nodes per axis");
  ngp_ = cfg.ngp;
  micro_type_ = cfg.micro_type;
  mpi_rank_ = cfg.mpi_rank;
  std::memcpy(geo_params_, cfg.geo_params, sizeof(geo_params_));
  for (int i = 0; i < 3; ++i) mat_in_[i] = cfg.materials[i];
  nr_max_its_ = cfg.nr_max_its;
  nr_max_tol_ = cfg.nr_max_tol;
  nr_rel_tol_ = cfg.nr_rel_tol;
  cg_max_its_ = cfg.cg_max_its;
  cg_abs_tol_ = cfg.cg_abs_tol;
  cg_rel_tol_ = cfg.cg_rel_tol;
  lin_stress_ = cfg.lin_stress != 0;
  subiterations_ = cfg.subiterations != 0;
  nsubiterations_ = cfg.nsubiterations;
  calc_ctan_lin_ = cfg.calc_ctan_lin != 0;
  precision_ = cfg.precision;
  ctan_mode_ = cfg.ctan_mode;
  if (precision_ != MICROPP3_FP64 && precision_ != MICROPP3_MIXED)
    throw std::invalid_argument("precision must be MICROPP3_FP64 or MICROPP3_MIXED");
  if (ctan_mode_ != MICROPP3_CTAN_PERTURB && ctan_mode_ != MICROPP3_CTAN_IMPLICIT)
    throw std::invalid_argument("ctan_mode must be MICROPP3_CTAN_PERTURB or MICROPP3_CTAN_IMPLICIT");

  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    throw std::runtime_error("no CUDA device is available: the GB300 homogenization library has no CPU path");

  build_mesh(cfg);
  build_elem_types(cfg);
  build_materials(cfg);
  build_phase_stiffness();
  // The FP32 Jacobian (mixed precision or implicit ctan) is assembled by node gather from the residual's
  // Gauss-point tangent terms when every phase in use is elastic or damage; a J2 phase keeps the element
  // colouring assembly.
  gather32_ = precision_ == MICROPP3_MIXED || ctan_mode_ == MICROPP3_CTAN_IMPLICIT;
  for (int e = 0; e < mesh_.nelem && gather32_; ++e) gather32_ = mats_.m[etype_[e]].type != 1;
  // Multigrid levels: every axis of n elements coarsens to ceil(n / 2) while each axis keeps at least 4
  // elements and some axis has more than 4.
  {
    const int pc0 = cfg.precond;
    if (pc0 != MICROPP3_PRECOND_JACOBI && pc0 != MICROPP3_PRECOND_MG && pc0 != MICROPP3_PRECOND_MG_HALF)
      throw std::invalid_argument("precond must be MICROPP3_PRECOND_JACOBI, MICROPP3_PRECOND_MG or "
                                  "MICROPP3_PRECOND_MG_HALF");
    mg_half_ = pc0 == MICROPP3_PRECOND_MG_HALF;
    const int pc = mg_half_ ? MICROPP3_PRECOND_MG : pc0;
    const bool fp32_solves = precision_ == MICROPP3_MIXED || ctan_mode_ == MICROPP3_CTAN_IMPLICIT;
    if (pc == MICROPP3_PRECOND_MG && !fp32_solves)
      throw std::invalid_argument("the multigrid preconditioner applies to the FP32 solves (MICROPP3_MIXED or "
                                  "MICROPP3_CTAN_IMPLICIT); the FP64 Newton keeps the reference's Jacobi CG");
    mg_mesh_.assign(1, mesh_);
    int ne[3] = {mesh_.nex, mesh_.ney, mesh_.nez};
    while ((int)mg_mesh_.size() < kMgMaxLevels) {
      const int lo = std::min(ne[0], std::min(ne[1], ne[2])), hi = std::max(ne[0], std::max(ne[1], ne[2]));
      if (lo < 4 || hi <= 4) break;
      for (int &e : ne) e = (e + 1) / 2;
      mg_mesh_.push_back(grid_of(ne[0] + 1, ne[1] + 1, ne[2] + 1));
    }
    mg_ = pc == MICROPP3_PRECOND_MG && mg_mesh_.size() >= 2;
    if (pc == MICROPP3_PRECOND_MG && !mg_)
      throw std::invalid_argument("the multigrid preconditioner needs at least 4 elements along every axis and "
                                  "more than 4 along one");
    if (!mg_) mg_mesh_.clear();
    if (!mg_) mg_half_ = false;
    if (mg_half_) {
      // Scale of the FP16 copy: an entry of the fine operator is a sum of at most 8 element blocks; with the
      // largest entry of the phases' elastic element matrices as the unit, 8 of them map to 2^10, which leaves a
      // factor 64 below the FP16 maximum for tangents stiffer than elastic (loading damage) and keeps entries
      // down to 1e-7 of it normal.
      double kmax = 0.0;
      for (int ph = 0; ph < 3; ++ph)
        for (int q = 0; q < 576; ++q) kmax = std::max(kmax, std::fabs(ke_phase_[ph][q]));
      const double bound = 8.0 * std::max(kmax, 1e-300);
      mg_scale16_ = (float)std::ldexp(1.0, (int)std::floor(std::log2(1024.0 / bound)));
    }
  }

  check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
  if (mg_) check_launch(mgb_mg_init_attributes(), "multigrid kernel attributes");
  check(cudaEventCreate(&ev0_), "event");
  check(cudaEventCreate(&ev1_), "event");
  d_etype_ = dalloc<int8_t>(mesh_.nelem, "elem_type");
  check(cudaMemcpy(d_etype_, etype_.data(), mesh_.nelem, cudaMemcpyHostToDevice), "elem_type upload");
  d_dsh_ = dalloc<double>(192, "dsh");
  check(cudaMemcpy(d_dsh_, dsh_, sizeof(dsh_), cudaMemcpyHostToDevice), "dsh upload");
  d_ke_ = dalloc<double>(3 * 576, "ke");
  check(cudaMemcpy(d_ke_, ke_phase_, sizeof(ke_phase_), cudaMemcpyHostToDevice), "ke upload");
  {
    float ke32[3 * 576];
    for (int i = 0; i < 3 * 576; ++i) ke32[i] = (float)(&ke_phase_[0][0])[i];
    d_ke32_ = dalloc<float>(3 * 576, "ke32");
    check(cudaMemcpy(d_ke32_, ke32, sizeof(ke32), cudaMemcpyHostToDevice), "ke32 upload");
    d_k0g32_ = dalloc<float>(k0g32_.size(), "k0g32");
    check(cudaMemcpy(d_k0g32_, k0g32_.data(), k0g32_.size() * sizeof(float), cudaMemcpyHostToDevice), "k0g upload");
    float dsh32[192];
    for (int i = 0; i < 192; ++i) dsh32[i] = (float)dsh_[i];
    d_dsh32_ = dalloc<float>(192, "dsh32");
    check(cudaMemcpy(d_dsh32_, dsh32, sizeof(dsh32), cudaMemcpyHostToDevice), "dsh32 upload");
  }
  {
    // interior nodes with a boundary neighbour: the rows of the tangent right-hand sides f_i = -K_IB w_i
    std::vector<int> near;
    for (int k = 1; k < mesh_.nz - 1; ++k)
      for (int j = 1; j < mesh_.ny - 1; ++j)
        for (int i = 1; i < mesh_.nx - 1; ++i)
          if (i == 1 || j == 1 || k == 1 || i == mesh_.nx - 2 || j == mesh_.ny - 2 || k == mesh_.nz - 2)
            near.push_back((k * mesh_.ny + j) * mesh_.nx + i);
    nnear_ = (int)near.size();
    if (nnear_ > 0) {
      d_near_ = dalloc<int>(near.size(), "near-boundary nodes");
      check(cudaMemcpy(d_near_, near.data(), near.size() * sizeof(int), cudaMemcpyHostToDevice), "near upload");
    }
  }
  check(cudaMallocHost((void **)&h_count_, sizeof(unsigned int)), "pinned count");
  d_count_ = dalloc<unsigned int>(1, "count");
  check(cudaMallocHost((void **)&h_chunks_, sizeof(unsigned int)), "pinned chunk count");
  d_chunks_ = dalloc<unsigned int>(1, "chunk count");

  gps_.resize(ngp_);
  int n_fe = 0;
  for (int i = 0; i < ngp_; ++i) {
    GpState &g = gps_[i];
    g.coupling = cfg.coupling ? cfg.coupling[i] : MICROPP3_FE_ONE_WAY;
    if (g.coupling < MICROPP3_FE_LINEAR || g.coupling > MICROPP3_MIX_RULE_CHAMIS)
      throw std::invalid_argument("coupling must be FE_LINEAR, FE_ONE_WAY, FE_FULL or MIX_RULE_CHAMIS");
    if (!cfg.coupling || g.coupling == MICROPP3_FE_ONE_WAY || g.coupling == MICROPP3_FE_FULL) {
      g.u_n = dalloc<double>(nndim(), "u_n");
      g.u_k = dalloc<double>(nndim(), "u_k");
      check(cudaMemsetAsync(g.u_n, 0, nndim() * sizeof(double), stream_), "u_n zero");
      check(cudaMemsetAsync(g.u_k, 0, nndim() * sizeof(double), stream_), "u_k zero");
    }
    if (g.coupling != MICROPP3_MIX_RULE_CHAMIS) n_fe++;
  }

  // calc_volume_fractions (micropp.cpp:609-627)
  const double evol = mesh_.dx * mesh_.dy * mesh_.dz;
  Vm_ = Vf_ = 0.0;
  for (int e = 0; e < mesh_.nelem; ++e) {
    if (etype_[e] == 0)
      Vm_ += evol;
    else if (etype_[e] >= 1)
      Vf_ += evol;
  }
  Vm_ /= mesh_.vol_tot;
  Vf_ /= mesh_.vol_tot;

  // A0 (micropp.cpp:128-143): the Jacobian at u = 0 without history, assembled once before the linear ctan
  // (whose solves use it).  FP64 form only: the mixed form always assembles its FP32 Jacobian.
  use_A0_ = cfg.use_A0 != 0 && precision_ == MICROPP3_FP64;
  its_with_A0_ = cfg.its_with_A0;
  if (use_A0_) {
    ensure_slots(1);
    d_A0_ = dalloc<double>((size_t)kEllPerNode * mesh_.np, "A0");
    check(cudaMemsetAsync(slots_[0].u, 0, nndim() * sizeof(double), stream_), "A0 u");
    Inst &I = h_insts_[0];
    I.vars_old = nullptr;
    I.has_vars_old = 0;
    I.vals = d_A0_;
    upload_insts();
    upload_list({0});
    launches_ += 9;
    check_launch(mgb_launch_assembly(&mesh_, &mats_, d_etype_, d_dsh_, d_ke_, d_insts_, d_list_, 1, stream_), "A0");
    I.vals = slots_[0].vals;
    upload_insts();
  }

  std::memset(ctan_lin_, 0, sizeof(ctan_lin_));
  if (calc_ctan_lin_ && n_fe > 0) calc_ctan_lin();
  for (auto &g : gps_) {
    if (g.coupling == MICROPP3_MIX_RULE_CHAMIS)
      ctan_mix_rule_chamis(g.ctan);
    else
      std::memcpy(g.ctan, ctan_lin_, sizeof(ctan_lin_));
  }
  sync();
}

Engine::~Engine() {
  if (stream_) cudaStreamSynchronize(stream_);
  for (auto &g : gps_) {
    dfree(g.u_n);
    dfree(g.u_k);
    dfree(g.vars_n);
    dfree(g.vars_k);
  }
  clear_graphs();
  path_free();
  free_slots();
  for (KernelTimer *t : {&t_spmv_, &t_update_, &t_asm_, &t_res_, &t_spmv6_, &t_upd6_, &t_mg1_, &t_mg6_, &t_mgc_, &t_rap_,
                          &t_tan_})
    for (auto &e : t->pool) {
      cudaEventDestroy(e.first);
      cudaEventDestroy(e.second);
    }
  dfree(d_etype_);
  dfree(d_dsh_);
  dfree(d_ke_);
  dfree(d_ke32_);
  dfree(d_k0g32_);
  dfree(d_dsh32_);
  dfree(d_near_);
  dfree(d_A0_);
  dfree(d_count_);
  if (h_count_) cudaFreeHost(h_count_);
  dfree(d_chunks_);
  if (h_chunks_) cudaFreeHost(h_chunks_);
  dfree(d_eta_);
  if (h_eta_) cudaFreeHost(h_eta_);
  for (cudaEvent_t e : tune_ev_)
    if (e) cudaEventDestroy(e);
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
  if (stream_) cudaStreamDestroy(stream_);
}

void Engine::build_mesh(const micropp3_config &cfg) {
  MeshDev &m = mesh_;
  m.nx = cfg.size[0];
  m.ny = cfg.size[1];
  m.nz = cfg.size[2];
  m.nxny = m.nx * m.ny;
  const long long nn = (long long)m.nx * m.ny * m.nz;
  if (nn * kEllPerNode > 2000000000LL)
    throw std::invalid_argument("RVE too large for one device instance (at most ~8.2M nodes)");
  m.nn = (int)nn;
  m.np = (m.nn + 31) & ~31;
  m.nex = m.nx - 1;
  m.ney = m.ny - 1;
  m.nez = m.nz - 1;
  m.nelem = m.nex * m.ney * m.nez;
  m.lx = m.ly = m.lz = 1.0;
  m.dx = m.lx / m.nex;
  m.dy = m.ly / m.ney;
  m.dz = m.lz / m.nez;
  m.wg = m.dx * m.dy * m.dz / kNpe;
  m.vol_tot = m.lx * m.ly * m.lz;
  // calc_bmat (micro3D.cpp:80-120): gradient of shape function i at Gauss point gp, formed as
  // (s_a (1 + s_b xi_b)) (1 + s_c xi_c) / 8 * 2 / h, the reference's expression with the signs factored.
  const double h[3] = {m.dx, m.dy, m.dz};
  for (int gp = 0; gp < 8; ++gp) {
    double xg[3];
    for (int d = 0; d < 3; ++d) xg[d] = kCorner[gp][d] ? kConstXg : -kConstXg;
    for (int i = 0; i < 8; ++i) {
      double s[3], g[3];
      for (int d = 0; d < 3; ++d) s[d] = kCorner[i][d] ? 1.0 : -1.0;
      for (int d = 0; d < 3; ++d) {
        const int p = (d == 0) ? 1 : 0, q = (d == 2) ? 1 : 2;
        const double f1 = 1 + s[p] * xg[p];
        const double f2 = 1 + s[q] * xg[q];
        g[d] = s[d] * f1 * f2 / 8. * 2. / h[d];
        dsh_[gp * 24 + i * 3 + d] = g[d];
      }
      double *B = &bmat_[gp][0][0];
      const int c = i * 3;
      for (int r = 0; r < 6; ++r) B[r * 24 + c] = B[r * 24 + c + 1] = B[r * 24 + c + 2] = 0.0;
      B[0 * 24 + c] = g[0];
      B[1 * 24 + c + 1] = g[1];
      B[2 * 24 + c + 2] = g[2];
      B[3 * 24 + c] = g[1];
      B[3 * 24 + c + 1] = g[0];
      B[4 * 24 + c] = g[2];
      B[4 * 24 + c + 2] = g[0];
      B[5 * 24 + c + 1] = g[2];
      B[5 * 24 + c + 2] = g[1];
    }
  }
}

void Engine::build_elem_types(const micropp3_config &cfg) {
  const MeshDev &m = mesh_;
  etype_.resize(m.nelem);
  for (int ez = 0; ez < m.nez; ++ez)
    for (int ey = 0; ey < m.ney; ++ey)
      for (int ex = 0; ex < m.nex; ++ex) {
        const int e = (ez * m.ney + ey) * m.nex + ex;
        const int t = cfg.elem_type ? cfg.elem_type[e]
                                    : micro_elem_type(micro_type_, geo_params_, ex, ey, ez, m.dx, m.dy, m.dz);
        if (t < 0 || t > 2) {
          std::ostringstream os;
          os << "element " << e << " has phase " << t << " (micro_type " << micro_type_
             << "); phases must be 0, 1 or 2";
          throw std::invalid_argument(os.str());
        }
        etype_[e] = (int8_t)t;
      }
}

// Material constants with the expressions of material.hpp:73-135 and material.cpp:205-225.
// Constants of one material for the device laws, by the reference's expressions (material.c:26-38,
// material.cpp:110-147, 205-225).
MatDev make_matdev(int type, double E, double nu, double Ka, double Sy, double Xt) {
  MatDev d{};
  d.type = type;
  d.E = E;
  d.nu = nu;
  d.k = E / (3. * (1. - 2. * nu));
  d.mu = E / (2. * (1. + nu));
  d.lambda = nu * E / ((1. + nu) * (1. - 2. * nu));
  d.Ka = (type == 1) ? Ka : -1.0;
  d.Sy = (type == 1) ? Sy : -1.0;
  d.Xt = (type == 2) ? Xt : -1.0;
  d.two_mu = 2 * d.mu;
  const double sqE = std::sqrt(d.E);
  d.xt_thr = d.Xt / sqE;
  const double Ey = 10.0e4, inf_Ey = 10. * Ey, H0 = 10.0;
  d.dmg_r0 = Ey / sqE;
  d.dmg_q0 = d.dmg_r0;
  d.dmg_q1 = inf_Ey / sqE;
  d.dmg_r1 = d.dmg_r0 + (d.dmg_q1 - d.dmg_q0) / H0;
  d.pl_den = 2. * d.mu * (1. + d.Ka / (3. * d.mu));
  return d;
}

void Engine::build_materials(const micropp3_config &cfg) {
  for (int i = 0; i < 3; ++i) {
    const material_base &b = cfg.materials[i];
    if (b.type < 0 || b.type > 2) throw std::invalid_argument("material type must be 0, 1 or 2");
    mats_.m[i] = make_matdev(b.type, b.E, b.nu, b.Ka, b.Sy, b.Xt);
  }
}

// Element stiffness of an elastic phase, get_elem_mat (assembly.cpp:140-178) with the elastic ctan
// (material.cpp:84-95).  B and wg are uniform over the mesh, so one Ke serves every element of the phase.
void Engine::build_phase_stiffness() { phase_stiffness(mats_, ke_phase_, &k0g32_); }

void Engine::phase_stiffness(const Mats &mats, double (*ke)[576], std::vector<float> *k0g) const {
  if (k0g) k0g->assign((size_t)3 * 8 * 576, 0.0f);
  for (int ph = 0; ph < 3; ++ph) {
    const MatDev &m = mats.m[ph];
    double C[36] = {0};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) C[i * 6 + j] += m.lambda;
    for (int i = 0; i < 3; ++i) C[i * 6 + i] += 2 * m.mu;
    for (int i = 3; i < 6; ++i) C[i * 6 + i] = m.mu;
    double *K = ke[ph];
    std::memset(K, 0, 576 * sizeof(double));
    for (int gp = 0; gp < 8; ++gp) {
      double cxb[6][24];
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 24; ++j) {
          double t = 0.0;
          for (int k = 0; k < 6; ++k) t += C[i * 6 + k] * bmat_[gp][k][j];
          cxb[i][j] = t * mesh_.wg;
        }
      double Kg[576] = {0};
      for (int mm = 0; mm < 6; ++mm)
        for (int i = 0; i < 24; ++i) {
          const double bmi = bmat_[gp][mm][i];
          for (int j = 0; j < 24; ++j) {
            K[i * 24 + j] += bmi * cxb[mm][j];
            Kg[i * 24 + j] += bmi * cxb[mm][j];
          }
        }
      if (k0g)
        for (int q = 0; q < 576; ++q) (*k0g)[((size_t)ph * 8 + gp) * 576 + q] = (float)Kg[q];
    }
  }
}

// calc_ctan_lin_mix_rule_Chamis (micropp.cpp:286-331).
void Engine::ctan_mix_rule_chamis(double *ctan) const {
  const double Em = mat_in_[0].E, nu_m = mat_in_[0].nu, Gm = Em / (2 * (1 + nu_m));
  const double Ef = mat_in_[1].E, nu_f = mat_in_[1].nu, Gf = Ef / (2 * (1 + nu_f));
  const double E11 = Vf_ * Ef + Vm_ * Em;
  const double E22 = Em / (1 - std::sqrt(Vf_) * (1 - Em / Ef));
  const double nu12 = Vf_ * nu_f + Vm_ * nu_m;
  const double G12 = Gm / (1 - std::sqrt(Vf_) * (1 - Gm / Gf));
  const double nu23 = nu12;
  const double S[3][3] = {{1 / E11, -nu12 / E11, -nu12 / E11},
                          {-nu12 / E11, 1 / E22, -nu23 / E22},
                          {-nu12 / E11, -nu23 / E22, 1 / E22}};
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
  std::memset(ctan, 0, 36 * sizeof(double));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) ctan[i * 6 + j] = Si[i][j];
  ctan[3 * 6 + 3] = G12;
  ctan[4 * 6 + 4] = G12;
  ctan[5 * 6 + 5] = G12;
}

// ------------------------------------------------------------------------------------------------
// Workspace slots

// Device bytes of one workspace slot in this handle's mode.
double Engine::slot_bytes() const {
  const double nd = nndim(), np = mesh_.np;
  double b = 8.0 * (3.0 * nd + 24.0 * mesh_.nelem + nvars());  // u, du, b, be, vars_aux
  if (precision_ == MICROPP3_FP64) b += 8.0 * (kEllPerNode * np + 5.0 * nd);
  if (precision_ == MICROPP3_MIXED || ctan_mode_ == MICROPP3_CTAN_IMPLICIT)
    b += 4.0 * (kEllPerNode * np + nd + (gather32_ ? 64.0 * mesh_.nelem : 0.0));
  if (precision_ == MICROPP3_MIXED) b += 4.0 * 5.0 * nd;
  if (ctan_mode_ == MICROPP3_CTAN_IMPLICIT) b += (8.0 * 2.0 + 4.0 * 5.0) * 18.0 * np;
  if (mg_) {
    b += 4.0 * 21.0 * np;
    for (size_t l = 1; l < mg_mesh_.size(); ++l) b += 4.0 * (kEllPerNode + 3.0 + 4.0 * 18.0) * mg_mesh_[l].np;
    const MeshDev &c = mg_mesh_[1];
    b += 4.0 * kEllPerNode * (grid_of(c.nx, mesh_.ny, mesh_.nz).np + grid_of(c.nx, c.ny, mesh_.nz).np);
  }
  return b;
}

void Engine::ensure_slots(int n) {
  if ((int)slots_.size() >= n) return;
  const int old = (int)slots_.size();
  const size_t nd = nndim(), nv = nvars();
  // Reduction partials: one slot per block of the largest reducing grid (the row-parallel CG updates,
  // 3*nn/kNodeBlock blocks; the Gauss-point kernels, 8*nelem/128 blocks).
  const int nblocks = std::max((3 * mesh_.nn + kNodeBlock - 1) / kNodeBlock, (mesh_.nelem * 8 + 127) / 128) + 8;
  const bool fp64 = precision_ == MICROPP3_FP64, mixed = precision_ == MICROPP3_MIXED;
  const bool implicit = ctan_mode_ == MICROPP3_CTAN_IMPLICIT;
  slots_.resize(n);
  for (int s = old; s < n; ++s) {
    Slot &w = slots_[s];
    w.u = dalloc<double>(nd, "u");
    w.du = dalloc<double>(nd, "du");
    w.b = dalloc<double>(nd, "b");
    w.be = dalloc<double>((size_t)24 * mesh_.nelem, "element residuals");
    w.vars_aux = dalloc<double>(nv, "vars_new_aux");
    w.red = dalloc<double>((size_t)nblocks * kRedStride, "partials");
    w.ticket = dalloc<unsigned int>(1, "ticket");
    w.cg = dalloc<CgState>(1, "cg state");
    w.out = dalloc<InstOut>(1, "out");
    if (fp64) {
      w.r = dalloc<double>(nd, "r");
      w.z = dalloc<double>(nd, "z");
      w.p = dalloc<double>(nd, "p");
      w.Ap = dalloc<double>(nd, "Ap");
      w.kinv = dalloc<double>(nd, "kinv");
      w.vals = dalloc<double>((size_t)kEllPerNode * mesh_.np, "ELL values");
    }
    if (mixed || implicit) {
      w.vals32 = dalloc<float>((size_t)kEllPerNode * mesh_.np, "ELL values (FP32)");
      w.kinv32 = dalloc<float>(nd, "kinv32");
      if (gather32_) w.gpd = dalloc<float>((size_t)64 * mesh_.nelem, "Gauss-point tangent terms");
    }
    if (mixed) {
      w.r32 = dalloc<float>(nd, "r32");
      w.z32 = dalloc<float>(nd, "z32");
      w.p32 = dalloc<float>(nd, "p32");
      w.Ap32 = dalloc<float>(nd, "Ap32");
      w.du32 = dalloc<float>(nd, "du32");
    }
    if (implicit) {
      const size_t n6 = (size_t)18 * mesh_.np;  // six right-hand sides, component-major
      w.X6h = dalloc<float>(n6, "X6 (hi)");
      w.X6l = dalloc<float>(n6, "X6 (lo)");
      w.F6h = dalloc<float>(n6, "F6 (hi)");
      w.F6l = dalloc<float>(n6, "F6 (lo)");
      w.R6 = dalloc<float>(n6, "R6");
      w.Z6 = dalloc<float>(n6, "Z6");
      w.P6 = dalloc<float>(n6, "P6");
      w.AP6 = dalloc<float>(n6, "AP6");
      w.D6 = dalloc<float>(n6, "D6");
      w.cg6 = dalloc<Cg6State>(1, "cg6 state");
    }
    if (mg_) {
      // level 0: the residual / prolonged iterate (6 right-hand sides component-major, or 1 node-interleaved);
      // levels >= 1: the Galerkin operator, its inverse diagonal and four vectors of 6 right-hand sides
      MgInst h{};
      auto buf = [&](size_t n, const char *what) {
        float *p = dalloc<float>(n, what);
        w.mg_bufs.push_back(p);
        return p;
      };
      h.lv[0].t = buf((size_t)18 * mesh_.np, "multigrid level-0 residual");
      if (mg_half_) {
        h.vals16 = dalloc<unsigned short>((size_t)kEllPerNode * mesh_.np, "multigrid FP16 fine operator");
        w.mg_bufs16.push_back(h.vals16);
        h.scale16 = mg_scale16_;
        h.inv16 = 1.0f / mg_scale16_;
      }
      h.lv[0].kinv = buf((size_t)3 * mesh_.np, "multigrid level-0 smoother diagonal");
      {
        const MeshDev &c = mg_mesh_[1];  // the first product has the largest intermediates
        h.mid1 = buf((size_t)kEllPerNode * grid_of(c.nx, mesh_.ny, mesh_.nz).np, "multigrid intermediate operator");
        h.mid2 = buf((size_t)kEllPerNode * grid_of(c.nx, c.ny, mesh_.nz).np, "multigrid intermediate operator");
      }
      for (size_t l = 1; l < mg_mesh_.size(); ++l) {
        const size_t np = mg_mesh_[l].np;
        h.lv[l].vals = buf((size_t)kEllPerNode * np, "multigrid operator");
        h.lv[l].kinv = buf((size_t)3 * np, "multigrid diagonal");
        h.lv[l].b = buf((size_t)18 * np, "multigrid vector");
        h.lv[l].x = buf((size_t)18 * np, "multigrid vector");
        h.lv[l].y = buf((size_t)18 * np, "multigrid vector");
        h.lv[l].t = buf((size_t)18 * np, "multigrid vector");
      }
      w.mg = dalloc<MgInst>(1, "multigrid hierarchy");
      check(cudaMemcpy(w.mg, &h, sizeof(MgInst), cudaMemcpyHostToDevice), "multigrid hierarchy upload");
    }
    check(cudaMemsetAsync(w.ticket, 0, sizeof(unsigned int), stream_), "ticket");
    check(cudaMemsetAsync(w.out, 0, sizeof(InstOut), stream_), "out");
  }
  clear_graphs();  // the captured chunks hold the instance and list pointers
  dfree(d_insts_);
  d_insts_ = dalloc<Inst>(n, "insts");
  if (eta_cap_ < n) {
    dfree(d_eta_);
    if (h_eta_) cudaFreeHost(h_eta_);
    h_eta_ = nullptr;
    d_eta_ = dalloc<double>(n, "CG tolerances");
    check(cudaMallocHost((void **)&h_eta_, n * sizeof(double)), "pinned CG tolerances");
    eta_cap_ = n;
  }
  if (h_out_) cudaFreeHost(h_out_);
  check(cudaMallocHost((void **)&h_out_, n * sizeof(InstOut)), "pinned out");
  h_insts_.assign(n, Inst{});
  for (int s = 0; s < n; ++s) {
    const Slot &w = slots_[s];
    Inst &I = h_insts_[s];
    I.u = w.u; I.du = w.du; I.b = w.b; I.r = w.r; I.z = w.z; I.p = w.p; I.Ap = w.Ap; I.kinv = w.kinv;
    I.vals = w.vals; I.be = w.be; I.red = w.red; I.ticket = w.ticket; I.cg = w.cg; I.out = w.out;
    I.vals32 = w.vals32; I.kinv32 = w.kinv32; I.r32 = w.r32; I.z32 = w.z32; I.p32 = w.p32; I.Ap32 = w.Ap32;
    I.du32 = w.du32;
    I.X6h = w.X6h; I.X6l = w.X6l; I.F6h = w.F6h; I.F6l = w.F6l; I.R6 = w.R6; I.Z6 = w.Z6; I.P6 = w.P6; I.AP6 = w.AP6; I.D6 = w.D6; I.cg6 = w.cg6;
    I.gpd = w.gpd;
    I.mg = w.mg;
    I.vars_old = nullptr;
    I.vars_new = w.vars_aux;
  }
  if (list_cap_ < n) {
    dfree(d_list_);
    d_list_ = dalloc<int>(n, "list");
    list_cap_ = n;
  }
}

void Engine::free_slots() {
  for (auto &w : slots_) {
    for (double *p : {w.u, w.du, w.b, w.r, w.z, w.p, w.Ap, w.kinv, w.vals, w.be, w.vars_aux, w.red}) dfree(p);
    for (float *p : {w.vals32, w.kinv32, w.r32, w.z32, w.p32, w.Ap32, w.du32, w.R6, w.Z6, w.P6, w.AP6, w.D6, w.gpd,
                     w.X6h, w.X6l, w.F6h, w.F6l})
      dfree(p);
    for (float *p : w.mg_bufs) dfree(p);
    w.mg_bufs.clear();
    for (unsigned short *p : w.mg_bufs16) dfree(p);
    w.mg_bufs16.clear();
    dfree(w.mg);
    dfree(w.ticket);
    dfree(w.cg);
    dfree(w.cg6);
    dfree(w.out);
  }
  slots_.clear();
  dfree(d_insts_);
  d_insts_ = nullptr;
  dfree(d_list_);
  d_list_ = nullptr;
  list_cap_ = 0;
  if (h_out_) cudaFreeHost(h_out_);
  h_out_ = nullptr;
}

void Engine::upload_insts() {
  check(cudaMemcpyAsync(d_insts_, h_insts_.data(), h_insts_.size() * sizeof(Inst), cudaMemcpyHostToDevice, stream_),
        "insts upload");
}

void Engine::upload_list(const std::vector<int> &slots) {
  check(cudaMemcpyAsync(d_list_, slots.data(), slots.size() * sizeof(int), cudaMemcpyHostToDevice, stream_),
        "list upload");
  // The host vector may change right after; wait for the copy of pageable memory to be consumed.
  check(cudaStreamSynchronize(stream_), "list sync");
}

void Engine::download_out() {
  for (size_t s = 0; s < slots_.size(); ++s)
    check(cudaMemcpyAsync(&h_out_[s], slots_[s].out, sizeof(InstOut), cudaMemcpyDeviceToHost, stream_), "out");
  sync();
}

double Engine::listed_cg_its(const std::vector<int> &slots) {
  download_out();
  double its = 0.0;
  for (int s : slots) its += h_out_[s].cg_its;
  return its;
}

void Engine::sync() { check(cudaStreamSynchronize(stream_), "stream synchronize"); }

// A chunk of CG iterations (`body` launches them on stream_): replayed from a CUDA graph captured the first
// time this (solver, batch size) pair runs, or launched directly while per-kernel timing is on or graphs are
// off.  The kernels read the instance list and the CG states from device memory, so one capture serves every
// later solve with the same number of listed instances.
void Engine::run_chunk(int kind, int n, const std::function<void()> &body) {
  const bool timing = t_spmv_.enabled || t_update_.enabled || t_spmv6_.enabled || t_upd6_.enabled || t_mg1_.enabled;
  if (!graphs_ || timing) {
    body();
    return;
  }
  const long key = (long)kind * 1000000L + n;
  auto it = graph_cache_.find(key);
  if (it == graph_cache_.end()) {
    cudaGraph_t g = nullptr;
    check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "graph capture");
    try {
      body();
    } catch (...) {
      cudaStreamEndCapture(stream_, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    check(cudaStreamEndCapture(stream_, &g), "graph capture end");
    cudaGraphExec_t ex = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    check(e, "graph instantiate");
    it = graph_cache_.emplace(key, ex).first;
  }
  check(cudaGraphLaunch(it->second, stream_), "graph launch");
}

// Autotuner of the FP32 SpMV block sizes.  The first time a (kernel, RVE size, batch size) runs, each block
// size is timed on the live data right after the CG set-up (3 launches each, CUDA events on the stream; an
// SpMV launch is idempotent: same p in, same Ap and alpha out) and the fastest is kept for the process.
namespace {
std::mutex g_tune_mutex;
std::map<std::tuple<int, int, int>, int> g_tuned;
}  // namespace

int Engine::tuned_block(int kind, int nlist) {
  const auto key = std::make_tuple(kind, mesh_.nn, nlist);
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) return it->second;
  }
  if (!tune_ev_[0]) {
    check(cudaEventCreate(&tune_ev_[0]), "tune event");
    check(cudaEventCreate(&tune_ev_[1]), "tune event");
  }
  int best = 128;
  float best_ms = 0.0f;
  for (int block : {64, 128, 256}) {
    auto launch = [&] {
      launches_ += 1;
      if (kind == 0)
        check_launch(mgb_launch_cg32_spmv(&mesh_, d_insts_, d_list_, nlist, block, stream_), "tune spmv");
      else
        check_launch(mgb_launch_cg6_spmv(&mesh_, d_insts_, d_list_, nlist, block, stream_), "tune spmv6");
    };
    launch();  // warm
    check(cudaEventRecord(tune_ev_[0], stream_), "tune event");
    for (int r = 0; r < 3; ++r) launch();
    check(cudaEventRecord(tune_ev_[1], stream_), "tune event");
    check(cudaEventSynchronize(tune_ev_[1]), "tune sync");
    float ms = 0.0f;
    check(cudaEventElapsedTime(&ms, tune_ev_[0], tune_ev_[1]), "tune elapsed");
    if (block == 64 || ms < best_ms) {
      best_ms = ms;
      best = block;
    }
  }
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tuned[key] = best;
  return best;
}

int Engine::known_block(int kind, int nlist) const {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  auto it = g_tuned.find(std::make_tuple(kind, mesh_.nn, nlist));
  return it == g_tuned.end() ? 0 : it->second;
}

bool Engine::timing_on() const {
  return t_spmv_.enabled || t_update_.enabled || t_spmv6_.enabled || t_upd6_.enabled || t_mg1_.enabled ||
         t_asm_.enabled || t_res_.enabled;
}

void Engine::clear_graphs() {
  if ((!graph_cache_.empty() || !newton_graphs_.empty()) && stream_) cudaStreamSynchronize(stream_);
  for (auto &kv : graph_cache_) cudaGraphExecDestroy(kv.second);
  graph_cache_.clear();
  for (auto &kv : newton_graphs_) cudaGraphExecDestroy(kv.second.exec);
  newton_graphs_.clear();
}

void Engine::set_graphs(bool on) {
  if (!on) clear_graphs();
  graphs_ = on;
}

void Engine::timer_begin(KernelTimer &t, double bytes) {
  if (!t.enabled) return;
  if (t.used == t.pool.size()) {
    cudaEvent_t a, b;
    check(cudaEventCreate(&a), "timer event");
    check(cudaEventCreate(&b), "timer event");
    t.pool.emplace_back(a, b);
  }
  check(cudaEventRecord(t.pool[t.used].first, stream_), "timer record");
  t.pending_bytes += bytes;
}

void Engine::timer_end(KernelTimer &t) {
  if (!t.enabled) return;
  check(cudaEventRecord(t.pool[t.used].second, stream_), "timer record");
  t.used++;
  t.launches++;
  if (t.used >= 512) {  // fold the finished pairs into the totals
    check(cudaEventSynchronize(t.pool[t.used - 1].second), "timer sync");
    for (size_t i = 0; i < t.used; ++i) {
      float ms = 0;
      check(cudaEventElapsedTime(&ms, t.pool[i].first, t.pool[i].second), "timer elapsed");
      t.ms += ms;
    }
    t.used = 0;
    t.bytes += t.pending_bytes;
    t.pending_bytes = 0;
  }
}

void Engine::set_kernel_timing(bool on) {
  sync();
  for (KernelTimer *t : {&t_spmv_, &t_update_, &t_asm_, &t_res_, &t_spmv6_, &t_upd6_, &t_mg1_, &t_mg6_, &t_mgc_, &t_rap_,
                          &t_tan_}) {
    t->enabled = on;
    t->used = 0;
    t->launches = 0;
    t->ms = t->bytes = t->pending_bytes = 0.0;
  }
}

bool Engine::kernel_stats(const std::string &family, long *launches, double *ms, double *bytes) {
  KernelTimer *t = nullptr;
  if (family == "spmv") t = &t_spmv_;
  else if (family == "cg_update") t = &t_update_;
  else if (family == "assembly") t = &t_asm_;
  else if (family == "mg_rap") t = &t_rap_;
  else if (family == "tangent") t = &t_tan_;
  else if (family == "residual") t = &t_res_;
  else if (family == "spmv6") t = &t_spmv6_;
  else if (family == "cg6_update") t = &t_upd6_;
  else if (family == "mg") t = &t_mg1_;
  else if (family == "mg6") t = &t_mg6_;
  else if (family == "mg_coarse") t = &t_mgc_;
  if (!t) return false;
  sync();
  for (size_t i = 0; i < t->used; ++i) {
    float m = 0;
    check(cudaEventElapsedTime(&m, t->pool[i].first, t->pool[i].second), "timer elapsed");
    t->ms += m;
  }
  t->used = 0;
  t->bytes += t->pending_bytes;
  t->pending_bytes = 0;
  *launches = t->launches;
  *ms = t->ms;
  *bytes = t->bytes;
  return true;
}

// ------------------------------------------------------------------------------------------------
// Batched solver pieces

// assembly_rhs for the listed slots: out.norm and out.sig of each slot are valid afterwards.
void Engine::residual(const std::vector<int> &slots) {
  // Algorithmic bytes: u gathered once, history read once, b written once (element blocks stay in L2/HBM
  // scratch and are not counted).
  const double bytes = (double)slots.size() * (16.0 * nndim() + 8.0 * nvars());
  timer_begin(t_res_, bytes);
  launches_ += 2;
  check_launch(mgb_launch_residual(&mesh_, &mats_, d_etype_, d_dsh_, d_insts_, d_list_, (int)slots.size(),
                                   precision_ == MICROPP3_FP64 ? 1 : (gather32_ ? 2 : 0), stream_),
               "residual");
  timer_end(t_res_);
}

// ell_solve_cgpd for the listed slots (b -> du); out.cg_its of each slot is valid afterwards.
void Engine::cg_solve(const std::vector<int> &slots) {
  const int n = (int)slots.size();
  for (int s : slots) {
    CgState c{};
    c.min_err = cg_abs_tol_;
    c.rel_err = cg_rel_tol_;
    c.max_its = cg_max_its_;
    check(cudaMemcpyAsync(slots_[s].cg, &c, sizeof(CgState), cudaMemcpyHostToDevice, stream_), "cg init");
  }
  launches_ += 2;
  check_launch(mgb_launch_cg_setup(&mesh_, d_insts_, d_list_, n, stream_), "cg setup");
  // Algorithmic bytes per iteration and RVE (spmv): 81 values per row + x read + y written.
  const double nrow = (double)nndim();
  // Algorithmic bytes of one iteration of one instance.  SpMV: 81 values per row, x read, y written; update:
  // read p, Ap, r, x, kinv, write x, r, z; p-update: read z, p, write p.  They are credited after the solve
  // for the iterations each instance ran (an instance that has stopped skips the batch's later launches).
  const double spmv_bytes = nrow * (81.0 * 8 + 2.0 * 8);
  const double upd_bytes = nrow * 11.0 * 8;
  const int chunk = (mesh_.nn > 200000) ? 8 : 32;
  int done_its = 0;
  while (done_its <= cg_max_its_) {
    run_chunk(0, n, [&] {
      for (int it = 0; it < chunk; ++it) {
        if (it == chunk - 1) check(cudaMemsetAsync(d_count_, 0, sizeof(unsigned int), stream_), "count reset");
        timer_begin(t_spmv_, 0.0);
        check_launch(mgb_launch_cg_spmv(&mesh_, d_insts_, d_list_, n, stream_), "cg spmv");
        timer_end(t_spmv_);
        timer_begin(t_update_, 0.0);
        check_launch(mgb_launch_cg_update(&mesh_, d_insts_, d_list_, n, stream_), "cg update");
        check_launch(mgb_launch_cg_pupdate(&mesh_, d_insts_, d_list_, n, d_count_, stream_), "cg p-update");
        timer_end(t_update_);
      }
    });
    launches_ += 3 * chunk;
    done_its += chunk;
    check(cudaMemcpyAsync(h_count_, d_count_, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream_), "count");
    sync();
    if (*h_count_ == 0) break;
  }
  if (t_spmv_.enabled) {
    const double its = listed_cg_its(slots);
    timer_add_bytes(t_spmv_, its * spmv_bytes);
    timer_add_bytes(t_update_, its * upd_bytes);
  }
}

// The mixed form's CG: FP32 values and vectors, FP64 dot products, same iteration and stop rule, with a
// relative tolerance per slot.  use_mg: multigrid-preconditioned (when the handle has multigrid), capped at
// kMgMaxIts iterations; otherwise Jacobi with cg_max_its.
void Engine::cg_solve32(const std::vector<int> &slots, const std::vector<double> &rel_tols, bool use_mg) {
  const int n = (int)slots.size();
  const bool mg = mg_ && use_mg;
  for (int a = 0; a < n; ++a) {
    CgState c{};
    c.min_err = cg_abs_tol_;
    c.rel_err = rel_tols[a];
    c.max_its = mg ? std::min(cg_max_its_, kMgMaxIts) : cg_max_its_;
    check(cudaMemcpyAsync(slots_[slots[a]].cg, &c, sizeof(CgState), cudaMemcpyHostToDevice, stream_), "cg init");
  }
  launches_ += 1;
  check_launch(mgb_launch_cg32_setup(&mesh_, d_insts_, d_list_, n, mg ? 1 : 0, stream_), "cg32 setup");
  if (mg) mg_vcycle(1, n, true, 128);
  const int block = tuned_block(0, n);
  const double nrow = (double)nndim();
  const double spmv_bytes = nrow * (81.0 * 4 + 2.0 * 4);  // per iteration and instance, as in cg_solve
  const double upd_bytes = nrow * 11.0 * 4;
  const int chunk = mg ? kMgChunk : (mesh_.nn > 200000) ? 8 : 32;
  int done_its = 0;
  while (done_its <= cg_max_its_) {
    run_chunk(mg ? 1 : 3, n, [&] {
      for (int it = 0; it < chunk; ++it) {
        if (it == chunk - 1) check(cudaMemsetAsync(d_count_, 0, sizeof(unsigned int), stream_), "count reset");
        timer_begin(t_spmv_, 0.0);
        check_launch(mgb_launch_cg32_spmv(&mesh_, d_insts_, d_list_, n, block, stream_), "cg32 spmv");
        timer_end(t_spmv_);
        timer_begin(t_update_, 0.0);
        check_launch(mgb_launch_cg32_update(&mesh_, d_insts_, d_list_, n, mg ? 1 : 0, stream_), "cg32 update");
        timer_end(t_update_);
        if (mg) mg_vcycle(1, n, false, 128);
        timer_begin(t_update_, 0.0);
        check_launch(mgb_launch_cg32_pupdate(&mesh_, d_insts_, d_list_, n, d_count_, stream_), "cg32 p-update");
        timer_end(t_update_);
      }
    });
    launches_ += 3 * chunk;
    done_its += chunk;
    check(cudaMemcpyAsync(h_count_, d_count_, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream_), "count");
    sync();
    if (*h_count_ == 0) break;
  }
  if (t_spmv_.enabled) {
    const double its = listed_cg_its(slots);
    timer_add_bytes(t_spmv_, its * spmv_bytes);
    timer_add_bytes(t_update_, its * upd_bytes);
    if (mg) {
      timer_add_bytes(t_mg1_, (its + n) * mg_fine_bytes(1));
      timer_add_bytes(t_mgc_, (its + n) * mg_coarse_bytes(1));
    }
  }
}

// Algorithmic bytes: the values written once, plus u and the history read once per element (colouring) or
// the Gauss-point tangent terms (8 floats per Gauss point) read once (gather).
void Engine::assemble32(int nlist) {
  if (gather32_) {
    timer_begin(t_asm_, (double)nlist * (4.0 * kEllPerNode * mesh_.np + 4.0 * 64.0 * mesh_.nelem));
    launches_ += 1;
    check_launch(mgb_launch_assembly_gather32(&mesh_, &mats_, d_etype_, d_k0g32_, d_ke32_, d_dsh32_, d_insts_,
                                              d_list_, nlist, kMgOmega, kMgSafe, mg_ ? 1 : 0, stream_),
                 "assembly (FP32 gather)");
  } else {
    timer_begin(t_asm_, (double)nlist * (4.0 * kEllPerNode * mesh_.np + 8.0 * nndim() + 8.0 * nvars()));
    launches_ += 9;
    check_launch(mgb_launch_assembly32(&mesh_, &mats_, d_etype_, d_dsh_, d_ke32_, d_insts_, d_list_, nlist, stream_),
                 "assembly (FP32)");
  }
  timer_end(t_asm_);
  if (mg_) mg_rap(nlist, gather32_);
}

// Galerkin operators P^T A P of every coarse level, finest first, each as three 1-D steps (x, y, z) through
// the intermediate operators mid1 and mid2, and the safeguarded smoother diagonal of every level (of level 0 only
// when the assembly did not write it: sdiag0_done).  Algorithmic bytes: each step reads its input operator and
// writes its output once; each diagonal pass reads its operator.
void Engine::mg_rap(int nlist, bool sdiag0_done) {
  double bytes = 0.0;
  for (size_t l = 0; l < mg_mesh_.size(); ++l) {
    const MeshDev &f = mg_mesh_[l];
    if (l > 0 || !sdiag0_done) bytes += 4.0 * kEllPerNode * (double)f.np;
    if (l + 1 < mg_mesh_.size()) {
      const MeshDev &c = mg_mesh_[l + 1];
      const double n1 = grid_of(c.nx, f.ny, f.nz).np, n2 = grid_of(c.nx, c.ny, f.nz).np;
      bytes += 4.0 * kEllPerNode * ((double)f.np + 2.0 * n1 + 2.0 * n2 + (double)c.np);
    }
  }
  timer_begin(t_rap_, nlist * bytes);
  if (!sdiag0_done) {
    launches_ += 1;
    check_launch(mgb_launch_mg_sdiag(&mg_mesh_[0], d_insts_, d_list_, nlist, 0, kMgOmega, kMgSafe, stream_),
                 "multigrid smoother diagonal");
  }
  if (mg_half_) {
    launches_ += 1;
    check_launch(mgb_launch_mg_half0(&mg_mesh_[0], d_insts_, d_list_, nlist, stream_), "multigrid FP16 operator");
  }
  for (size_t l = 0; l + 1 < mg_mesh_.size(); ++l) {
    const MeshDev &f = mg_mesh_[l], &c = mg_mesh_[l + 1];
    const MeshDev m1 = grid_of(c.nx, f.ny, f.nz), m2 = grid_of(c.nx, c.ny, f.nz);
    const int lf = (int)l;
    launches_ += 4;
    check_launch(mgb_launch_mg_rap1(&f, &m1, d_insts_, d_list_, nlist, lf, 0, 0, 1, stream_), "multigrid product x");
    check_launch(mgb_launch_mg_rap1(&m1, &m2, d_insts_, d_list_, nlist, lf, 1, 1, 2, stream_), "multigrid product y");
    check_launch(mgb_launch_mg_rap1(&m2, &c, d_insts_, d_list_, nlist, lf, 2, 2, 3, stream_), "multigrid product z");
    check_launch(mgb_launch_mg_sdiag(&c, d_insts_, d_list_, nlist, lf + 1, kMgOmega, kMgSafe, stream_),
                 "multigrid smoother diagonal");
  }
  timer_end(t_rap_);
}

// Algorithmic bytes of one V-cycle per instance.  Level 0: the residual and the post-smoother, each 81 values
// per row, and per right-hand side x (or t) read, b read, the result written.  The rest: on each coarse level
// above the coarsest two operator passes and about eight vector passes; on the coarsest level the Jacobi
// sweeps (one operator pass and three vector passes each); the level-0 restriction and prolongation (three
// vector passes).
double Engine::mg_fine_bytes(int nr) const {
  const double value_bytes = mg_half_ ? 2.0 : 4.0;  // FP16 copy or FP32 operator
  return 2.0 * (double)nndim() * (81.0 * value_bytes + 3.0 * nr * 4);
}

double Engine::mg_coarse_bytes(int nr) const {
  const size_t L = mg_mesh_.size();
  double b = 3.0 * 4.0 * nr * (double)nndim();
  for (size_t l = 1; l < L; ++l) {
    const double nn = mg_mesh_[l].nn, vec = 4.0 * 3.0 * nr * nn, op = 4.0 * kEllPerNode * nn;
    if (l + 1 < L)
      b += 2.0 * op + 8.0 * vec;
    else
      b += (2.0 * kMgCoarsePairs) * (op + 3.0 * vec);
  }
  return b;
}

// One V-cycle of the nr-RHS CG of the listed instances (their level-0 iterate x0 = D^-1 r is already
// written), ending with the level-0 post-smoother that forms z and the CG scalars.  block: threads per block of
// the 6-RHS level-0 residual and post-smoother (the tuned block of the 6-RHS SpMV, whose access pattern they
// share).
void Engine::mg_vcycle(int nr, int nlist, bool setup, int block) {
  const int L = (int)mg_mesh_.size();
  KernelTimer &fine = (nr == 1) ? t_mg1_ : t_mg6_;
  for (int l = 0; l + 1 < L; ++l) {
    if (l == 0) timer_begin(fine, 0.0);
    check_launch(mgb_launch_mg_resid(&mg_mesh_[l], d_insts_, d_list_, nlist, nr, l, block, mg_half_ ? 1 : 0,
                                     stream_),
                 "multigrid residual");
    if (l == 0) {
      timer_end(fine);
      timer_begin(t_mgc_, 0.0);
    }
    check_launch(mgb_launch_mg_restrict(&mg_mesh_[l], &mg_mesh_[l + 1], d_insts_, d_list_, nlist, nr, l, 1.0f,
                                        stream_),
                 "multigrid restriction");
  }
  const bool one_block = mg_mesh_[L - 1].nn <= kMgCoarseNodes;
  if (one_block) {
    check_launch(mgb_launch_mg_coarse_sweeps(&mg_mesh_[L - 1], d_insts_, d_list_, nlist, nr, L - 1, kMgCoarsePairs,
                                             1.0f, stream_),
                 "multigrid coarse sweeps");
  } else {
    for (int k = 0; k < kMgCoarsePairs; ++k) {
      check_launch(mgb_launch_mg_jacobi(&mg_mesh_[L - 1], d_insts_, d_list_, nlist, nr, L - 1, 0, 1, 1.0f, stream_),
                   "multigrid coarse sweep");
      check_launch(mgb_launch_mg_jacobi(&mg_mesh_[L - 1], d_insts_, d_list_, nlist, nr, L - 1, 1, 0, 1.0f, stream_),
                   "multigrid coarse sweep");
    }
  }
  for (int l = L - 2; l >= 0; --l) {
    check_launch(mgb_launch_mg_prolong(&mg_mesh_[l], &mg_mesh_[l + 1], d_insts_, d_list_, nlist, nr, l, stream_),
                 "multigrid prolongation");
    if (l > 0)
      check_launch(mgb_launch_mg_jacobi(&mg_mesh_[l], d_insts_, d_list_, nlist, nr, l, 2, 0, 1.0f, stream_),
                   "multigrid post-smoother");
  }
  timer_end(t_mgc_);
  timer_begin(fine, 0.0);
  check_launch(mgb_launch_mg_post0(&mesh_, d_insts_, d_list_, nlist, nr, 1.0f, setup ? 1 : 0, block, mg_half_ ? 1 : 0,
                                   stream_),
               "multigrid level-0 post-smoother");
  timer_end(fine);
  launches_ += 2 * (L - 1) + (one_block ? 1 : 2 * kMgCoarsePairs) + (L - 1) + (L - 2) + 1;
}

// Implicit ctan of the listed slots at their current u with their vars_old: assemble the FP32 tangent, form
// the six right-hand sides, solve with refined FP32 CG sweeps, average.  out.ctan of each slot is valid
// afterwards.  Returns the CG iterations each slot spent.
std::vector<int> Engine::tangent_solve(const std::vector<int> &slots, bool use_mg) {
  const int n = (int)slots.size();
  const bool mg = mg_ && use_mg;
  // The gather assembly (elastic and damage phases) gives a symmetric tangent: ctan in the energy form.
  const bool energy = gather32_;
  const double sweep_rel = energy ? kTangentSweepRelEnergy : kTangentSweepRel;
  const double tangent_tol = energy ? kTangentTolEnergy : kTangentTol;
  std::vector<char> mg_capped(n, 0);  // a multigrid sweep of the slot reached kMgMaxIts
  std::vector<int> its(n, 0);
  upload_insts();
  upload_list(slots);
  assemble32(n);
  launches_ += 2;
  timer_begin(t_tan_, 0.0);
  check_launch(mgb_launch_t6_rhs(&mesh_, d_near_, nnear_, d_insts_, d_list_, n, stream_), "tangent rhs");
  timer_end(t_tan_);
  const double nrow = (double)nndim();
  // Per iteration and instance: SpMV 81 values per row, 6 x read and 6 y written; update: read P, AP, R, D,
  // write D, R, Z; p-update: read Z, P, write P (per right-hand side).  Credited per instance iteration.
  const double spmv_bytes = nrow * (81.0 * 4 + 2.0 * 6 * 4);
  const double upd6_bytes = nrow * 6.0 * 10.0 * 4;
  const int chunk = mg ? kMgChunk : (mesh_.nn > 200000) ? 8 : 32;
  std::vector<int> live = slots;
  std::vector<int> live_idx(n);
  for (int i = 0; i < n; ++i) live_idx[i] = i;
  for (int sweep = 0; sweep < kTangentSweeps && !live.empty(); ++sweep) {
    for (int s : live) {
      Cg6State c{};
      c.min_err = 0.0;
      c.rel_err = sweep_rel;
      c.max_its = mg ? std::min(cg_max_its_, kMgMaxIts) : cg_max_its_;
      check(cudaMemcpyAsync(slots_[s].cg6, &c, sizeof(Cg6State), cudaMemcpyHostToDevice, stream_), "cg6 init");
    }
    if (sweep > 0) upload_list(live);
    launches_ += 1;
    timer_begin(t_tan_, 0.0);
    check_launch(mgb_launch_t6_residual(&mesh_, d_insts_, d_list_, (int)live.size(), sweep == 0 ? 1 : 0,
                                        mg ? 1 : 0, stream_),
                 "tangent residual");
    timer_end(t_tan_);
    download_out();
    std::vector<int> next, next_idx;
    for (size_t a = 0; a < live.size(); ++a) {
      const InstOut &o = h_out_[live[a]];
      bool ok = true;
      for (int r = 0; r < 6; ++r) ok &= o.res6[r] <= tangent_tol * o.f6[r];
      if (!ok && std::isfinite(o.res6[0])) {
        next.push_back(live[a]);
        next_idx.push_back(live_idx[a]);
      }
    }
    if (next.size() != live.size()) {
      // Converged slots leave; the CG states of the others were initialised by the residual kernel.
      live = next;
      live_idx = next_idx;
      if (live.empty()) break;
      upload_list(live);
      for (int s : live) {
        Cg6State c{};
        c.min_err = 0.0;
        c.rel_err = sweep_rel;
        c.max_its = mg ? std::min(cg_max_its_, kMgMaxIts) : cg_max_its_;
        check(cudaMemcpyAsync(slots_[s].cg6, &c, sizeof(Cg6State), cudaMemcpyHostToDevice, stream_), "cg6 init");
      }
      launches_ += 1;
      timer_begin(t_tan_, 0.0);
      check_launch(mgb_launch_t6_residual(&mesh_, d_insts_, d_list_, (int)live.size(), sweep == 0 ? 1 : 0,
                                          mg ? 1 : 0, stream_),
                   "tangent residual");
      timer_end(t_tan_);
    }
    const int nl = (int)live.size();
    const int block = tuned_block(1, nl);
    if (mg) mg_vcycle(6, nl, true, block);
    int done_its = 0;
    while (done_its <= cg_max_its_) {
      run_chunk(mg ? 2 : 4, nl, [&] {
        for (int it = 0; it < chunk; ++it) {
          if (it == chunk - 1) check(cudaMemsetAsync(d_count_, 0, sizeof(unsigned int), stream_), "count reset");
          timer_begin(t_spmv6_, 0.0);
          check_launch(mgb_launch_cg6_spmv(&mesh_, d_insts_, d_list_, nl, block, stream_), "cg6 spmv");
          timer_end(t_spmv6_);
          timer_begin(t_upd6_, 0.0);
          check_launch(mgb_launch_cg6_update(&mesh_, d_insts_, d_list_, nl, mg ? 1 : 0, stream_), "cg6 update");
          timer_end(t_upd6_);
          if (mg) mg_vcycle(6, nl, false, block);
          timer_begin(t_upd6_, 0.0);
          check_launch(mgb_launch_cg6_pupdate(&mesh_, d_insts_, d_list_, nl, d_count_, stream_), "cg6 p-update");
          timer_end(t_upd6_);
        }
      });
      launches_ += 3 * chunk;
      done_its += chunk;
      check(cudaMemcpyAsync(h_count_, d_count_, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream_), "count");
      sync();
      if (*h_count_ == 0) break;
    }
    launches_ += 1;
    timer_begin(t_tan_, 0.0);
    check_launch(mgb_launch_t6_accumulate(&mesh_, d_insts_, d_list_, nl, stream_), "tangent accumulate");
    timer_end(t_tan_);
    download_out();
    for (size_t a = 0; a < live.size(); ++a) {
      its[live_idx[a]] += h_out_[live[a]].cg6_its;
      total_cg_its_ += h_out_[live[a]].cg6_its;
      timer_add_bytes(t_spmv6_, h_out_[live[a]].cg6_its * spmv_bytes);
      timer_add_bytes(t_upd6_, h_out_[live[a]].cg6_its * upd6_bytes);
      if (mg && h_out_[live[a]].cg6_its >= std::min(cg_max_its_, kMgMaxIts)) mg_capped[live_idx[a]] = 1;
      if (mg) {
        timer_add_bytes(t_mg6_, (h_out_[live[a]].cg6_its + 1) * mg_fine_bytes(6));
        timer_add_bytes(t_mgc_, (h_out_[live[a]].cg6_its + 1) * mg_coarse_bytes(6));
      }
    }
  }
  upload_list(slots);
  launches_ += 1;
  if (gather32_) {
    timer_begin(t_tan_, 0.0);
    check_launch(mgb_launch_ctan_energy(&mesh_, &mats_, d_etype_, d_dsh32_, d_insts_, d_list_, n, stream_),
                 "ctan (energy form)");
    timer_end(t_tan_);
  } else {
    timer_begin(t_tan_, 0.0);
    check_launch(mgb_launch_ctan_avg(&mesh_, &mats_, d_etype_, d_dsh_, d_insts_, d_list_, n, stream_), "ctan average");
    timer_end(t_tan_);
  }
  download_out();
  if (mg) {
    // Slots whose multigrid sweeps reached the iteration cap are solved again with Jacobi, from the start.
    std::vector<int> redo, redo_idx;
    for (int i = 0; i < n; ++i)
      if (mg_capped[i]) {
        redo.push_back(slots[i]);
        redo_idx.push_back(i);
      }
    if (!redo.empty()) {
      const std::vector<int> its2 = tangent_solve(redo, false);
      for (size_t a = 0; a < redo.size(); ++a) its[redo_idx[a]] += its2[a];
      upload_list(slots);
    }
  }
  return its;
}

// One Newton iteration of the mixed form with the multigrid for the nlist slots listed in d_list_, as one CUDA
// graph: the FP32 assembly with the multigrid operators, the CG start (tolerances from d_eta_), a WHILE node
// whose body runs a chunk of preconditioned CG iterations and then a kernel that continues the loop while some
// listed instance still iterates (at most min(cg_max_its, kMgMaxIts) / kMgChunk + 2 chunks), u += du and the
// residual.  The host's part of an iteration -- the tolerances before it, convergence, the line search and
// the Jacobi redo of a capped solve after it -- stays outside.  A graph is built the first time a batch size
// runs once the SpMV autotuner has picked that batch size's block (the autotuner times live launches, which a
// capture cannot hold) and is replayed afterwards: its kernels read the listed instances and the tolerances
// from device memory.
bool Engine::newton_graph(int nlist) {
  if (!newton_graphs_ok_ || known_block(0, nlist) == 0) return false;
  auto it = newton_graphs_.find(nlist);
  if (it == newton_graphs_.end()) {
    const int block = known_block(0, nlist);
    const int chunk = kMgChunk;
    const int max_its = std::min(cg_max_its_, kMgMaxIts);
    const unsigned cap = (unsigned)(max_its / chunk + 2);
    const std::vector<int> listed(nlist);  // residual() takes the count of the listed slots only
    auto capture = [&](cudaGraph_t into, const std::function<void()> &body) {
      if (into)
        check(cudaStreamBeginCaptureToGraph(stream_, into, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
              "graph capture");
      else
        check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "graph capture");
      cudaGraph_t out = nullptr;
      try {
        body();
      } catch (...) {
        cudaStreamEndCapture(stream_, &out);
        if (out && !into) cudaGraphDestroy(out);
        throw;
      }
      check(cudaStreamEndCapture(stream_, &out), "graph capture end");
      return out;
    };
    NewtonGraph ng;
    const long l0 = launches_;
    cudaGraph_t g = nullptr, prefix = nullptr, suffix = nullptr;
    try {
      prefix = capture(nullptr, [&] {
        assemble32(nlist);
        check_launch(mgb_launch_cg32_init(d_insts_, d_list_, nlist, d_eta_, cg_abs_tol_, max_its, stream_),
                     "cg32 init");
        check_launch(mgb_launch_zero_u32(d_chunks_, stream_), "chunk count");
        check_launch(mgb_launch_cg32_setup(&mesh_, d_insts_, d_list_, nlist, 1, stream_), "cg32 setup");
        mg_vcycle(1, nlist, true, 128);
      });
      launches_ += 3;
      suffix = capture(nullptr, [&] {
        check_launch(mgb_launch_add_du32(&mesh_, d_insts_, d_list_, nlist, stream_), "u += du");
        residual(listed);
      });
      launches_ += 1;
      ng.fixed_launches = launches_ - l0;
      check(cudaGraphCreate(&g, 0), "graph");
      cudaGraphNode_t n1 = nullptr, n2 = nullptr, n3 = nullptr;
      check(cudaGraphAddChildGraphNode(&n1, g, nullptr, 0, prefix), "graph prefix");
      cudaGraphConditionalHandle cond;
      check(cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault), "graph condition");
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = cond;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      check(cudaGraphAddNode(&n2, g, &n1, nullptr, 1, &cp), "graph loop");
      const long l1 = launches_;
      capture(cp.conditional.phGraph_out[0], [&] {
        for (int k = 0; k < chunk; ++k) {
          if (k == chunk - 1) check_launch(mgb_launch_zero_u32(d_count_, stream_), "count reset");
          check_launch(mgb_launch_cg32_spmv(&mesh_, d_insts_, d_list_, nlist, block, stream_), "cg32 spmv");
          check_launch(mgb_launch_cg32_update(&mesh_, d_insts_, d_list_, nlist, 1, stream_), "cg32 update");
          mg_vcycle(1, nlist, false, 128);
          check_launch(mgb_launch_cg32_pupdate(&mesh_, d_insts_, d_list_, nlist, d_count_, stream_),
                       "cg32 p-update");
        }
        check_launch(mgb_launch_cg_continue(cond, d_count_, d_chunks_, cap, stream_), "cg loop condition");
      });
      ng.chunk_launches = (launches_ - l1) + 3 * chunk + 2;
      check(cudaGraphAddChildGraphNode(&n3, g, &n2, 1, suffix), "graph suffix");
      check(cudaGraphInstantiate(&ng.exec, g, 0), "graph instantiate");
    } catch (const std::exception &) {
      // Graphs of this form are unavailable here (for instance no conditional nodes): run unfused from now on.
      for (cudaGraph_t x : {g, prefix, suffix})
        if (x) cudaGraphDestroy(x);
      cudaGetLastError();
      launches_ = l0;
      newton_graphs_ok_ = false;
      return false;
    }
    for (cudaGraph_t x : {g, prefix, suffix}) cudaGraphDestroy(x);
    launches_ = l0;
    it = newton_graphs_.emplace(nlist, ng).first;
  }
  check(cudaGraphLaunch(it->second.exec, stream_), "graph launch");
  check(cudaMemcpyAsync(h_chunks_, d_chunks_, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream_), "chunks");
  sync();
  launches_ += it->second.fixed_launches + (long)*h_chunks_ * it->second.chunk_launches;
  return true;
}

// newton_raphson (solve.cpp:28-82) for a batch: slot s solves for strains[i] with its h_insts_ vars_old.
// The per-slot state machine reproduces the reference loop exactly: a slot stops when its norm meets the
// absolute or relative tolerance (checked before each iteration while its < nr_max_its), or after
// nr_max_its iterations (then unconverged).  In the mixed form the Jacobian and its CG are FP32 while the
// residual that decides convergence stays FP64.
std::vector<NewtonResult> Engine::newton(const std::vector<int> &slots,
                                         const std::vector<std::array<double, 6>> &strains) {
  const int n = (int)slots.size();
  const bool mixed = precision_ == MICROPP3_MIXED;
  std::vector<NewtonResult> res(n);
  std::vector<double> norm0(n, 0.0), norm(n, 0.0);
  std::vector<char> done(n, 0);
  for (int i = 0; i < n; ++i) std::memcpy(h_insts_[slots[i]].strain, strains[i].data(), 6 * sizeof(double));
  upload_insts();
  upload_list(slots);
  launches_ += 1;
  check_launch(mgb_launch_set_bc(&mesh_, d_insts_, d_list_, n, stream_), "set_bc");
  residual(slots);
  download_out();
  for (int i = 0; i < n; ++i) norm0[i] = norm[i] = h_out_[slots[i]].norm;
  if (!predict_de_.empty()) {
    // Predictor (mixed form): |b0| stays the residual at u_n with the new boundary values, as in the reference,
    // so nr_rel_tol keeps its meaning; Newton then starts from u_n + deps . X (boundary values unchanged).
    for (int i = 0; i < n; ++i) {
      launches_ += 1;
      check_launch(mgb_launch_affine_add(&mesh_, slots_[slots[i]].u, predict_de_[i].data(), stream_), "predictor");
    }
    predict_de_.clear();
    launches_ += 1;
    check_launch(mgb_launch_set_bc(&mesh_, d_insts_, d_list_, n, stream_), "set_bc");
    residual(slots);
    download_out();
    for (int i = 0; i < n; ++i) norm[i] = h_out_[slots[i]].norm;
  }
  while (true) {
    std::vector<int> active;
    std::vector<int> idx;
    for (int i = 0; i < n; ++i) {
      if (done[i]) continue;
      if (!(res[i].its < nr_max_its_)) {
        done[i] = 1;
        continue;
      }
      if (norm[i] < nr_max_tol_ || norm[i] < norm0[i] * nr_rel_tol_) {
        res[i].converged = true;
        done[i] = 1;
        continue;
      }
      active.push_back(slots[i]);
      idx.push_back(i);
    }
    if (active.empty()) break;
    upload_list(active);
    const int na = (int)active.size();
    int bicg_its = 0;
    bool have_residual = false;
    bool a0_iteration = false;
    std::vector<int> mg_its(na, 0);  // iterations of multigrid solves redone with Jacobi
    // The mixed multigrid form runs the iteration's device work as one CUDA graph where it can (graphs on,
    // kernel timers off); otherwise kernel by kernel.
    const bool fused = mixed && mg_ && graphs_ && !timing_on() && newton_graphs_ok_ && known_block(0, na) > 0;
    if (mixed) {
      if (!fused) assemble32(na);
    } else if (use_A0_ && !exact_tangent_ && res[idx[0]].its < its_with_A0_) {
      // solve.cpp:55-66: this iteration solves with A0 (every active slot started this Newton together, so
      // they share the iteration count)
      for (int s : active) h_insts_[s].vals = d_A0_;
      upload_insts();
      a0_iteration = true;
    } else {
      timer_begin(t_asm_, (double)na * (8.0 * kEllPerNode * mesh_.np + 8.0 * nndim() + 8.0 * nvars()));
      launches_ += 9;
      if (exact_tangent_)  // load paths: the exact consistent tangent (quadratic Newton)
        check_launch(mgb_launch_assembly_dual(&mesh_, &mats_, d_etype_, d_dsh_, d_ke_, d_insts_, d_list_, na, stream_),
                     "assembly");
      else
        check_launch(mgb_launch_assembly(&mesh_, &mats_, d_etype_, d_dsh_, d_ke_, d_insts_, d_list_, na, stream_),
                     "assembly");
      timer_end(t_asm_);
    }
    launches_ += 1;
    if (mixed) {
      // Inexact Newton: the FP64-accurate residual corrects each FP32 solve, so a correction only needs to gain the
      // digits still missing to the Newton tolerance: eta = 0.05 * nr_rel_tol * |b0| / |b_k|, kept within
      // [max(cg_rel_tol, kFp32CgFloor), 0.1] (an FP32 CG cannot reduce its residual much below 1e-6).
      std::vector<double> eta(active.size());
      const double floor = std::max(cg_rel_tol_, kFp32CgFloor);
      for (size_t a = 0; a < active.size(); ++a) {
        const int i = idx[a];
        const double want = (norm[i] > 0) ? 0.05 * nr_rel_tol_ * norm0[i] / norm[i] : floor;
        eta[a] = std::max(floor, std::min(0.1, want));
      }
      bool graphed = false;
      if (fused) {
        for (int a = 0; a < na; ++a) h_eta_[a] = eta[a];
        check(cudaMemcpyAsync(d_eta_, h_eta_, na * sizeof(double), cudaMemcpyHostToDevice, stream_), "CG tolerances");
        graphed = newton_graph(na);
        if (!graphed) assemble32(na);  // the graph could not be built: the unfused iteration follows
      }
      if (graphed) {
        // assembly, solve, u += du and the residual have run; a multigrid solve that reached its cap is undone
        // and redone from du = 0 with Jacobi, then the residual of those slots is taken again
        download_out();
        std::vector<int> redo;
        std::vector<double> redo_eta;
        for (int a = 0; a < na; ++a)
          if (h_out_[active[a]].cg_maxed) {
            mg_its[a] = h_out_[active[a]].cg_its;
            redo.push_back(active[a]);
            redo_eta.push_back(eta[a]);
          }
        if (!redo.empty()) {
          for (int s : redo) {
            launches_ += 1;
            check_launch(mgb_launch_axpy_du32(&mesh_, slots_[s].u, slots_[s].du32, -1.0, stream_), "undo du");
          }
          upload_list(redo);
          cg_solve32(redo, redo_eta, false);
          launches_ += 1;
          check_launch(mgb_launch_add_du32(&mesh_, d_insts_, d_list_, (int)redo.size(), stream_), "u += du");
          residual(redo);
          upload_list(active);
          download_out();
        }
      } else {
        cg_solve32(active, eta);
        if (mg_) {
          // A multigrid solve that reached its iteration cap is redone from du = 0 with Jacobi.
          download_out();
          std::vector<int> redo;
          std::vector<double> redo_eta;
          for (int a = 0; a < na; ++a)
            if (h_out_[active[a]].cg_maxed) {
              mg_its[a] = h_out_[active[a]].cg_its;
              redo.push_back(active[a]);
              redo_eta.push_back(eta[a]);
            }
          if (!redo.empty()) {
            upload_list(redo);
            cg_solve32(redo, redo_eta, false);
            upload_list(active);
          }
        }
        launches_ += 1;
        check_launch(mgb_launch_add_du32(&mesh_, d_insts_, d_list_, na, stream_), "u += du");
        residual(active);
        download_out();
      }
      have_residual = true;
      // Backtracking line search per instance (Armijo on |b|, step halved up to 8 times): a full step that
      // does not reduce the residual (J2 points crossing the yield surface) is shortened.
      std::vector<double> t(na, 1.0);
      for (int ls = 0; ls < 8; ++ls) {
        std::vector<int> back;
        for (int a = 0; a < na; ++a) {
          const double nb = h_out_[active[a]].norm;
          if (std::isfinite(nb) && nb > (1.0 - 1e-4 * t[a]) * norm[idx[a]]) back.push_back(a);
        }
        if (back.empty()) break;
        std::vector<int> bslots;
        for (int a : back) {
          launches_ += 1;
          check_launch(mgb_launch_axpy_du32(&mesh_, slots_[active[a]].u, slots_[active[a]].du32, -0.5 * t[a], stream_),
                       "line search");
          t[a] *= 0.5;
          bslots.push_back(active[a]);
        }
        upload_list(bslots);
        residual(bslots);
        download_out();
      }
    } else if (exact_tangent_) {
      // A load path (slot 0 alone): BiCGSTAB on the non-symmetric exact tangent, then a backtracking line
      // search on |b| (Armijo, step halved up to 8 times): J2 points crossing the yield surface make the
      // full Newton step cycle on fine meshes.
      const int s0 = active[0];
      Slot &w = slots_[s0];
      bicg_its = bicg_solve(false, w.du);
      const double nb0 = norm[idx[0]];
      double t = 1.0, best_t = 1.0, best = -1.0;
      launches_ += 1;
      check_launch(mgb_launch_axpy(nndim(), w.u, w.du, 1.0, stream_), "u += du");
      for (int ls = 0; ls <= 8; ++ls) {
        residual(active);
        download_out();
        const double nb = h_out_[s0].norm;
        if (best < 0 || nb < best) {
          best = nb;
          best_t = t;
        }
        if (nb <= (1.0 - 1e-4 * t) * nb0 || !std::isfinite(nb)) break;
        if (ls == 8) break;
        launches_ += 1;
        check_launch(mgb_launch_axpy(nndim(), w.u, w.du, -0.5 * t, stream_), "line search");
        t *= 0.5;
      }
      if (best_t != t) {
        launches_ += 1;
        check_launch(mgb_launch_axpy(nndim(), w.u, w.du, best_t - t, stream_), "line search");
      }
    } else {
      cg_solve(active);
      check_launch(mgb_launch_add_du(&mesh_, d_insts_, d_list_, na, stream_), "u += du");
      if (a0_iteration) {
        for (int s : active) h_insts_[s].vals = slots_[s].vals;
        upload_insts();
      }
    }
    if (!have_residual) {
      residual(active);
      download_out();
    }
    for (size_t a = 0; a < active.size(); ++a) {
      const int i = idx[a];
      const InstOut &o = h_out_[slots[i]];
      const int its = ((exact_tangent_ && !mixed) ? bicg_its : o.cg_its) + mg_its[a];
      res[i].solver_its += its;
      res[i].cg_maxed |= (exact_tangent_ && !mixed) ? !last_bicg_converged_ : o.cg_maxed != 0;
      total_cg_its_ += its;
      res[i].its++;
      norm[i] = o.norm;
    }
  }
  for (int i = 0; i < n; ++i) res[i].rel_norm = (norm0[i] > 0) ? norm[i] / norm0[i] : 0.0;
  return res;
}

void Engine::allocate_vars(GpState &g) {
  const size_t nv = nvars();
  g.vars_n = dalloc<double>(nv, "vars_n");
  g.vars_k = dalloc<double>(nv, "vars_k");
  check(cudaMemsetAsync(g.vars_n, 0, nv * sizeof(double), stream_), "vars_n zero");
  check(cudaMemsetAsync(g.vars_k, 0, nv * sizeof(double), stream_), "vars_k zero");
  g.allocated = true;
}

// homogenize_fe_one_way / homogenize_fe_full (homogenize.cpp:111-282) for a batch of macro points.
void Engine::homogenize_fe_batch(const std::vector<int> &gp_ids) {
  const int n = (int)gp_ids.size();
  const size_t ubytes = nndim() * sizeof(double);
  std::vector<int> all(n);
  for (int i = 0; i < n; ++i) all[i] = i;
  std::vector<std::array<double, 6>> strains(n);
  for (int i = 0; i < n; ++i) {
    GpState &g = gps_[gp_ids[i]];
    Slot &w = slots_[i];
    Inst &I = h_insts_[i];
    check(cudaMemcpyAsync(w.u, g.u_n, ubytes, cudaMemcpyDeviceToDevice, stream_), "u <- u_n");
    I.vars_old = g.allocated ? g.vars_n : nullptr;
    I.has_vars_old = g.allocated ? 1 : 0;
    I.vars_new = g.allocated ? g.vars_k : w.vars_aux;
    if (!g.allocated) check(cudaMemsetAsync(w.vars_aux, 0, nvars() * sizeof(double), stream_), "vars aux");
    check(cudaMemsetAsync(w.out, 0, sizeof(InstOut), stream_), "out reset");
    g.cost = 0;
    g.subiterated = false;
    g.status = 0;
    std::memcpy(strains[i].data(), g.strain, sizeof(g.strain));
  }
  if (precision_ == MICROPP3_MIXED) {
    // the mixed form's Newton starts from u_n moved with the affine field of the strain increment
    predict_de_.resize(n);
    for (int i = 0; i < n; ++i) {
      const GpState &g = gps_[gp_ids[i]];
      for (int v = 0; v < 6; ++v) predict_de_[i][v] = g.strain[v] - g.strain_old[v];
    }
  }
  std::vector<NewtonResult> r = newton(all, strains);
  std::vector<int> last_sits(n);
  std::vector<int> unconv;
  for (int i = 0; i < n; ++i) {
    GpState &g = gps_[gp_ids[i]];
    check(cudaMemcpyAsync(g.u_k, slots_[i].u, ubytes, cudaMemcpyDeviceToDevice, stream_), "u_k <- u");
    g.nr_its = r[i].its;
    g.nr_solver_its = r[i].solver_its;
    g.nr_converged = r[i].converged;
    g.cost += r[i].solver_its;
    g.converged = r[i].converged;
    if (r[i].cg_maxed) g.status |= MICROPP3_STATUS_CG_MAX_ITS;
    last_sits[i] = r[i].solver_its;
    if (!g.converged && subiterations_) unconv.push_back(i);
  }

  // Sub-iterations (homogenize.cpp:215-232): walk the increment again in nsubiterations steps from u_n.
  if (!unconv.empty()) {
    std::vector<std::array<double, 6>> eps_sub(unconv.size()), deps(unconv.size());
    for (size_t a = 0; a < unconv.size(); ++a) {
      GpState &g = gps_[gp_ids[unconv[a]]];
      check(cudaMemcpyAsync(slots_[unconv[a]].u, g.u_n, ubytes, cudaMemcpyDeviceToDevice, stream_), "u <- u_n");
      std::memcpy(eps_sub[a].data(), g.strain_old, sizeof(g.strain_old));
      g.subiterated = true;
      for (int v = 0; v < 6; ++v) deps[a][v] = (g.strain[v] - g.strain_old[v]) / nsubiterations_;
    }
    std::vector<NewtonResult> rs;
    for (int it = 0; it < nsubiterations_; ++it) {
      for (size_t a = 0; a < unconv.size(); ++a)
        for (int v = 0; v < 6; ++v) eps_sub[a][v] += deps[a][v];
      rs = newton(unconv, eps_sub);
      for (size_t a = 0; a < unconv.size(); ++a) {
        GpState &g = gps_[gp_ids[unconv[a]]];
        g.cost += rs[a].solver_its;
        if (rs[a].cg_maxed) g.status |= MICROPP3_STATUS_CG_MAX_ITS;
        last_sits[unconv[a]] = rs[a].solver_its;
      }
    }
    for (size_t a = 0; a < unconv.size(); ++a) {
      GpState &g = gps_[gp_ids[unconv[a]]];
      if (!rs.empty()) g.converged = rs[a].converged;
      check(cudaMemcpyAsync(g.u_k, slots_[unconv[a]].u, ubytes, cudaMemcpyDeviceToDevice, stream_), "u_k <- u");
    }
  }

  // Average stress from the last residual evaluation: it was made at u_k with vars_n.
  download_out();
  for (int i = 0; i < n; ++i) {
    GpState &g = gps_[gp_ids[i]];
    const InstOut &o = h_out_[i];
    if (lin_stress_) {
      std::memset(g.stress, 0, sizeof(g.stress));
      for (int a = 0; a < 6; ++a)
        for (int b = 0; b < 6; ++b) g.stress[a] += g.ctan[a * 6 + b] * g.strain[b];
    } else {
      std::memcpy(g.stress, o.sig, sizeof(g.stress));
    }
    if (!g.converged) g.status |= MICROPP3_STATUS_NEWTON_MAX_ITS;
    if (o.nonfinite) g.status |= MICROPP3_STATUS_NONFINITE;
  }

  // calc_vars_new (update.cpp:32-56) at u_k = the slot's u.
  for (int i = 0; i < n; ++i) check(cudaMemsetAsync(&slots_[i].out->nonlinear, 0, sizeof(int), stream_), "flag");
  upload_insts();
  upload_list(all);
  launches_ += 1;
  check_launch(mgb_launch_evolve(&mesh_, &mats_, d_etype_, d_dsh_, d_insts_, d_list_, n, stream_), "evolve");
  download_out();
  std::vector<int> pert;
  for (int i = 0; i < n; ++i) {
    GpState &g = gps_[gp_ids[i]];
    if (h_out_[i].nonlinear && !g.allocated) {
      allocate_vars(g);
      check(cudaMemcpyAsync(g.vars_k, slots_[i].vars_aux, nvars() * sizeof(double), cudaMemcpyDeviceToDevice, stream_),
            "vars_k <- vars_new");
    }
    if (g.coupling == MICROPP3_FE_FULL && g.allocated) pert.push_back(i);
  }

  // ctan by implicit differentiation at the converged state (u_k, vars_n): one 6-RHS tangent solve.
  if (!pert.empty() && ctan_mode_ == MICROPP3_CTAN_IMPLICIT) {
    for (int i : pert) {
      GpState &g = gps_[gp_ids[i]];
      h_insts_[i].vars_old = g.vars_n;
    }
    std::vector<int> its = tangent_solve(pert);
    for (size_t a = 0; a < pert.size(); ++a) {
      const int i = pert[a];
      GpState &g = gps_[gp_ids[i]];
      const InstOut &o = h_out_[i];
      std::memcpy(g.ctan, o.ctan, sizeof(g.ctan));
      g.cost += its[a];
      if (o.nonfinite) g.status |= MICROPP3_STATUS_NONFINITE;
    }
    pert.clear();
  }

  // ctan by 6 perturbed nonlinear solves (homogenize.cpp:256-275): u carried from u_k across the six
  // solves, history vars_n, cost charged with the main solve's CG count each time.
  if (!pert.empty()) {
    std::vector<std::array<double, 6>> sig0(pert.size());
    for (size_t a = 0; a < pert.size(); ++a) {
      const int i = pert[a];
      GpState &g = gps_[gp_ids[i]];
      check(cudaMemcpyAsync(slots_[i].u, g.u_k, ubytes, cudaMemcpyDeviceToDevice, stream_), "u <- u_k");
      h_insts_[i].vars_old = g.vars_n;
      std::memcpy(sig0[a].data(), g.stress, sizeof(g.stress));
    }
    for (int c = 0; c < 6; ++c) {
      std::vector<std::array<double, 6>> eps1(pert.size());
      for (size_t a = 0; a < pert.size(); ++a) {
        const GpState &g = gps_[gp_ids[pert[a]]];
        std::memcpy(eps1[a].data(), g.strain, sizeof(g.strain));
        eps1[a][c] += kDepsCtanAve;
      }
      std::vector<NewtonResult> rp = newton(pert, eps1);
      for (size_t a = 0; a < pert.size(); ++a) {
        const int i = pert[a];
        GpState &g = gps_[gp_ids[i]];
        g.cost += last_sits[i];
        if (rp[a].cg_maxed) g.status |= MICROPP3_STATUS_CG_MAX_ITS;
        const InstOut &o = h_out_[i];
        for (int v = 0; v < 6; ++v) g.ctan[v * 6 + c] = (o.sig[v] - sig0[a][v]) / kDepsCtanAve;
        if (o.nonfinite) g.status |= MICROPP3_STATUS_NONFINITE;
      }
    }
  }
  sync();
}

// ------------------------------------------------------------------------------------------------
// Public operations

void Engine::set_strain(int gp, const double *strain) { std::memcpy(gps_.at(gp).strain, strain, 6 * sizeof(double)); }
void Engine::get_stress(int gp, double *stress) const { std::memcpy(stress, gps_.at(gp).stress, 6 * sizeof(double)); }
void Engine::get_ctan(int gp, double *ctan) const { std::memcpy(ctan, gps_.at(gp).ctan, 36 * sizeof(double)); }

// homogenize (homogenize.cpp:68-99): linear points on the host, FE points batched on the GPU.
void Engine::homogenize() {
  check(cudaEventRecord(ev0_, stream_), "event");
  std::vector<int> fe;
  for (int i = 0; i < ngp_; ++i) {
    GpState &g = gps_[i];
    if (g.coupling == MICROPP3_FE_LINEAR || g.coupling == MICROPP3_MIX_RULE_CHAMIS) {
      std::memset(g.stress, 0, sizeof(g.stress));
      for (int a = 0; a < 6; ++a)
        for (int b = 0; b < 6; ++b) g.stress[a] += g.ctan[a * 6 + b] * g.strain[b];
    } else {
      fe.push_back(i);
    }
  }
  if (!fe.empty()) {
    // Slots for as many points as memory allows (at most all of them).
    size_t free_b = 0, total_b = 0;
    check(cudaMemGetInfo(&free_b, &total_b), "mem info");
    const int fit = std::max(1, (int)((double)free_b * 0.6 / slot_bytes()) + (int)slots_.size());
    const int want = std::min((int)fe.size(), fit);
    ensure_slots(want);
    const int per = (int)slots_.size();
    for (size_t b = 0; b < fe.size(); b += per) {
      std::vector<int> part(fe.begin() + b, fe.begin() + std::min(fe.size(), b + per));
      homogenize_fe_batch(part);
    }
  }
  check(cudaEventRecord(ev1_, stream_), "event");
  check(cudaEventSynchronize(ev1_), "event sync");
  float ms = 0;
  check(cudaEventElapsedTime(&ms, ev0_, ev1_), "elapsed");
  last_ms_ = ms;
}

void Engine::homogenize_linear() {
  for (auto &g : gps_) {
    std::memset(g.stress, 0, sizeof(g.stress));
    for (int a = 0; a < 6; ++a)
      for (int b = 0; b < 6; ++b) g.stress[a] += g.ctan[a * 6 + b] * g.strain[b];
  }
}

// update_vars (gp.hpp:95-105).
void Engine::update_vars() {
  for (auto &g : gps_) {
    std::swap(g.vars_n, g.vars_k);
    std::swap(g.u_n, g.u_k);
    std::memcpy(g.strain_old, g.strain, sizeof(g.strain));
  }
}

int Engine::get_non_linear_gps() const {
  int c = 0;
  for (const auto &g : gps_) c += g.allocated ? 1 : 0;
  return c;
}

void Engine::get_newton(int gp, int *its, int *sits, int *conv) const {
  const GpState &g = gps_.at(gp);
  if (its) *its = g.nr_its;
  if (sits) *sits = g.nr_solver_its;
  if (conv) *conv = g.nr_converged ? 1 : 0;
}

// calc_ctan_lin_fe_models (micropp.cpp:255-284): 6 linear solves from u = 0 at strain 1e-8 e_i, batched.
void Engine::calc_ctan_lin() {
  size_t free_b = 0, total_b = 0;
  check(cudaMemGetInfo(&free_b, &total_b), "mem info");
  const int fit = std::max(1, (int)((double)free_b * 0.6 / slot_bytes()));
  ensure_slots(std::min(6, fit));
  if (ctan_mode_ == MICROPP3_CTAN_IMPLICIT) {
    // The linear ctan is the implicit derivative at u = 0 with no history: one 6-RHS tangent solve.
    check(cudaMemsetAsync(slots_[0].u, 0, nndim() * sizeof(double), stream_), "u zero");
    check(cudaMemsetAsync(slots_[0].out, 0, sizeof(InstOut), stream_), "out reset");
    h_insts_[0].vars_old = nullptr;
    h_insts_[0].has_vars_old = 0;
    tangent_solve(std::vector<int>{0});
    std::memcpy(ctan_lin_, h_out_[0].ctan, sizeof(ctan_lin_));
    return;
  }
  const int per = (int)slots_.size();
  for (int c0 = 0; c0 < 6; c0 += per) {
    const int cnt = std::min(per, 6 - c0);
    std::vector<int> sl(cnt);
    std::vector<std::array<double, 6>> eps(cnt);
    for (int a = 0; a < cnt; ++a) {
      sl[a] = a;
      eps[a].fill(0.0);
      eps[a][c0 + a] += kDepsCtanAve;
      check(cudaMemsetAsync(slots_[a].u, 0, nndim() * sizeof(double), stream_), "u zero");
      h_insts_[a].vars_old = nullptr;
      h_insts_[a].has_vars_old = 0;
      h_insts_[a].vars_new = slots_[a].vars_aux;
    }
    newton(sl, eps);
    download_out();
    for (int a = 0; a < cnt; ++a)
      for (int v = 0; v < 6; ++v) ctan_lin_[v * 6 + c0 + a] = h_out_[a].sig[v] / kDepsCtanAve;
  }
}

void Engine::get_vars(int gp, int which, double *out) const {
  const GpState &g = gps_.at(gp);
  const double *src = g.allocated ? (which ? g.vars_k : g.vars_n) : nullptr;
  if (src) {
    check(cudaMemcpyAsync(out, src, nvars() * sizeof(double), cudaMemcpyDeviceToHost, stream_), "vars download");
    check(cudaStreamSynchronize(stream_), "sync");
  } else {
    std::memset(out, 0, nvars() * sizeof(double));
  }
}

void Engine::get_u(int gp, int which, double *out) const {
  const GpState &g = gps_.at(gp);
  const double *src = which ? g.u_k : g.u_n;
  if (src) {
    check(cudaMemcpyAsync(out, src, nndim() * sizeof(double), cudaMemcpyDeviceToHost, stream_), "u download");
    check(cudaStreamSynchronize(stream_), "sync");
  } else {
    std::memset(out, 0, nndim() * sizeof(double));
  }
}

void Engine::get_elem_type(int *out) const {
  for (int e = 0; e < mesh_.nelem; ++e) out[e] = etype_[e];
}

void Engine::get_ctan_lin(double *out) const { std::memcpy(out, ctan_lin_, sizeof(ctan_lin_)); }

static std::string restart_name(int rank, int id) {
  std::ostringstream os;
  os << "micropp-restart-" << rank << "-" << id << ".bin";
  return os.str();
}

// write_restart (output.cpp:216-238, gp.hpp:107-113): per point a one-byte `allocated`, then vars_n and u_n.
void Engine::write_restart(int restart_id) const {
  std::ofstream f(restart_name(mpi_rank_, restart_id), std::ios::out | std::ios::binary);
  if (!f) throw std::runtime_error("cannot open restart file for writing");
  std::vector<double> vars(nvars()), u(nndim());
  for (int i = 0; i < ngp_; ++i) {
    const GpState &g = gps_[i];
    const char a = g.allocated ? 1 : 0;
    f.write(&a, 1);
    if (g.allocated) {
      get_vars(i, 0, vars.data());
      get_u(i, 0, u.data());
      f.write((const char *)vars.data(), vars.size() * sizeof(double));
      f.write((const char *)u.data(), u.size() * sizeof(double));
    }
  }
}

// read_restart (output.cpp:240-262, gp.hpp:115-124): an allocated record brings vars_n and u_n back and
// leaves vars_k zeroed.
void Engine::read_restart(int restart_id) {
  std::ifstream f(restart_name(mpi_rank_, restart_id), std::ios::in | std::ios::binary);
  if (!f) throw std::runtime_error("cannot open restart file for reading");
  std::vector<double> vars(nvars()), u(nndim());
  for (int i = 0; i < ngp_; ++i) {
    GpState &g = gps_[i];
    char a = 0;
    if (!f.read(&a, 1)) break;
    if (a) {
      if (!g.allocated) allocate_vars(g);
      check(cudaMemsetAsync(g.vars_k, 0, nvars() * sizeof(double), stream_), "vars_k zero");
      f.read((char *)vars.data(), vars.size() * sizeof(double));
      f.read((char *)u.data(), u.size() * sizeof(double));
      check(cudaMemcpyAsync(g.vars_n, vars.data(), vars.size() * sizeof(double), cudaMemcpyHostToDevice, stream_),
            "vars_n upload");
      if (g.u_n)
        check(cudaMemcpyAsync(g.u_n, u.data(), u.size() * sizeof(double), cudaMemcpyHostToDevice, stream_), "u_n");
      sync();
    } else if (g.allocated) {
      dfree(g.vars_n);
      dfree(g.vars_k);
      g.vars_n = g.vars_k = nullptr;
      g.allocated = false;
    }
  }
  sync();
}

// print_info (micropp.cpp:546-597).
void Engine::print_info() const {
  static const char *names[] = {"MIC_HOMOGENEOUS", "MIC_SPHERE", "MIC_LAYER_Y", "MIC_CILI_FIB_X", "MIC_CILI_FIB_Z",
                                "MIC_CILI_FIB_XZ", "MIC_QUAD_FIB_XYZ", "MIC_QUAD_FIB_XZ",
                                "MIC_QUAD_FIB_XZ_BROKEN_X", "MIC3D_SPHERES", "MIC3D_8", "MIC3D_FIBS_20_ORDER",
                                "MIC3D_FIBS_20_DISORDER"};
  int count[4] = {0, 0, 0, 0};
  for (const auto &g : gps_) count[g.coupling]++;
  std::cout << "micropp3 (GB300)" << std::endl;
  std::cout << "Micro-structure   : " << ((micro_type_ >= 0 && micro_type_ < 13) ? names[micro_type_] : "?") << std::endl;
  std::cout << "MATRIX [%]        : " << Vm_ << std::endl;
  std::cout << "FIBER  [%]        : " << Vf_ << std::endl;
  std::cout << "FE_LINEAR         : " << count[0] << " GPs" << std::endl;
  std::cout << "FE_ONE_WAY        : " << count[1] << " GPs" << std::endl;
  std::cout << "FE_FULL           : " << count[2] << " GPs" << std::endl;
  std::cout << "MIX_RULE_CHAMIS   : " << count[3] << " GPs" << std::endl;
  std::cout << "NUM SUBITS        : " << nsubiterations_ << std::endl;
  std::cout << "MPI RANK          : " << mpi_rank_ << std::endl;
  std::cout << "ngp :" << ngp_ << " nx :" << mesh_.nx << " ny :" << mesh_.ny << " nz :" << mesh_.nz
            << " nn :" << mesh_.nn << std::endl;
  std::cout << "geo_params:";
  for (double g : geo_params_) std::cout << " " << g;
  std::cout << std::endl;
  for (int i = 0; i < 3; ++i)
    std::cout << "material " << i << ": type " << mats_.m[i].type << " E = " << mats_.m[i].E << " nu = " << mats_.m[i].nu
              << " Ka = " << mats_.m[i].Ka << " Sy = " << mats_.m[i].Sy << " Xt = " << mats_.m[i].Xt << std::endl;
  std::cout << std::endl << "ctan_lin_fe = " << std::endl;
  for (int i = 0; i < 6; ++i) {
    for (int j = 0; j < 6; ++j) std::cout << ctan_lin_[i * 6 + j] << "\t";
    std::cout << std::endl;
  }
  std::cout << std::endl;
}

// output / write_vtu (output.cpp:29-214): element fields computed on the device (calc_fields,
// average.cpp:84-112) from u_k and vars_n, written as the reference's ASCII VTU (<filename>.vtu).
void Engine::output_vtu(int gp, const char *filename) {
  const GpState &g = gps_.at(gp);
  if (!g.u_k) throw std::runtime_error("output needs an FE-coupled Gauss point (it has no displacement field)");
  const MeshDev &m = mesh_;
  const double ivol = 1.0 / (m.wg * kNpe);
  double *d_fields = dalloc<double>((size_t)12 * m.nelem, "fields");
  std::vector<double> fields((size_t)12 * m.nelem), u(nndim()), vars;
  try {
    launches_ += 1;
    check_launch(mgb_launch_elem_fields(&mesh_, &mats_, d_etype_, d_dsh_, g.u_k, g.allocated ? g.vars_n : nullptr,
                                        ivol, d_fields, stream_),
                 "element fields");
    check(cudaMemcpyAsync(fields.data(), d_fields, fields.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_),
          "fields download");
    sync();
  } catch (...) {
    dfree(d_fields);
    throw;
  }
  dfree(d_fields);
  get_u(gp, 1, u.data());
  if (g.allocated) {
    vars.resize(nvars());
    get_vars(gp, 0, vars.data());
  }
  std::ofstream f(std::string(filename) + ".vtu");
  if (!f) throw std::runtime_error("cannot open the VTU file for writing");
  f << "<?xml version=\"1.0\"?>\n"
    << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
    << "<UnstructuredGrid>\n"
    << "<Piece NumberOfPoints=\"" << m.nn << "\" NumberOfCells=\"" << m.nelem << "\">\n"
    << "<Points>\n"
    << "<DataArray type=\"Float64\" Name=\"Position\" NumberOfComponents=\"3\" format=\"ascii\">" << std::endl;
  f << std::scientific;
  for (int k = 0; k < m.nz; ++k)
    for (int j = 0; j < m.ny; ++j)
      for (int i = 0; i < m.nx; ++i) f << i * m.dx << " " << j * m.dy << " " << k * m.dz << " \n";
  f << "</DataArray>\n</Points>\n<Cells>\n" << std::endl;
  f << "<DataArray type=\"Int32\" Name=\"connectivity\" NumberOfComponents=\"1\" format=\"ascii\">" << std::endl;
  for (int ez = 0; ez < m.nez; ++ez)
    for (int ey = 0; ey < m.ney; ++ey)
      for (int ex = 0; ex < m.nex; ++ex) {
        const int n0 = ez * m.nxny + ey * m.nx + ex;
        for (int a = 0; a < 8; ++a) f << n0 + kCorner[a][2] * m.nxny + kCorner[a][1] * m.nx + kCorner[a][0] << ' ';
        f << "\n";
      }
  f << "</DataArray>" << std::endl;
  f << "<DataArray type=\"Int32\" Name=\"offsets\" NumberOfComponents=\"1\" format=\"ascii\">" << std::endl;
  for (int e = 0, ce = 8; e < m.nelem; ++e, ce += 8) f << ce << " ";
  f << "\n</DataArray>" << std::endl;
  f << "<DataArray type=\"UInt8\"  Name=\"types\" NumberOfComponents=\"1\" format=\"ascii\">" << std::endl;
  for (int e = 0; e < m.nelem; ++e) f << 12 << " ";
  f << "\n</DataArray>" << std::endl;
  f << "</Cells>" << std::endl;
  f << "<PointData Vectors=\"displ\" >" << std::endl;
  f << "<DataArray type=\"Float64\" Name=\"displ\" NumberOfComponents=\"3\" format=\"ascii\" >" << std::endl;
  for (int n = 0; n < m.nn; ++n) {
    for (int d = 0; d < 3; ++d) f << u[n * 3 + d] << " ";
    f << "\n";
  }
  f << "</DataArray>" << std::endl;
  f << "</PointData>" << std::endl;
  f << "<CellData>" << std::endl;
  f << "<DataArray type=\"Float64\" Name=\"strain\" NumberOfComponents=\"6\" format=\"ascii\">" << std::endl;
  for (int e = 0; e < m.nelem; ++e) {
    for (int v = 0; v < 6; ++v) f << fields[(size_t)e * 12 + v] << " ";
    f << "\n";
  }
  f << "</DataArray>\n";
  f << "<DataArray type=\"Float64\" Name=\"stress\" NumberOfComponents=\"6\" format=\"ascii\">" << std::endl;
  for (int e = 0; e < m.nelem; ++e) {
    for (int v = 0; v < 6; ++v) f << fields[(size_t)e * 12 + 6 + v] << " ";
    f << "\n";
  }
  f << "</DataArray>\n";
  f << "<DataArray type=\"Int32\" Name=\"elem_type\" NumberOfComponents=\"1\" format=\"ascii\">" << std::endl;
  for (int e = 0; e < m.nelem; ++e) f << (int)etype_[e] << " ";
  f << "\n</DataArray>" << std::endl;
  // Per element: the plastic-strain norm field keeps the reference's expression (x + sqrt(x), output.cpp:162-175),
  // then the averages of r (damage_e), D (damage_D) and alpha (hardening) over the 8 Gauss points.
  auto var = [&](int e, int gpi, int v) { return vars.empty() ? 0.0 : vars[((size_t)e * 8 + gpi) * kNvarGp + v]; };
  f << "<DataArray type=\"Float64\" Name=\"plasticity\" NumberOfComponents=\"1\" format=\"ascii\">" << std::endl;
  for (int e = 0; e < m.nelem; ++e) {
    double pl = 0.0;
    for (int gpi = 0; gpi < 8; ++gpi)
      for (int v = 0; v < 6; ++v) pl += var(e, gpi, v) * var(e, gpi, v);
    pl += std::sqrt(pl);
    f << pl / 8 << " ";
  }
  f << "\n</DataArray>" << std::endl;
  const char *names[3] = {"damage_e", "damage_D", "hardening"};
  const int idx[3] = {0, 1, 6};
  for (int q = 0; q < 3; ++q) {
    f << "<DataArray type=\"Float64\" Name=\"" << names[q] << "\" NumberOfComponents=\"1\" format=\"ascii\">"
      << std::endl;
    for (int e = 0; e < m.nelem; ++e) {
      double a = 0.0;
      for (int gpi = 0; gpi < 8; ++gpi) a += var(e, gpi, idx[q]);
      f << a / 8 << " ";
    }
    f << "\n</DataArray>" << std::endl;
  }
  f << "</CellData>" << std::endl;
  f << "</Piece>" << std::endl;
  f << "</UnstructuredGrid>" << std::endl;
  f << "</VTKFile>" << std::endl;
}

}  // namespace mgb
