// engine.hpp -- host side of the GB300 homogenization: one Engine per micropp3 handle.
//
// The Engine owns the device state of every macro Gauss point of a handle (displacements u_n/u_k and the
// internal variables vars_n/vars_k, mirroring gp_t, gp.hpp:33-125) and a pool of workspace slots.  A
// homogenize() call runs all FE-coupled points of the handle through the solver at once: the slots of a
// batch advance in lockstep through set_bc -> residual -> (assemble -> CG -> u += du -> residual)* with a
// per-slot Newton mask, so each point sees exactly the reference's sequence of operations
// (homogenize.cpp:188-282, solve.cpp:28-82) while every kernel launch covers the whole batch.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "device.cuh"
#include "micropp_gb300.h"

namespace mgb {

struct GpState {
  double strain_old[6] = {0, 0, 0, 0, 0, 0};
  double strain[6] = {0, 0, 0, 0, 0, 0};
  double stress[6] = {0, 0, 0, 0, 0, 0};
  double ctan[36] = {0};
  bool allocated = false;
  long cost = 0;
  bool converged = true;
  bool subiterated = false;
  int coupling = MICROPP3_FE_ONE_WAY;
  int status = 0;
  int nr_its = 0, nr_solver_its = 0;
  bool nr_converged = false;
  double *u_n = nullptr, *u_k = nullptr;        // device, nndim
  double *vars_n = nullptr, *vars_k = nullptr;  // device, nvars (when allocated)
};

struct Slot {
  double *u = nullptr, *du = nullptr, *b = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *Ap = nullptr;
  double *kinv = nullptr, *vals = nullptr, *be = nullptr, *vars_aux = nullptr, *red = nullptr;
  float *vals32 = nullptr, *kinv32 = nullptr, *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *Ap32 = nullptr,
        *du32 = nullptr;
  float *X6h = nullptr, *X6l = nullptr, *F6h = nullptr, *F6l = nullptr;  // double-float pairs
  float *R6 = nullptr, *Z6 = nullptr, *P6 = nullptr, *AP6 = nullptr, *D6 = nullptr;
  float *gpd = nullptr;
  MgInst *mg = nullptr;          // device copy of the multigrid hierarchy's pointers
  std::vector<float *> mg_bufs;  // its buffers
  std::vector<unsigned short *> mg_bufs16;
  unsigned int *ticket = nullptr;
  CgState *cg = nullptr;
  Cg6State *cg6 = nullptr;
  InstOut *out = nullptr;
};

// Constants of one material for the device laws (engine.cpp).
MatDev make_matdev(int type, double E, double nu, double Ka, double Sy, double Xt);

// A load path of one RVE for reverse-mode gradients (path.cpp): the materials it runs with, the checkpoints
// of its forward pass and the buffers of the adjoint pass.
struct PathState {
  int nsteps = 0, every = 1;
  std::vector<double> strains;           // nsteps x 6
  Mats mats{};
  double ke[3][576];
  double *d_ke = nullptr;                // per-phase elastic element matrices of `mats`
  std::vector<double *> ck_u, ck_h;      // (u, history) before step c * every
  std::vector<double *> seg_u, seg_h;    // a recomputed segment: u after step, history before step
  double *h_a = nullptr, *h_b = nullptr, *mu_a = nullptr, *mu_b = nullptr;
  AdjDev adj{};                          // BiCGSTAB vectors (x = the adjoint solution)
  BicgState *d_st = nullptr;
  double *d_out = nullptr;               // 21 sums of one backward step
  bool ready = false;
  int bicg_its = 0;                      // BiCGSTAB iterations of the last backward pass
  bool bicg_converged = true;
  std::vector<int> nr_its, cg_its, nr_conv, cg_maxed;  // per step of the forward pass
  std::vector<double> nr_norm;           // |b| / |b0| at the end of each step's Newton
};

struct NewtonResult {
  int its = 0, solver_its = 0;
  bool converged = false;
  bool cg_maxed = false;  // some CG solve of this Newton run stopped at cg_max_its
  double rel_norm = 0.0;  // |b| / |b0| of the last residual
};

struct KernelTimer {
  bool enabled = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pool;
  size_t used = 0;
  long launches = 0;
  double ms = 0.0, bytes = 0.0, pending_bytes = 0.0;
};

class Engine {
 public:
  explicit Engine(const micropp3_config &cfg);
  ~Engine();
  Engine(const Engine &) = delete;
  Engine &operator=(const Engine &) = delete;

  int ngp() const { return ngp_; }
  int nelem() const { return mesh_.nelem; }
  int nndim() const { return mesh_.nn * 3; }
  int nvars() const { return mesh_.nelem * kNpe * kNvarGp; }

  void set_strain(int gp, const double *strain);
  void get_stress(int gp, double *stress) const;
  void get_ctan(int gp, double *ctan) const;
  void homogenize();
  void homogenize_linear();
  void update_vars();

  int is_non_linear(int gp) const { return gps_.at(gp).allocated ? 1 : 0; }
  int get_non_linear_gps() const;
  long get_cost(int gp) const { return gps_.at(gp).cost; }
  bool has_converged(int gp) const { return gps_.at(gp).converged; }
  bool has_subiterated(int gp) const { return gps_.at(gp).subiterated; }
  int get_status(int gp) const { return gps_.at(gp).status; }
  void get_newton(int gp, int *its, int *sits, int *conv) const;

  void get_vars(int gp, int which, double *out) const;
  void get_u(int gp, int which, double *out) const;
  void get_elem_type(int *out) const;
  void get_ctan_lin(double *out) const;
  void write_restart(int restart_id) const;
  void read_restart(int restart_id);
  void output_vtu(int gp, const char *filename);
  void print_info() const;

  // Load path from the undeformed state with per-phase parameters (E, nu, Xt, Sy, Ka); checkpoints every
  // `every` steps.  Returns 0, or 1 when a step's Newton did not converge.
  int path_forward(int nsteps, const double *strains, const double *params, int every, double *sigma);
  // Reverse pass of the last path: dL/dparams (3 x 5) and dL/dstrain_n (nsteps x 6, may be NULL) for
  // L = sum_n gsigma_n . sigma_n.  Returns 0, or 1 when an adjoint solve did not converge.
  int path_vjp(const double *gsigma, double *grad_params, double *grad_strains);
  // Newton record of step `step` of the last path's forward pass.
  void path_newton(int step, int *its, int *cg_its, int *converged, double *rel_norm) const;

  // Levels of the multigrid preconditioner of the FP32 solves (0: Jacobi).
  int mg_levels() const { return mg_ ? (int)mg_mesh_.size() : 0; }
  double last_homogenize_ms() const { return last_ms_; }
  void set_graphs(bool on);
  bool graphs() const { return graphs_; }
  void set_kernel_timing(bool on);
  bool kernel_stats(const std::string &family, long *launches, double *ms, double *bytes);
  long total_cg_its() const { return total_cg_its_; }
  long kernel_launches() const { return launches_; }
  int mpi_rank() const { return mpi_rank_; }

 private:
  // setup
  void build_mesh(const micropp3_config &cfg);
  void build_elem_types(const micropp3_config &cfg);
  void build_materials(const micropp3_config &cfg);
  void build_phase_stiffness();
  // Element matrices of the three phases' elastic tangents (ke) and, optionally, their Gauss-point terms.
  void phase_stiffness(const Mats &mats, double (*ke)[576], std::vector<float> *k0g) const;
  // FP32 Jacobian of the listed slots at their current u (the residual at that u was the last one made).
  void assemble32(int nlist);
  void ensure_slots(int n);
  void free_slots();
  void calc_ctan_lin();
  void ctan_mix_rule_chamis(double *ctan) const;

  // batched solver pieces (slot indices)
  void upload_insts();
  void upload_list(const std::vector<int> &slots);
  void download_out();
  void residual(const std::vector<int> &slots);
  void cg_solve(const std::vector<int> &slots);
  void cg_solve32(const std::vector<int> &slots, const std::vector<double> &rel_tols, bool use_mg = true);
  std::vector<int> tangent_solve(const std::vector<int> &slots, bool use_mg = true);
  double slot_bytes() const;
  std::vector<NewtonResult> newton(const std::vector<int> &slots, const std::vector<std::array<double, 6>> &strains);
  void homogenize_fe_batch(const std::vector<int> &gp_ids);
  void allocate_vars(GpState &g);
  // path.cpp
  void ensure_fp64_slot0();
  bool path_step(int n, double *h_prev, double *h_next, double *sigma, bool record);
  void path_free();
  void path_alloc_adj();
  void run_chunk(int kind, int n, const std::function<void()> &body);
  // Block size of the FP32 SpMV (kind 0) or the 6-RHS SpMV (kind 1) for this RVE size and batch (autotuned).
  int tuned_block(int kind, int nlist);
  // The tuned block if the autotuner has already run for (kind, RVE size, nlist), else 0.
  int known_block(int kind, int nlist) const;
  void clear_graphs();
  bool timing_on() const;
  // One Newton iteration of the mixed multigrid form for the nlist slots in d_list_ (tolerances in d_eta_) as
  // one CUDA graph with a WHILE node over the CG chunks; false where graphs cannot be used (then nothing ran).
  bool newton_graph(int nlist);
  int bicg_solve(bool transpose, double *x);
  // Multigrid (engine.cpp): Galerkin operators of the listed slots after an FP32 assembly; one V-cycle of the
  // 1- or 6-RHS CG of the listed slots, ending with the level-0 post-smoother (setup: start of a solve).
  void mg_rap(int nlist, bool sdiag0_done);
  void mg_vcycle(int nr, int nlist, bool setup, int block);
  // Algorithmic bytes of one V-cycle per instance: its two level-0 operator passes, and the rest.
  double mg_fine_bytes(int nr) const;
  double mg_coarse_bytes(int nr) const;
  void timer_begin(KernelTimer &t, double bytes);
  void timer_end(KernelTimer &t);
  // Adds algorithmic bytes to a timer whose launches were recorded with 0 bytes.
  void timer_add_bytes(KernelTimer &t, double bytes) {
    if (t.enabled) t.pending_bytes += bytes;
  }
  // Sum of out.cg_its over the listed slots (reads the outputs back; call when timing is enabled).
  double listed_cg_its(const std::vector<int> &slots);
  void sync();

  int ngp_ = 0;
  int micro_type_ = 0;
  int mpi_rank_ = 0;
  double geo_params_[4] = {0, 0, 0, 0};
  struct material_base mat_in_[3];
  int nr_max_its_ = 4, cg_max_its_ = 1000;
  double nr_max_tol_ = 1e-10, nr_rel_tol_ = 1e-3, cg_abs_tol_ = 1e-50, cg_rel_tol_ = 1e-5;
  bool lin_stress_ = true, subiterations_ = false, calc_ctan_lin_ = true;
  int nsubiterations_ = 10;
  int precision_ = 0, ctan_mode_ = 0;
  bool mg_ = false;                 // the FP32 solves are multigrid-preconditioned
  bool mg_half_ = false;            // ... with the FP16 copy of the fine operator in the level-0 smoothing passes
  float mg_scale16_ = 1.0f;         // power-of-two scale of that copy
  std::vector<MeshDev> mg_mesh_;    // grids of the multigrid levels (level 0 = mesh_)
  bool exact_tangent_ = false;  // FP64 Newton with the exact tangent and BiCGSTAB corrections (paths, slot 0)
  bool use_A0_ = false;         // micropp.cpp:128-143: the first its_with_A0 FP64 Newton iterations solve with A0
  int its_with_A0_ = 1;
  double *d_A0_ = nullptr;      // the FP64 Jacobian at u = 0 without history
  bool last_bicg_converged_ = true;
  std::vector<std::array<double, 6>> predict_de_;  // strain increments of the next newton() call's predictor

  MeshDev mesh_{};
  Mats mats_{};
  double bmat_[8][6][24];
  double dsh_[8 * 24];
  double ke_phase_[3][576];
  std::vector<float> k0g32_;  // wg B_g^T C_phase B_g in FP32, [3][8][576]
  bool gather32_ = false;     // the FP32 Jacobian is assembled by node gather (every phase elastic or damage)
  std::vector<int8_t> etype_;
  double Vm_ = 0, Vf_ = 0;
  double ctan_lin_[36] = {0};
  std::vector<GpState> gps_;

  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  cudaEvent_t tune_ev_[2] = {nullptr, nullptr};
  int8_t *d_etype_ = nullptr;
  double *d_dsh_ = nullptr, *d_ke_ = nullptr;
  float *d_ke32_ = nullptr, *d_k0g32_ = nullptr, *d_dsh32_ = nullptr;
  int *d_near_ = nullptr;  // interior nodes with a boundary neighbour, ascending
  int nnear_ = 0;
  std::vector<Slot> slots_;
  std::vector<Inst> h_insts_;
  Inst *d_insts_ = nullptr;
  int *d_list_ = nullptr;
  int list_cap_ = 0;
  InstOut *h_out_ = nullptr;  // pinned mirror of the slots' out records
  unsigned int *d_count_ = nullptr, *h_count_ = nullptr;
  double last_ms_ = 0.0;
  long total_cg_its_ = 0;
  long launches_ = 0;  // kernels of this library launched by the handle
  KernelTimer t_spmv_, t_update_, t_asm_, t_res_, t_spmv6_, t_upd6_;
  KernelTimer t_rap_;  // multigrid operators after an assembly: smoother diagonals and Galerkin products
  KernelTimer t_tan_;  // FP64 kernels of the implicit ctan: right-hand sides, refinement residuals, ctan sums
  KernelTimer t_mg1_, t_mg6_, t_mgc_;  // V-cycles: level-0 passes (1 and 6 RHS), coarse levels and transfers
  PathState path_;
  bool graphs_ = true;                         // CG chunks replayed from captured CUDA graphs
  std::map<long, cudaGraphExec_t> graph_cache_;  // (solver, listed instances) -> executable graph
  // Newton-iteration graphs of the mixed multigrid form, per number of listed instances.
  struct NewtonGraph {
    cudaGraphExec_t exec = nullptr;
    long fixed_launches = 0;  // kernels outside the WHILE node
    long chunk_launches = 0;  // kernels per pass of its body
  };
  std::map<int, NewtonGraph> newton_graphs_;
  bool newton_graphs_ok_ = true;               // cleared if building one fails (the iteration then runs unfused)
  double *d_eta_ = nullptr, *h_eta_ = nullptr;  // CG tolerances of the listed slots (device, pinned host)
  int eta_cap_ = 0;
  unsigned int *d_chunks_ = nullptr, *h_chunks_ = nullptr;  // chunks the last captured CG loop ran
};

}  // namespace mgb
