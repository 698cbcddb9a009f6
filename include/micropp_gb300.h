/*
 * micropp_gb300.h -- extensions of the micropp3 C ABI served by the GB300 library.
 *
 * The reference's C wrapper fixes most micropp_params_t fields (micropp_c.cpp:33-58); these entry points
 * expose the full parameter set of the C++ constructor (types.hpp:43-83), the GB300 solver options, per-RVE
 * diagnostics and timing.  They add to the drop-in ABI of micropp_c.h and change none of it.
 */
#ifndef MICROPP_GB300_EXT_H
#define MICROPP_GB300_EXT_H

#include <stdbool.h>

#include "micropp_c.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Coupling modes per macro point (types.hpp:110). */
enum { MICROPP3_FE_LINEAR = 0, MICROPP3_FE_ONE_WAY = 1, MICROPP3_FE_FULL = 2, MICROPP3_MIX_RULE_CHAMIS = 3 };

/* Arithmetic of the homogenization. */
enum {
  MICROPP3_FP64 = 0,  /* the reference algorithm in FP64 throughout (drop-in parity form) */
  MICROPP3_MIXED = 1  /* FP32 Jacobian and CG inside FP64 iterative refinement; FP64-accurate residual and
                        * averages (double-float arithmetic on the FP32 pipe, about 46 bits, for elastic and
                        * damage phases; FP64 with a J2 phase).  Newton starts from the previous solution moved
                        * with the strain increment and has a line search; its FP32 CG stops at no less than
                        * 1e-6 relative (the FP64-accurate residual decides convergence, to nr_rel_tol). */
};

/* How ctan is obtained for a nonlinear macro point. */
enum {
  MICROPP3_CTAN_PERTURB = 0,  /* the reference's 6 perturbed Newton solves (homogenize.cpp:256-275) */
  MICROPP3_CTAN_IMPLICIT = 1  /* implicit differentiation at the converged state: one 6-RHS tangent solve */
};

/* Preconditioner of the FP32 CG solves (the mixed form's Newton corrections and the implicit ctan's 6-RHS
 * tangent solve). */
enum {
  MICROPP3_PRECOND_JACOBI = 0, /* point Jacobi, as the reference's DPCG (default) */
  MICROPP3_PRECOND_MG = 1,     /* geometric multigrid V-cycle: trilinear transfers, Galerkin coarse operators,
                                * Jacobi smoothing with the safeguarded diagonal max(a_ii / 0.6, 0.55 sum_j
                                * |a_ij|); every axis coarsens to ceil(elements / 2).  Needs at least 4 elements
                                * along every axis and more than 4 along one.  A solve that reaches 100
                                * iterations is redone with Jacobi. */
  MICROPP3_PRECOND_MG_HALF = 2 /* MICROPP3_PRECOND_MG whose two fine-level smoothing passes read an FP16 copy of
                                * the fine operator (scaled by a power of two), half the bytes of the FP32 values;
                                * the CG itself keeps the FP32 operator */
};

/* Per-RVE status word of the last homogenize(). */
enum {
  MICROPP3_STATUS_OK = 0,
  MICROPP3_STATUS_NEWTON_MAX_ITS = 1, /* Newton stopped at nr_max_its without meeting its tolerance */
  MICROPP3_STATUS_CG_MAX_ITS = 2,     /* a linear solve stopped at cg_max_its */
  MICROPP3_STATUS_NONFINITE = 4       /* a residual norm or an average stress was NaN or Inf */
};

/* Full construction parameters: the fields of micropp_params_t (types.hpp:43-63) in C form, plus the
 * GB300 options.  Fill with micropp3_config_default() and override. */
struct micropp3_config {
  int ngp;
  int size[3];            /* nodes per axis (elements + 1) */
  int micro_type;         /* MIC_* (types.hpp:85-99) */
  double geo_params[4];
  struct material_base materials[3];
  const int *coupling;    /* ngp entries; NULL = FE_ONE_WAY everywhere (micropp.cpp:88-96) */
  int subiterations;
  int nsubiterations;
  int mpi_rank;
  int nr_max_its;
  double nr_max_tol;
  double nr_rel_tol;
  int cg_max_its;         /* honoured (the reference ignores it and uses CG_MAX_ITS = 1000) */
  double cg_abs_tol;      /* honoured (reference: CG_ABS_TOL = 1e-50) */
  double cg_rel_tol;      /* honoured (reference: CG_REL_TOL = 1e-5) */
  int calc_ctan_lin;
  int use_A0;             /* FP64 form: the first its_with_A0 Newton iterations solve with the Jacobian at
                           * u = 0 (micropp.cpp:128-143, solve.cpp:55-66); ignored by the mixed form */
  int its_with_A0;
  int lin_stress;
  int write_log;
  const int *elem_type;   /* optional element phase map, nelem entries in glo_elem order (0, 1 or 2) */
  int precision;          /* MICROPP3_FP64 | MICROPP3_MIXED */
  int ctan_mode;          /* MICROPP3_CTAN_PERTURB | MICROPP3_CTAN_IMPLICIT */
  int precond;            /* MICROPP3_PRECOND_*: preconditioner of the FP32 solves (mixed-form Newton, implicit
                           * ctan); the FP64 Newton always uses the reference's Jacobi CG */
  int reserved[3];        /* zero */
};

/* The reference defaults (types.hpp:43-63 with params.hpp:32-35 and ell.hpp:33-35), FP64, perturbation
 * ctan. */
void micropp3_config_default(struct micropp3_config *cfg);

/* Construct from the full parameter set.  On failure self->ptr is NULL and micropp3_last_error() says why. */
void micropp3_new_ext(struct micropp3 *self, const struct micropp3_config *cfg);

/* Message of the last failure in this thread ("" if none), and its reset. */
const char *micropp3_last_error(void);
void micropp3_clear_error(void);

/* Homogenize several handles at once (RVEs of different sizes, microstructures or materials): each handle's
 * Gauss points form one batch on the handle's own stream, and the handles run concurrently from worker
 * threads.  Do not use the handles from another thread meanwhile. */
void micropp3_homogenize_many(struct micropp3 *const *handles, int n);

/* Status word (MICROPP3_STATUS_*) of macro point gp after the last homogenize(). */
int micropp3_get_status(const struct micropp3 *self, int gp_id);

/* Newton iterations and CG iterations of the last main solve of gp. */
void micropp3_get_newton(const struct micropp3 *self, int gp_id, int *its, int *solver_its, int *converged);

/* Sizes: number of elements and of displacement unknowns of one RVE. */
int micropp3_get_nelem(const struct micropp3 *self);
int micropp3_get_nndim(const struct micropp3 *self);

/* Copies of device state.  which = 0 selects vars_n / u_n, 1 selects vars_k / u_k.  Internal variables are
 * 7 doubles per Gauss point in the reference order (params.hpp:41); zeros while the point is linear. */
void micropp3_get_vars(const struct micropp3 *self, int gp_id, int which, double *out);
void micropp3_get_u(const struct micropp3 *self, int gp_id, int which, double *out);
void micropp3_get_elem_type(const struct micropp3 *self, int *out);
void micropp3_get_ctan_lin(const struct micropp3 *self, double *out36);

/* Levels of the multigrid preconditioner in use (0: Jacobi). */
int micropp3_get_mg_levels(const struct micropp3 *self);

/* Device time of the last homogenize() (CUDA events on the handle's stream), in milliseconds. */
double micropp3_last_homogenize_ms(const struct micropp3 *self);

/* Kernel timing.  When enabled, every launch of the named kernel family is bracketed by CUDA events on the
 * launching stream; micropp3_kernel_stats returns the launch count, the summed device time (ms) and the
 * algorithmic bytes moved by those launches.  Families: "spmv" (the Newton CG's SpMV), "cg_update" (its two
 * vector kernels), "spmv6" and "cg6_update" (the same for the 6-RHS tangent CG), "mg" and "mg6" (the two
 * fine-level operator passes of the multigrid V-cycles of the two CGs), "mg_coarse" (the rest of the V-cycles),
 * "assembly" (with the multigrid Galerkin operators), "residual". */
void micropp3_set_kernel_timing(struct micropp3 *self, int enable);
/* CUDA graphs: the CG iterations run in chunks captured once per (solver, batch size) and replayed
 * (default on; chunks are launched directly while kernel timing is on). */
void micropp3_set_cuda_graphs(struct micropp3 *self, int enable);
int micropp3_kernel_stats(const struct micropp3 *self, const char *family, long *launches, double *ms,
                          double *bytes);

/* Jacobi-preconditioned CG on a stencil ELL matrix held in device memory; the counterpart of the reference's
 * ell_solve_cgpd (ell.hpp:63, ell.cpp:66-122): x0 = 0, stop when ||z|| < abs_tol or ||z|| < rel_tol * ||z0||,
 * or after max_its iterations; *its receives the iteration count.  The work vectors are allocated on the
 * device for the duration of the call.
 *   nodes  grid of nodes nx, ny, nz (3 unknowns per node, nrow = 3 nx ny nz)
 *   vals   243 * np doubles, np = nx ny nz rounded up to a multiple of 32: entry (s, fi, fj) of node n at
 *          vals[(s*9 + fi*3 + fj) * np + n], stencil slot s = 9 (dz+1) + 3 (dy+1) + (dx+1) for the neighbour
 *          at offset (dx, dy, dz).  Rows of boundary nodes are identity rows; their entries are not read.
 *   b, x   nrow doubles, node-interleaved (row = 3 n + d)
 *   stream a cudaStream_t (NULL: the default stream)
 * Returns 0, -1 for invalid arguments, or the CUDA error code. */
int micropp3_ell_solve_cgpd(const int nodes[3], const double *vals, const double *b, double *x, double rel_tol,
                            double abs_tol, int max_its, int *its, void *stream);

/* The same solve as micropp3_ell_solve_cgpd, for callers that must not allocate device memory while they
 * run (a code that has already handed the device to its own memory pool, or a time step that must not wait
 * on the allocator).  This entry point has no counterpart in the reference.  Its work vectors live in one
 * fixed array of device memory that the library holds on every GPU where it is loaded, until the process
 * exits (about 16 MB), so the grid may have at most MICROPP3_NOALLOC_MAX_NODES nodes (50 x 50 x 50);
 * larger grids return -3.  The caller passes vals, b and x as for micropp3_ell_solve_cgpd.  Each call looks
 * up the array's address on the current device; the first call on a device also loads the library's device
 * code there, so make it before any stream capture.  The call returns when the solve has finished (it
 * synchronises the stream).  All calls share the array and find the previous call's data in it: calls that
 * overlap on the GPU (other host threads, other streams) race and must be serialised.
 * Returns 0, -1 for invalid arguments, -3 for a grid over the limit, or the CUDA error code. */
#define MICROPP3_NOALLOC_MAX_NODES 131072
int micropp3_ell_solve_cgpd_noalloc(const int nodes[3], const double *vals, const double *b, double *x,
                                    double rel_tol, double abs_tol, int max_its, int *its, void *stream);

/* Reverse-mode gradients of a load path (no counterpart in the reference, which has no derivatives other
 * than ctan).  micropp3_path_forward runs the RVE of this handle from the undeformed state (zero history)
 * through nsteps macro strains strains[nsteps][6], accepting every step, with the per-phase material
 * parameters params[3][5] = (E, nu, Xt, Sy, Ka) in place of the handle's (phase types and all other settings
 * are the handle's; Newton is the FP64 plain form at the handle's tolerances, with the exact consistent
 * tangent).  It writes the average stress
 * of every step to sigma[nsteps][6] and keeps the state before every checkpoint_every-th step.
 * micropp3_path_vjp then returns, for L = sum_n gsigma[n] . sigma[n], grad_params[3][5] = dL/dparams and, if
 * grad_strains is not NULL, grad_strains[nsteps][6] = dL/dstrains[n]: an adjoint solve per step on the
 * exact consistent tangent, the history sensitivities carried backwards, each segment recomputed from its
 * checkpoint.  Entries of a parameter a phase's law does not use are 0.
 * Both return 0, 1 when a Newton step (forward) or an adjoint solve (reverse) did not converge, -2 on an
 * error (see micropp3_last_error). */
int micropp3_path_forward(struct micropp3 *self, int nsteps, const double *strains, const double *params,
                          int checkpoint_every, double *sigma);
int micropp3_path_vjp(struct micropp3 *self, const double *gsigma, double *grad_params, double *grad_strains);
/* Newton record of one step of the last micropp3_path_forward: iterations, CG iterations, status (bit 0:
 * converged, bit 1: a CG solve stopped at cg_max_its) and |b| / |b0| of the last residual. */
void micropp3_path_newton(const struct micropp3 *self, int step, int *its, int *cg_its, int *status,
                          double *rel_norm);

/* Totals since construction: CG iterations summed over the handle's RVEs, and kernels launched. */
long micropp3_total_cg_its(const struct micropp3 *self);
long micropp3_kernel_launches(const struct micropp3 *self);

#ifdef __cplusplus
}
#endif
#endif
