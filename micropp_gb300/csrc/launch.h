// launch.h -- the internal C-ABI layer between the host engine (C++) and the CUDA kernels.
//
// Every entry launches one stage of the homogenization over a batch of instances on a stream and returns
// the cudaError_t of the launch (0 on success).  `insts` is a device array of per-instance views, `list` a
// device array of the `nlist` instance indices that take part.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "device.cuh"

#ifdef __cplusplus
extern "C" {
#endif

int mgb_launch_set_bc(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
int mgb_launch_add_du(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
int mgb_launch_copy(int n, const double *const *src, double *const *dst, const int *list, int nlist, cudaStream_t s);
// form: 1 = the element residual by B-matrix products in the reference's order (the FP64 form); 0 = by sum
// factorisation in FP64 (the mixed form with a J2 phase); 2 = by sum factorisation in double-float arithmetic
// (the mixed form with elastic and damage phases only).
int mgb_launch_residual(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const double *dsh,
                        const mgb::Inst *insts, const int *list, int nlist, int form, cudaStream_t s);
int mgb_launch_assembly(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const double *dsh,
                        const double *ke_phase, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
// FP64 Jacobian with the exact Gauss-point tangents (forward-mode dual numbers), for the adjoint.
int mgb_launch_assembly_dual(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const double *dsh,
                             const double *ke_phase, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
int mgb_launch_evolve(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const double *dsh,
                      const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
int mgb_launch_elem_fields(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const double *dsh,
                           const double *u, const double *vars, double ivol, double *fields, cudaStream_t s);
int mgb_launch_cg_setup(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
int mgb_launch_cg_spmv(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
int mgb_launch_cg_update(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
int mgb_launch_cg_pupdate(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist,
                          unsigned int *active_count, cudaStream_t s);

int mgb_launch_assembly32(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const double *dsh,
                          const float *ke_phase, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
// FP32 Jacobian by node gather (every phase elastic or damage): k0g = wg B_g^T C B_g per phase and Gauss
// point [3][8][576], kesum = its sum over g per phase [3][576], dsh32 = the shape-function gradients [8][24].
// sdiag = 1: also the multigrid's level-0 smoother diagonal, as mgb_launch_mg_sdiag(l = 0, omega, csafe).
int mgb_launch_assembly_gather32(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const float *k0g,
                              const float *kesum, const float *dsh32, const mgb::Inst *insts, const int *list,
                              int nlist, float omega, float csafe, int sdiag, cudaStream_t s);
// mg = 1: a V-cycle and mgb_launch_mg_post0 with setup = 1 follow.
int mgb_launch_cg32_setup(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int mg,
                          cudaStream_t s);
// block: 64, 128 or 256 threads (any other value: 128).
int mgb_launch_cg32_spmv(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int block,
                         cudaStream_t s);
// mg = 1: a V-cycle and mgb_launch_mg_post0 follow (they set rz and beta).
int mgb_launch_cg32_update(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int mg,
                           cudaStream_t s);
int mgb_launch_cg32_pupdate(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist,
                            unsigned int *active_count, cudaStream_t s);
int mgb_launch_add_du32(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
// CG states of the listed instances at the start of a solve, from a device array of relative tolerances.
int mgb_launch_cg32_init(const mgb::Inst *insts, const int *list, int nlist, const double *rel_tol, double abs_tol,
                         int max_its, cudaStream_t s);
// *p = 0 (a kernel, so that it can sit in a conditional node's body).
int mgb_launch_zero_u32(unsigned int *p, cudaStream_t s);
// The condition of a captured CG loop (a WHILE node): continue while *count != 0 and fewer than cap chunks ran.
int mgb_launch_cg_continue(cudaGraphConditionalHandle h, const unsigned int *count, unsigned int *chunks,
                           unsigned int cap, cudaStream_t s);
int mgb_launch_axpy_du32(const mgb::MeshDev *m, double *u, const float *du, double a, cudaStream_t s);
// near: the interior nodes with a boundary neighbour (the only nonzero rows of f_i = -K_IB w_i), nnear of them.
int mgb_launch_t6_rhs(const mgb::MeshDev *m, const int *near, int nnear, const mgb::Inst *insts, const int *list,
                      int nlist, cudaStream_t s);
int mgb_launch_t6_residual(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int x_zero,
                           int mg, cudaStream_t s);
int mgb_launch_cg6_spmv(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int block,
                        cudaStream_t s);
int mgb_launch_cg6_update(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int mg,
                          cudaStream_t s);
int mgb_launch_cg6_pupdate(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist,
                           unsigned int *active_count, cudaStream_t s);
int mgb_launch_t6_accumulate(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist,
                             cudaStream_t s);
// ctan in the energy form from element energies (elastic and damage phases: a symmetric tangent).
int mgb_launch_ctan_energy(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const float *dsh32,
                           const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
// ctan as the FP64 Gauss-point average of the tangent fields' stresses (a J2 phase: a non-symmetric tangent).
int mgb_launch_ctan_avg(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const double *dsh,
                        const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);

// Geometric multigrid preconditioner of the mixed form's FP32 CG (mg_kernels.cu).  mf / mc: the grids of levels
// lf and lf + 1; nr: 1 (the Newton CG's vectors) or 6 (the tangent CG's).  src / dst of the Jacobi sweep:
// 0 = x, 1 = y, 2 = t of level l >= 1.
// One 1-D step of the separable Galerkin product (axis 0, 1, 2): operator on grid mi -> grid mo.  src / dst:
// 0 = level lf's operator, 1 / 2 = the intermediate operators, 3 = level lf + 1's operator.
int mgb_launch_mg_rap1(const mgb::MeshDev *mi, const mgb::MeshDev *mo, const mgb::Inst *insts, const int *list,
                       int nlist, int lf, int axis, int src, int dst, cudaStream_t s);
// Inverse safeguarded smoother diagonal of level l: 1 / max(a_dd / omega, c sum_j |a_dj|).
int mgb_launch_mg_sdiag(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int l,
                        float omega, float c, cudaStream_t s);
// block: threads per block of the 6-RHS level-0 residual (64, 128 or 256; two nodes per thread).  half: the
// level-0 passes read the FP16 copy of the fine operator (MgInst::vals16).
int mgb_launch_mg_resid(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int nr, int l,
                        int block, int half, cudaStream_t s);
// The FP16 copy of the level-0 operator, scale16 x vals32, of the listed instances.
int mgb_launch_mg_half0(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
int mgb_launch_mg_restrict(const mgb::MeshDev *mf, const mgb::MeshDev *mc, const mgb::Inst *insts, const int *list,
                           int nlist, int nr, int lf, float omega, cudaStream_t s);
int mgb_launch_mg_prolong(const mgb::MeshDev *mf, const mgb::MeshDev *mc, const mgb::Inst *insts, const int *list,
                          int nlist, int nr, int lf, cudaStream_t s);
int mgb_launch_mg_jacobi(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int nr, int l,
                         int src, int dst, float omega, cudaStream_t s);
// `pairs` pairs of Jacobi sweeps x -> y -> x on level l >= 1 of at most kMgCoarseNodes nodes, in one launch
// (one block per instance, the level in shared memory when it fits); the same result as 2 x pairs
// mgb_launch_mg_jacobi calls.  mgb_mg_init_attributes must have run on the device first.
// The kernel attributes the multigrid launches need (the shared-memory size of the coarse sweeps), on the current
// device; call before the first V-cycle and outside any stream capture.
int mgb_mg_init_attributes();
int mgb_launch_mg_coarse_sweeps(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int nr,
                                int l, int pairs, float omega, cudaStream_t s);
// block: threads per block of the 6-RHS form (64, 128 or 256; two nodes per thread), as mgb_launch_mg_resid.
int mgb_launch_mg_post0(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, int nr,
                        float omega, int setup, int block, int half, cudaStream_t s);

// Adjoint of a load path (adjoint_kernels.cu); one instance (list[0]).
int mgb_launch_node_gather(const mgb::MeshDev *m, const mgb::Inst *insts, const int *list, int nlist, cudaStream_t s);
int mgb_launch_adj_rhs(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const double *dsh,
                       const mgb::Inst *insts, const int *list, const mgb::AdjStep *st, cudaStream_t s);
int mgb_launch_adj_back(const mgb::MeshDev *m, const mgb::Mats *mats, const int8_t *etype, const double *dsh,
                        const mgb::Inst *insts, const int *list, const mgb::AdjStep *st, cudaStream_t s);
int mgb_launch_affine_add(const mgb::MeshDev *m, double *u, const double *deps, cudaStream_t s);
int mgb_launch_axpy(int n, double *x, const double *y, double a, cudaStream_t s);
int mgb_launch_bicg_init(const mgb::MeshDev *m, const mgb::AdjDev *A, cudaStream_t s);
int mgb_launch_bicg_iter(const mgb::MeshDev *m, const mgb::AdjDev *A, unsigned int *active, int transpose,
                         cudaStream_t s);

#ifdef __cplusplus
}
#endif
