// ell_api.h -- internal interface of the standalone DPCG driver (ell_api.cpp).
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "device.cuh"

namespace mgb {

// A failed CUDA call inside the standalone solve; `code` is what the entry points return.
struct CudaFailure : std::runtime_error {
  cudaError_t code;
  CudaFailure(cudaError_t c, const char *what)
      : std::runtime_error(std::string(what) + ": " + cudaGetErrorString(c)), code(c) {}
};

// Mesh of an nx x ny x nz node grid (only the node counts matter to the CG kernels).
MeshDev stencil_mesh(const int nodes[3]);

// DPCG on the single instance d_inst[0] (listed by d_list) whose pointers are already set; allocates
// nothing.  Returns the iteration count; throws CudaFailure on a CUDA error.
int run_dpcg(const MeshDev &m, Inst *d_inst, int *d_list, unsigned int *d_count, CgState *d_cg, InstOut *d_out,
             double rel_tol, double abs_tol, int max_its, cudaStream_t s);

}  // namespace mgb
