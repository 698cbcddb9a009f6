// noalloc.cu -- micropp3_ell_solve_cgpd_noalloc: the stencil-ELL DPCG solve without any device allocation.
//
// Who needs it: a caller that is not allowed to allocate GPU memory at solve time -- for instance a
// macro-scale solver that has reserved the whole device for its own memory pool before the first step, or a
// time step that must not stall on the allocator.  micropp3_ell_solve_cgpd allocates its work vectors with
// cudaMalloc on every call; this variant takes them from one fixed array of device memory that belongs to
// the library and exists on every GPU that loads it, from then until the process exits.
//
// Limit: at most MICROPP3_NOALLOC_MAX_NODES (131,072) nodes, i.e. RVEs up to 50 x 50 x 50 nodes (49^3
// elements); the array holds five work vectors of 3 * 131,072 doubles plus the reduction partials and a few
// counters, about 16.3 MB.
//
// Sharing: every call uses the same array and leaves its contents behind; the counters and the result record
// that must start at zero are cleared at the start of each call.  Two calls whose work overlaps on the GPU --
// from two host threads, or on two streams -- race on the array and give wrong results; serialise them.
//
// Set-up: each call resolves the device address of the array on the current device (cudaGetSymbolAddress)
// before it launches anything.  The address is not cached: a cudaDeviceReset or a re-created primary context
// reloads the library's device code and moves the array, and a kept address would then point at freed
// memory.  The first call on a device also loads the device code there; make that first call before any
// stream capture.  The call returns once the solve has finished (it synchronises the stream).
#include <cuda_runtime.h>

#include <cstdio>
#include <stdexcept>

#include "device.cuh"
#include "ell_api.h"
#include "micropp_gb300.h"

namespace mgb {

namespace {

constexpr size_t kNaRows = 3 * (size_t)MICROPP3_NOALLOC_MAX_NODES;
constexpr size_t kNaBlocks = kNaRows / kNodeBlock + 8;  // largest reducing grid of the CG kernels
constexpr size_t kNaVecBytes = kNaRows * sizeof(double);
constexpr size_t kNaOffRed = 5 * kNaVecBytes;
constexpr size_t kNaOffTicket = kNaOffRed + kNaBlocks * kRedStride * sizeof(double);
constexpr size_t kNaOffCount = kNaOffTicket + 256;
constexpr size_t kNaOffCg = kNaOffCount + 256;
constexpr size_t kNaOffOut = kNaOffCg + 256;
constexpr size_t kNaOffInst = kNaOffOut + 512;
constexpr size_t kNaOffList = kNaOffInst + 512;
constexpr size_t kNaBytes = kNaOffList + 256;
static_assert(sizeof(CgState) <= 256 && sizeof(InstOut) <= 512 && sizeof(Inst) <= 512, "scratch record sizes");

// The library's scratch for the allocation-free solve (see the file comment for its size and sharing).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

// Clears the counters that each call needs at zero (reduction ticket, active-instance count).
__global__ void k_noalloc_clear(unsigned int *ticket, unsigned int *count) {
  if (threadIdx.x == 0) {
    *ticket = 0u;
    *count = 0u;
  }
}

// Device address of g_noalloc_scratch in the current context.  In host code the symbol's own name is a
// host-side stand-in, not a device address, so kernels are given only what this returns.
cudaError_t scratch_address(unsigned char **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = (unsigned char *)p;
  return cudaSuccess;
}

}  // namespace

}  // namespace mgb

using namespace mgb;

extern "C" int micropp3_ell_solve_cgpd_noalloc(const int nodes[3], const double *vals, const double *b, double *x,
                                               double rel_tol, double abs_tol, int max_its, int *its, void *stream) {
  if (!nodes || !vals || !b || !x || nodes[0] < 2 || nodes[1] < 2 || nodes[2] < 2 || max_its < 0) return -1;
  const long long nn = (long long)nodes[0] * nodes[1] * nodes[2];
  if (nn > MICROPP3_NOALLOC_MAX_NODES) {
    std::fprintf(stderr,
                 "micropp3_ell_solve_cgpd_noalloc: %lld nodes exceed the fixed scratch of %d nodes; "
                 "use micropp3_ell_solve_cgpd for larger grids\n",
                 nn, MICROPP3_NOALLOC_MAX_NODES);
    return -3;
  }
  unsigned char *base = nullptr;
  cudaError_t e = scratch_address(&base);
  if (e != cudaSuccess) return (int)e;
  cudaStream_t s = (cudaStream_t)stream;
  const MeshDev m = stencil_mesh(nodes);
  Inst I{};
  I.vals = const_cast<double *>(vals);
  I.b = const_cast<double *>(b);
  I.du = x;
  I.r = (double *)(base + 0 * kNaVecBytes);
  I.z = (double *)(base + 1 * kNaVecBytes);
  I.p = (double *)(base + 2 * kNaVecBytes);
  I.Ap = (double *)(base + 3 * kNaVecBytes);
  I.kinv = (double *)(base + 4 * kNaVecBytes);
  I.red = (double *)(base + kNaOffRed);
  I.ticket = (unsigned int *)(base + kNaOffTicket);
  I.cg = (CgState *)(base + kNaOffCg);
  I.out = (InstOut *)(base + kNaOffOut);
  Inst *d_inst = (Inst *)(base + kNaOffInst);
  int *d_list = (int *)(base + kNaOffList);
  unsigned int *d_count = (unsigned int *)(base + kNaOffCount);
  const int zero = 0;
  try {
    k_noalloc_clear<<<1, 32, 0, s>>>(I.ticket, d_count);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemsetAsync(I.out, 0, sizeof(InstOut), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_inst, &I, sizeof(Inst), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_list, &zero, sizeof(int), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return (int)e;
    const int n = run_dpcg(m, d_inst, d_list, d_count, I.cg, I.out, rel_tol, abs_tol, max_its, s);
    if (its) *its = n;
  } catch (const CudaFailure &f) {
    std::fprintf(stderr, "micropp3_ell_solve_cgpd_noalloc: %s\n", f.what());
    return (int)f.code;
  }
  return 0;
}
