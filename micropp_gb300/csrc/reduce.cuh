// reduce.cuh -- deterministic block and grid reductions (FP64).
//
// A grid reduction is "last block done": every block reduces its K values with warp shuffles, writes them
// to its own slot of a partials array, fences, and takes a ticket; the block that draws the last ticket sums
// all partials in a fixed order and publishes the result.  The result is bitwise reproducible from run to
// run, and no kernel ever waits on another block.
#pragma once

#include "device.cuh"

namespace mgb {

template <int K>
__device__ __forceinline__ void warp_sum(double (&v)[K]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
}

// Sum of v over the block; the result is valid in thread 0.  `sh` holds 32*K doubles.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  warp_sum<K>(v);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sh[wid * K + k] = v[k];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = (lane < nw) ? sh[lane * K + k] : 0.0;
    warp_sum<K>(v);
  }
}

// Grid reduction over the blocks of one instance (blockIdx.x = 0..nblocks-1).  Returns true in the last
// block, where `total` (valid in every thread of that block) holds the sum.
template <int K>
__device__ __forceinline__ bool grid_sum(double (&v)[K], double *red, unsigned int *ticket, int nblocks,
                                         double (&total)[K]) {
  __shared__ double sh[32 * K];
  __shared__ bool last;
  block_sum<K>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) red[(size_t)blockIdx.x * kRedStride + k] = v[k];
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    last = (t == (unsigned int)(nblocks - 1));
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] += __ldcg(&red[(size_t)b * kRedStride + k]);
  block_sum<K>(acc, sh);
  __shared__ double res[K];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) res[k] = acc[k];
    *ticket = 0u;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) total[k] = res[k];
  return true;
}

}  // namespace mgb
