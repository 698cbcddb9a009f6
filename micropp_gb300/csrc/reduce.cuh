// reduce.cuh -- deterministic block and grid reductions.
//
// A grid reduction is "last block done": every block reduces its K values with warp shuffles, writes them
// to its own slot of a partials array, fences, and takes a ticket; the block that draws the last ticket sums
// all partials in a fixed order and publishes the result.  The result is bitwise reproducible from run to
// run, and no kernel ever waits on another block.
//
// Two entry precisions: grid_sum takes FP64 per-thread values; grid_sum_f takes FP32 per-thread partials
// (a thread's sum over its few rows), adds them in FP32 across the 32 lanes of a warp and in FP64 from the
// warp sums up.  The FP64 pipe of the GPU runs at 1/64 of the FP32 rate, so FP64 per-row accumulation and
// FP64 shuffles cost more than the memory traffic of a vector update; grid_sum_f keeps FP64 for the part of
// the sum that has many terms.
#pragma once

#include "device.cuh"
#include "df.cuh"

namespace mgb {

template <int K>
__device__ __forceinline__ void warp_sum(double (&v)[K]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
}

template <int K>
__device__ __forceinline__ void warp_sum(float (&v)[K]) {
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

// Block sum of FP32 per-thread partials: FP32 within each warp, FP64 across the warps, value k by thread k
// (one FP64 add per warp and value, issued by K lanes together rather than by one thread in turn).  The FP64
// result is valid in thread 0.  `sh` holds 32*K doubles: the warp sums as floats in its first half, the block
// sums as doubles in its second.
template <int K>
__device__ __forceinline__ void block_sum_f(float (&v)[K], double (&out)[K], double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  float *shf = reinterpret_cast<float *>(sh);
  double *shd = sh + 16 * K;
  warp_sum<K>(v);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) shf[wid * K + k] = v[k];
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double a = (double)shf[k];
    for (int w = 1; w < nw; ++w) a += (double)shf[w * K + k];
    shd[k] = a;
  }
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = shd[k];
}

// Second half of a grid reduction: `v` holds the block's sums in thread 0.  Returns true in the last block,
// where `total` (valid in every thread of that block) holds the sum over the blocks of the instance.
template <int K>
__device__ __forceinline__ bool grid_finish(const double (&v)[K], double *sh, double *red, unsigned int *ticket,
                                            int nblocks, double (&total)[K]) {
  __shared__ bool last;
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

// Grid reduction over the blocks of one instance (blockIdx.x = 0..nblocks-1) of FP64 per-thread values.
template <int K>
__device__ __forceinline__ bool grid_sum(double (&v)[K], double *red, unsigned int *ticket, int nblocks,
                                         double (&total)[K]) {
  __shared__ double sh[32 * K];
  block_sum<K>(v, sh);
  return grid_finish<K>(v, sh, red, ticket, nblocks, total);
}

// Grid reduction of FP32 per-thread partials (FP32 within a warp, FP64 above).
template <int K>
__device__ __forceinline__ bool grid_sum_f(float (&v)[K], double *red, unsigned int *ticket, int nblocks,
                                           double (&total)[K]) {
  __shared__ double sh[32 * K];
  double bs[K];
  block_sum_f<K>(v, bs, sh);
  __syncthreads();  // sh is reused by the last block
  return grid_finish<K>(bs, sh, red, ticket, nblocks, total);
}

// Grid reduction of double-float per-thread values: double-float within a warp (FP32 operations), FP64 from
// the warp sums up (value k by thread k, as block_sum_f).
template <int K>
__device__ __forceinline__ bool grid_sum_df(dfl (&v)[K], double *red, unsigned int *ticket, int nblocks,
                                            double (&total)[K]) {
  __shared__ double sh[32 * K];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const dfl u{__shfl_down_sync(0xffffffffu, v[k].h, o), __shfl_down_sync(0xffffffffu, v[k].l, o)};
      v[k] = v[k] + u;
    }
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sh[wid * K + k] = df_to_double(v[k]);
  __syncthreads();
  __shared__ double shd[K];
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double a = sh[k];
    for (int w = 1; w < nw; ++w) a += sh[w * K + k];
    shd[k] = a;
  }
  __syncthreads();
  double bs[K];
#pragma unroll
  for (int k = 0; k < K; ++k) bs[k] = shd[k];
  return grid_finish<K>(bs, sh, red, ticket, nblocks, total);
}

}  // namespace mgb
