// cuda_util.hpp -- error checks and device allocation helpers of the host engine.
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

namespace mgb {

inline void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
  }
}

inline void check_launch(int e, const char *what) { check((cudaError_t)e, what); }

template <typename T>
inline T *dalloc(size_t n, const char *what) {
  void *p = nullptr;
  if (n == 0) n = 1;
  check(cudaMalloc(&p, n * sizeof(T)), what);
  return (T *)p;
}

inline void dfree(void *p) {
  if (p) cudaFree(p);
}

}  // namespace mgb
