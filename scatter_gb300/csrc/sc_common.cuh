// Shared helpers for the scatter_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/scatter_gb300.h"

namespace sc {

constexpr int kWarp = 32;

// Records the last CUDA error text for sc_last_error().
void set_last_error(const char* where, cudaError_t e);
// Records a message (no CUDA error) for sc_last_error().
void set_last_message(const char* text);

inline int check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(where, e);
    return SC_CUDA_ERROR;
  }
  return SC_OK;
}

inline int check(cudaError_t e, const char* where) {
  if (e != cudaSuccess) {
    set_last_error(where, e);
    return SC_CUDA_ERROR;
  }
  return SC_OK;
}

inline unsigned grid_for(int64_t n, int threads, int64_t cap = 152 * 64) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of one double per thread (blockDim.x multiple of 32, <= 1024).
// Result valid in thread 0.  `sh` has at least 32 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    s = lane < nw ? sh[lane] : 0.0;
    s = warp_sum(s);
  }
  return s;
}

}  // namespace sc
