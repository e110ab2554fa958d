// Device helpers shared by the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include "bsl_internal.h"

namespace bsl {

constexpr int kThreads = 256;

inline int grid_for(long long n) {
  long long g = (n + kThreads - 1) / kThreads;
  return (int)(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------
// reductions: block sum, then the last block to finish sums the per-block
// partials in a fixed order (deterministic, no second launch).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (wid == 0) v = warp_sum(v);
  return v;  // valid in thread 0
}

// Stores this block's partial; returns true (in every thread) for the last
// block, which then holds the grand total in *total (thread 0 only).
__device__ __forceinline__ bool reduce_grid(double part, double* partials, unsigned int* counter, double* total) {
  __shared__ bool last;
  double s = block_sum(part);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s;
    __threadfence();
    const unsigned int prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc = 0.0;
  for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x) acc += __ldcg(partials + b);
  acc = block_sum(acc);
  if (threadIdx.x == 0) {
    *total = acc;
    *counter = 0u;
  }
  return true;
}

}  // namespace bsl
