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
// FP64 <-> FP32 conversions with integer operations only.  GB300 executes FP64
// arithmetic at about 1/64 of the FP32 rate, so the mixed-precision kernels
// keep FP64 instructions for the Lanczos recurrence and do conversions on the
// integer pipe.
// ---------------------------------------------------------------------------
// FP32 value of an FP64 number rounded to nearest, ties to even (the same as
// a hardware conversion for normal results); magnitudes below the FP32 normal
// range become signed zero.  Rounding rather than truncating matters: a
// truncated copy scales every H v by (1 - 2^-24) on average, which shifts high
// levels measurably.
__device__ __forceinline__ float f32_round(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned int hi = (unsigned int)(b >> 32);
  const unsigned int sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
  unsigned int mag = ((unsigned int)e << 23) | ((hi & 0xFFFFFu) << 3) | (unsigned int)((b >> 29) & 0x7u);
  const unsigned int rest = (unsigned int)(b & 0x1FFFFFFFull);  // the 29 discarded mantissa bits
  if (rest > 0x10000000u || (rest == 0x10000000u && (mag & 1u))) mag += 1u;  // carries into the exponent
  return __uint_as_float(sign | mag);
}

// Exact FP64 value of a normal FP32 number (FP32 subnormals become zero).
__device__ __forceinline__ double f64_of(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int e = (u >> 23) & 0xFFu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e == 0) return __longlong_as_double((long long)sign);
  const unsigned long long ee = (e == 255) ? 0x7FFull : (unsigned long long)(e - 127 + 1023);
  return __longlong_as_double((long long)(sign | (ee << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

// Error-free sum of two FP32 numbers: s + e == a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
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
