// Device helpers shared by the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include "bsl_internal.h"

namespace bsl {

constexpr int kThreads = 256;

inline int grid_for(long long n) {
  long long g = (n + kThreads - 1) / kThreads;
  return (int)(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------
// FP64 <-> FP32 conversions with integer operations only.  GB300 executes FP64
// arithmetic at about one operation per clock per SM, so the mixed-precision
// kernels avoid FP64 instructions per vector element: conversions run on the
// integer pipe and the Lanczos recurrence in double-float arithmetic below.
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
// Double-float arithmetic on the FP32 pipe.  A value is the unevaluated sum
// x + y of a float2 with |y| <= ulp(x)/2 (about 48 significant bits).
// Algorithms: Dekker's exact product and fast two-sum (Numer. Math. 18, 1971),
// Knuth's TwoSum, and the accurate addition of Hida, Li and Bailey's
// double-double library (ARITH-15, 2001) restated for FP32 components.  Every
// step uses the _rn intrinsics so that nothing is contracted or reassociated.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  float s1, s2, t1, t2;
  two_sum(a.x, b.x, s1, s2);
  two_sum(a.y, b.y, t1, t2);
  s2 = __fadd_rn(s2, t1);
  fast_two_sum(s1, s2, s1, s2);
  s2 = __fadd_rn(s2, t2);
  fast_two_sum(s1, s2, s1, s2);
  return make_float2(s1, s2);
}

__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  float s, t;
  fast_two_sum(p, e, s, t);
  return make_float2(s, t);
}

// Double-float addition without the second error term ("sloppy" addition,
// 11 operations): relative error ~2^-44 of |a| + |b| rather than of the sum;
// for adding terms whose own error is already larger than that.
__device__ __forceinline__ float2 df_add_fast(float2 a, float2 b) {
  float s, e;
  two_sum(a.x, b.x, s, e);
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  fast_two_sum(s, e, s, e);
  return make_float2(s, e);
}

// a * b + c
__device__ __forceinline__ float2 df_fma(float2 a, float2 b, float2 c) { return df_add(df_mul(a, b), c); }

// a * b + c with the fast addition: for accumulations and updates whose terms
// carry FP32-level noise of their own (relative error ~2^-44 of |a b| + |c|)
__device__ __forceinline__ float2 df_fma_fast(float2 a, float2 b, float2 c) { return df_add_fast(df_mul(a, b), c); }

// a^2 as a double-float (exact head product, 5 operations)
__device__ __forceinline__ float2 df_sqr(float2 a) {
  const float p = __fmul_rn(a.x, a.x);
  float e = __fmaf_rn(a.x, a.x, -p);
  e = __fmaf_rn(__fmul_rn(2.f, a.x), a.y, e);
  float s, t;
  fast_two_sum(p, e, s, t);
  return make_float2(s, t);
}

__device__ __forceinline__ float2 df_scale2(float2 a, float g) {  // g a power of two: exact
  return make_float2(__fmul_rn(a.x, g), __fmul_rn(a.y, g));
}

// double-float nearest to an FP64 number (one FP64 subtraction)
__device__ __forceinline__ float2 df_of(double d) {
  const float hi = f32_round(d);
  return make_float2(hi, f32_round(d - f64_of(hi)));
}

__device__ __forceinline__ double f64_of_df(float2 a) { return f64_of(a.x) + f64_of(a.y); }

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

__device__ __forceinline__ float2 warp_sum_df(float2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = df_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)));
  return v;
}

// reduce_grid for double-float per-thread parts: the block sums run on the
// FP32 pipe (double-float shuffles), only one FP64 value per block is formed,
// and the last block adds the per-block values in FP64 in a fixed order.
// The same over `count` blocks that share partials and counter, this block
// being number `index` of them (a grouped launch reduces each problem over its
// own blocks); reduce_grid_df is the whole grid.
__device__ __forceinline__ bool reduce_group_df(float2 part, double* partials, unsigned int* counter,
                                                unsigned int count, unsigned int index, double* total) {
  __shared__ float2 shd[32];
  __shared__ bool last_df;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2 v = warp_sum_df(part);
  if (lane == 0) shd[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = warp_sum_df(lane < nw ? shd[lane] : make_float2(0.f, 0.f));
    if (lane == 0) {
      partials[index] = f64_of_df(v);
      __threadfence();
      last_df = (atomicAdd(counter, 1u) == count - 1);
    }
  }
  __syncthreads();
  if (!last_df) return false;
  __threadfence();
  double acc = 0.0;
  for (unsigned int b = threadIdx.x; b < count; b += blockDim.x) acc += __ldcg(partials + b);
  acc = block_sum(acc);
  if (threadIdx.x == 0) {
    *total = acc;
    *counter = 0u;
  }
  return true;
}

__device__ __forceinline__ bool reduce_grid_df(float2 part, double* partials, unsigned int* counter,
                                               double* total) {
  return reduce_group_df(part, partials, counter, gridDim.x, blockIdx.x, total);
}

// Stores this block's partial; returns true (in every thread) for the last of
// `count` blocks (this one number `index`), which then holds the grand total in
// *total (thread 0 only).
__device__ __forceinline__ bool reduce_group(double part, double* partials, unsigned int* counter,
                                             unsigned int count, unsigned int index, double* total) {
  __shared__ bool last;
  double s = block_sum(part);
  if (threadIdx.x == 0) {
    partials[index] = s;
    __threadfence();
    const unsigned int prev = atomicAdd(counter, 1u);
    last = (prev == count - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc = 0.0;
  for (unsigned int b = threadIdx.x; b < count; b += blockDim.x) acc += __ldcg(partials + b);
  acc = block_sum(acc);
  if (threadIdx.x == 0) {
    *total = acc;
    *counter = 0u;
  }
  return true;
}

__device__ __forceinline__ bool reduce_grid(double part, double* partials, unsigned int* counter, double* total) {
  return reduce_group(part, partials, counter, gridDim.x, blockIdx.x, total);
}

// ---------------------------------------------------------------------------
// End of the double-float Lanczos update (the last block, thread 0), given
// total = ||R_new||^2 with R_new = g (R - alpha c V), g = 2^e: beta, its
// history, the next folded scales and the next g.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void finish_update_pair(double total, int e, double* scalars, double* hist, int hist_stride,
                                                   int j, int* status) {
  const double alpha = scalars[0], sv = scalars[4], sr = scalars[5];
  const double sr_g = ldexp(sr, -e);  // r = (sr / g) R_new
  const double b2 = sr_g * sr_g * total;
  const double b = sqrt(b2);
  scalars[1] = b;
  scalars[2] = b2;
  scalars[3] = 1. / b;
  hist[hist_stride + j] = b;
  hist[2 * hist_stride + j] = b2;
  const double sv_n = sr_g / b, sr_n = -b * sv;
  scalars[4] = sv_n;
  scalars[5] = sr_n;
  scalars[6] = sv_n / sr_n;
  scalars[7] = sv_n * sr_n;
  reinterpret_cast<float2*>(scalars)[8] = df_of(sv_n / sr_n);
  // next update: ||R_next|| = beta_{j+1} / |sr_n| ~ b / |sr_n|, so g = 2^(ilogb(sr_n) - ilogb(b))
  int en = (b > 0.0 && isfinite(b) && sr_n != 0.0) ? ilogb(sr_n) - ilogb(b) : 0;
  reinterpret_cast<int*>(scalars)[20] = max(-60, min(60, en));
  if (!(b > 0.0) || !isfinite(b) || !isfinite(alpha)) {
    if (status[0] == 0) status[1] = j;
    status[0] = 1;
  }
}

// ---------------------------------------------------------------------------
// Deferred Lanczos reductions (graph-replayed iterations of the double-float
// path).  Instead of the last CTA of a kernel summing everyone's partial sum
// while the rest of the GPU idles, the CTAs only store their block totals; the
// total is formed by a later kernel that runs anyway: alpha by every CTA of
// the update (each the same fixed-order sum, so all agree), beta by one CTA
// of the next iteration's x/y kinetic (or a one-CTA kernel after the last
// iteration).  Layout in the partials buffer: alpha's block totals from
// index 0, beta's from kBetaPartials; scalars' int slots: the pending flag of
// a deferred beta and the count of alpha's block totals.
// ---------------------------------------------------------------------------
constexpr int kPendingSlot = 24;     // int slot of scalars: 1 while a beta total is deferred
constexpr int kAlphaCountSlot = 25;  // int slot of scalars: alpha's block totals

// this block's double-float total (all threads call; the value in thread 0)
__device__ __forceinline__ double block_total_df(float2 part) {
  __shared__ float2 shb[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2 v = warp_sum_df(part);
  __syncthreads();
  if (lane == 0) shb[wid] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = (wid == 0 && lane < nw) ? shb[lane] : make_float2(0.f, 0.f);
  if (wid == 0) v = warp_sum_df(v);
  return f64_of_df(v);
}

// sum of parts[0..count) in a fixed order by `nthreads` threads (thread index
// t) that synchronise on named barrier `bar`; the total in every thread
__device__ __forceinline__ double sum_partials(const double* parts, int count, int t, int nthreads, int bar,
                                               double* shared8) {
  double acc = 0.0;
  for (int b = t; b < count; b += nthreads) acc += __ldcg(parts + b);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((t & 31) == 0) shared8[t >> 5] = acc;
  asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
  double total = 0.0;
  for (int w = 0; w < nthreads / 32; ++w) total += shared8[w];
  asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
  return total;
}

// The deferred beta of the last update, if one is pending: its block totals
// summed, then beta, its history and the next scales (finish_update_pair) and
// the iteration counter advanced.  Called by `nthreads` threads (index t) that
// synchronise on named barrier `bar`.
__device__ __forceinline__ void finish_deferred_beta(const double* parts, int count, double* scalars, double* hist,
                                                     int hist_stride, int* jdev, int* status, int t, int nthreads,
                                                     int bar, double* shared8) {
  int* si = reinterpret_cast<int*>(scalars);
  if (!*(volatile int*)(si + kPendingSlot)) return;  // the same value in every thread
  const double total = sum_partials(parts, count, t, nthreads, bar, shared8);
  if (t == 0) {
    const int j = *jdev;
    finish_update_pair(total, si[20], scalars, hist, hist_stride, j, status);
    *jdev = j + 1;
    si[kPendingSlot] = 0;
  }
}

// ---------------------------------------------------------------------------
// Programmatic dependent launch: the kernels of the Lanczos iteration are
// launched with programmatic stream serialization, so a kernel's CTAs may start
// (and run their prologue) while the previous kernel's last CTAs finish.
// pdl_wait() blocks until the previous kernel has completed and its memory is
// visible; every thread calls it before touching data another kernel writes or
// reads.  Without the launch attribute both are no-ops.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// launch with programmatic stream serialization
template <typename... K, typename... A>
cudaError_t launch_pdl(void (*kernel)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

}  // namespace bsl
