// Sinc-DVR kinetic contractions on the fifth-generation tensor cores
// (tcgen05.mma kind::f16, accumulators in tensor memory), sm_103a, with
// exact accumulation.
//
// Reference: Tv_5D_oneCompositeIndex / Mv_5D_oneCompositeIndex,
// Hv-calculators/linRotor/cartSphBasis/HvCalc/linRotCartSphHvRoutines.cpp:1807-1969.
//
// Each CTA takes two grid planes at a time (padded to 64 x 64) and forms
// D[(plane, row)][col] = sum_q A[(plane, row)][q] T[col][q] as M = 128, N = 64,
// K = 64 products:
//   x (plane (y, x) of fixed (s, z)):  A[(p, y)][q] = v(p, y, q),  out(y, x) += sum_q v(y, q) Tx[x][q]
//   y (same plane, transposed):        A[(p, x)][q] = v(p, q, x),  out(y, x) += sum_q Ty[y][q] v(q, x)
//   z (plane (z, x) of fixed (s, y)):  A[(p, x)][q] = v(p, q, x),  out(z, x) += sum_q Tz[z][q] v(q, x)
//
// Exactness (error-free slicing after Ozaki, Ogita, Oishi and Rump,
// Numer. Algorithms 59, 2012, here with 8-bit fixed-point slices): each row of
// A is scaled by a power of two to below 1 in magnitude and cut into four
// 8-bit signed integer slices, A = 2^(e_row - 7) (a1 + 2^-8 a2 + 2^-16 a3 +
// 2^-24 a4) (32 bits relative to the row maximum: every FP32 value within 2^8
// of the row maximum is exact); T is scaled from its largest element and cut
// into four slices likewise.  The slices are small integers, exact in FP16,
// their products are exact, and every partial sum of one product class is an
// integer below 4 * 2^20: the FP32 accumulation in tensor memory is exact
// whatever its internal rounding, so the result carries no accumulation bias.
// The products of each scale class k + l share one accumulator (classes 0..3;
// the rest lies below 2^-32 of the row scale) and the four classes are combined
// on the CUDA cores into a double-float pair.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "bsl_internal.h"
#include "bsl_tc.cuh"

namespace bsl {
namespace {

constexpr int kVS = 4;                  // slices of v
constexpr int kTS = 4;                  // slices of T
constexpr uint32_t kTileA = 128 * 128;  // 16 KiB: 128 rows x 64 FP16 (one 128-byte swizzle atom per row)
constexpr uint32_t kTileB = 64 * 128;   // 8 KiB
constexpr int kRaw = 65;                // padded row of the raw plane buffer
constexpr int kStage = 65;              // padded row of the x-result staging buffer
constexpr int kPairs = 10;              // slice products (k, l) with k + l <= 3 (0-based), by class
__constant__ int8_t c_pk[kPairs] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};
__constant__ int8_t c_pl[kPairs] = {0, 1, 0, 2, 1, 0, 3, 2, 1, 0};

struct KinTC {
  const uint16_t* tslices;  // [kTS][64][64] FP16 bits, row = output index, column = q, zero padded
  int e_t;                  // T = 2^(e_t - 7) (b1 + 2^-8 b2 + 2^-16 b3 + 2^-24 b4)
  const float* v32;
  float2* out;
  int nx, ny, nz, nplanes;
  int* status;
};

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~(uintptr_t)1023);
}

// byte offset of the 16-byte chunk c (8 FP16 values) of row r in an SW128 K-major tile with K = 64
__device__ __forceinline__ uint32_t chunk_offset(int r, int c) { return (uint32_t)(r * 128 + ((c ^ (r & 7)) << 4)); }

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// exponent e with max|x| 2^-e in [0.5, 1); 0 for an all-zero row
__device__ __forceinline__ int row_exponent(float maxabs) {
  if (!(maxabs > 0.f)) return 0;
  return max(-100, ilogbf(maxabs) + 1);
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((min(max(e, -126), 127) + 127) << 23); }

// Slices of 8 consecutive values already multiplied by 2^(7 - e), written as
// one 16-byte chunk per slice.  Every step is exact except the last rounding.
__device__ __forceinline__ void write_slices(uint8_t* A, int row, int chunk, const float (&y)[8]) {
  float s[kVS][8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    float r = y[u];
    const float a1 = rintf(r);
    r = __fmul_rn(__fsub_rn(r, a1), 256.f);
    const float a2 = rintf(r);
    r = __fmul_rn(__fsub_rn(r, a2), 256.f);
    const float a3 = rintf(r);
    r = __fmul_rn(__fsub_rn(r, a3), 256.f);
    s[0][u] = a1;
    s[1][u] = a2;
    s[2][u] = a3;
    s[3][u] = rintf(r);
  }
  const uint32_t off = chunk_offset(row, chunk);
#pragma unroll
  for (int k = 0; k < kVS; ++k)
    *reinterpret_cast<uint4*>(A + k * kTileA + off) = make_uint4(pack_h2(s[k][0], s[k][1]), pack_h2(s[k][2], s[k][3]),
                                                                 pack_h2(s[k][4], s[k][5]), pack_h2(s[k][6], s[k][7]));
}

// D_c += A_k B_l^T for the ten slice products, class c = k + l in accumulator columns [64 c, 64 c + 64)
__device__ __forceinline__ void issue_products(uint32_t d, uint32_t a, uint32_t b) {
  const uint32_t idesc = tc::idesc_f16(128, 64);
#pragma unroll 1
  for (int pr = 0; pr < kPairs; ++pr) {
    const int k = c_pk[pr], l = c_pl[pr];
    const uint32_t dc = d + (uint32_t)(k + l) * 64u;
    const bool first = (pr == 0 || pr == 1 || pr == 3 || pr == 6);  // first product of its class
#pragma unroll
    for (int s = 0; s < 4; ++s)
      tc::mma_f16(dc, tc::sw128_desc(a + (uint32_t)k * kTileA + (uint32_t)s * 32u),
                  tc::sw128_desc(b + (uint32_t)l * kTileB + (uint32_t)s * 32u), idesc, (first && s == 0) ? 0u : 1u);
  }
}

// the four class accumulators of 16 consecutive columns combined into
// double-float pairs and multiplied by `scale` (a power of two)
__device__ __forceinline__ void load_pairs(uint32_t taddr, float scale, float2 (&out)[16]) {
  float c0[16], c1[16], c2[16], c3[16];
  tc::tmem_ld16(taddr, c0);
  tc::tmem_ld16(taddr + 64u, c1);
  tc::tmem_ld16(taddr + 128u, c2);
  tc::tmem_ld16(taddr + 192u, c3);
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    float h, e1, e2, l;
    two_sum(c0[u], __fmul_rn(c1[u], 0x1p-8f), h, e1);
    two_sum(h, __fmul_rn(c2[u], 0x1p-16f), h, e2);
    l = __fadd_rn(__fadd_rn(e1, e2), __fmul_rn(c3[u], 0x1p-24f));
    fast_two_sum(h, l, h, l);
    out[u] = make_float2(__fmul_rn(h, scale), __fmul_rn(l, scale));
  }
}

__device__ __forceinline__ void load_b(uint8_t* B, const uint16_t* src, int tid, int nthreads) {
  for (int e = tid; e < kTS * 64 * 8; e += nthreads) {  // kTS tiles of 64 rows x 8 chunks
    const int l = e >> 9, r = (e >> 3) & 63, c = e & 7;
    *reinterpret_cast<uint4*>(B + l * kTileB + chunk_offset(r, c)) =
        *reinterpret_cast<const uint4*>(src + ((size_t)l * 64 + r) * 64 + c * 8);
  }
}

// x and y contractions; out(y, x) = (Tx v + Ty v) as double-float pairs.  256 threads:
// threads 0-127 slice the rows (x operand), 128-255 the columns (y operand); in the
// epilogues warps w and w + 4 share the tensor-memory lanes 32 (w % 4) and split the columns.
__global__ void __launch_bounds__(256, 1) k_kin_xy_tc(KinTC a) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = align1024(smraw);
  uint8_t* Ax = sm;                                          // kVS tiles
  uint8_t* Ay = sm + kVS * kTileA;                           // kVS tiles
  uint8_t* B = sm + 2 * kVS * kTileA;                        // kTS tiles
  float* raw = reinterpret_cast<float*>(B + kTS * kTileB);  // [2][64][kRaw]
  float2* Xs = reinterpret_cast<float2*>(sm);               // [128][kStage] over the A tiles once consumed
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  __shared__ int ex[128], ey[128];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nx = a.nx, ny = a.ny;
  const long long psz = (long long)ny * nx;
  const int npairs = (a.nplanes + 1) / 2;
  load_b(B, a.tslices, tid, 256);
  if (tid == 0) {
    failed = 0;
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 512);
  // raw planes of one pair into shared memory (zero padded)
  auto load_raw = [&](int pair) {
#pragma unroll 1
    for (int pl = 0; pl < 2; ++pl) {
      const int plane = 2 * pair + pl;
      const bool pv = plane < a.nplanes;
      const float* src = a.v32 + (pv ? (long long)plane * psz : 0);
#pragma unroll 4
      for (int e = tid; e < 64 * 64; e += 256) {
        const int j = e >> 6, i = e & 63;
        raw[(pl * 64 + j) * kRaw + i] = (pv && j < ny && i < nx) ? __ldg(src + (long long)j * nx + i) : 0.f;
      }
    }
  };
  if ((int)blockIdx.x < npairs) load_raw(blockIdx.x);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const int lrow = (warp & 3) * 32 + (tid & 31);  // tensor-memory lane of this thread
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  const int half = warp >> 2;                     // column half in the epilogues
  uint32_t phase = 0;
  for (int pair = blockIdx.x; pair < npairs; pair += gridDim.x) {
    // slices: rows (p, y) of the x operand, columns (p, x) of the y operand
    {
      const int r = tid & 127, pl = r >> 6, w = r & 63;
      const bool by_row = tid < 128;
      const float* base = raw + pl * 64 * kRaw;
      const int stride_q = by_row ? 1 : kRaw, off = by_row ? w * kRaw : w;
      float m = 0.f;
      for (int q = 0; q < 64; ++q) m = fmaxf(m, fabsf(base[off + q * stride_q]));
      const int e = row_exponent(m);
      (by_row ? ex : ey)[r] = e;
      const float sc = pow2f(7 - e);
      uint8_t* A = by_row ? Ax : Ay;
#pragma unroll 1
      for (int c = 0; c < 8; ++c) {
        float y[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) y[u] = __fmul_rn(base[off + (c * 8 + u) * stride_q], sc);
        write_slices(A, r, c, y);
      }
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && !failed) {
      issue_products(tmem, tc::smem_u32(Ax), tc::smem_u32(B));
      issue_products(tmem + 256u, tc::smem_u32(Ay), tc::smem_u32(B));
      tc::mma_commit(&bar);
    }
    // the next pair's raw planes load while the products run (the raw buffer is free)
    if (pair + (int)gridDim.x < npairs) load_raw(pair + gridDim.x);
    if (!failed && !tc::mbar_wait(&bar, phase)) failed = 1;
    phase ^= 1u;
    tc::fence_after_sync();
    __syncthreads();
    if (failed) break;
    // x results (lane = (p, y), columns x) to shared memory as pairs
    {
      const float scale = pow2f(ex[lrow] + a.e_t - 14);
#pragma unroll 1
      for (int c0 = half * 32; c0 < half * 32 + 32; c0 += 16) {
        float2 v[16];
        load_pairs(tmem + lane_base + (uint32_t)c0, scale, v);
#pragma unroll
        for (int u = 0; u < 16; ++u) Xs[lrow * kStage + c0 + u] = v[u];
      }
    }
    __syncthreads();
    // y results (lane = (p, x), columns y) plus the staged x results; consecutive
    // lanes write consecutive x of one row
    {
      const int pl = lrow >> 6, i = lrow & 63;
      const int plane = 2 * pair + pl;
      const bool colv = plane < a.nplanes && i < nx;
      const long long base = colv ? (long long)plane * psz + i : 0;
      const float scale = pow2f(ey[lrow] + a.e_t - 14);
#pragma unroll 1
      for (int c0 = half * 32; c0 < half * 32 + 32; c0 += 16) {
        float2 v[16];
        load_pairs(tmem + 256u + lane_base + (uint32_t)c0, scale, v);
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int j = c0 + u;
          if (colv && j < ny) a.out[base + (long long)j * nx] = df_add(Xs[(pl * 64 + j) * kStage + i], v[u]);
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (failed && tid == 0) a.status[3] = 1;
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// z contraction added into the pairs: out(z, x) += Tz v.  128 threads, one per
// row (p, x) of the operand; each thread loads its column of the (z, x) plane.
__global__ void __launch_bounds__(128) k_kin_z_tc(KinTC a) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = align1024(smraw);
  uint8_t* A = sm;                 // kVS tiles
  uint8_t* B = sm + kVS * kTileA;  // kTS tiles
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const long long pstride = (long long)ny * nx;
  load_b(B, a.tslices, tid, 128);
  if (tid == 0) {
    failed = 0;
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 256);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const int npairs = (a.nplanes + 1) / 2;
  const int pl = tid >> 6, i = tid & 63;
  uint32_t phase = 0;
  float col[64];
  auto load_col = [&](int pair) {
    const int plane = 2 * pair + pl;  // plane = s * ny + y
    const bool cv = plane < a.nplanes && i < nx;
    const float* src = a.v32 + (cv ? (long long)(plane / ny) * nz * pstride + (long long)(plane % ny) * nx + i : 0);
#pragma unroll
    for (int k = 0; k < 64; ++k) col[k] = (cv && k < nz) ? __ldg(src + k * pstride) : 0.f;
  };
  if ((int)blockIdx.x < npairs) load_col(blockIdx.x);
  for (int pair = blockIdx.x; pair < npairs; pair += gridDim.x) {
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 64; ++k) m = fmaxf(m, fabsf(col[k]));
    const int e = row_exponent(m);
    const float sc = pow2f(7 - e);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      float y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) y[u] = __fmul_rn(col[c * 8 + u], sc);
      write_slices(A, tid, c, y);
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && !failed) {
      issue_products(tmem, tc::smem_u32(A), tc::smem_u32(B));
      tc::mma_commit(&bar);
    }
    const int plane = 2 * pair + pl;
    const bool cv = plane < a.nplanes && i < nx;
    const long long ob = cv ? (long long)(plane / ny) * nz * pstride + (long long)(plane % ny) * nx + i : 0;
    if (pair + (int)gridDim.x < npairs) load_col(pair + gridDim.x);
    if (!failed && !tc::mbar_wait(&bar, phase)) failed = 1;
    phase ^= 1u;
    tc::fence_after_sync();
    __syncthreads();
    if (failed) break;
    const float scale = pow2f(e + a.e_t - 14);
#pragma unroll 1
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float2 v[16];
      load_pairs(tmem + lane_base + (uint32_t)c0, scale, v);
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int k = c0 + u;
        if (cv && k < nz) {
          const long long o = ob + k * pstride;
          a.out[o] = df_add(a.out[o], v[u]);
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (failed && tid == 0) a.status[3] = 1;
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 256);
}

constexpr size_t kSmemXY = 2 * kVS * kTileA + kTS * kTileB + 2 * 64 * kRaw * sizeof(float) + 1024;
constexpr size_t kSmemZ = kVS * kTileA + kTS * kTileB + 1024;
static_assert(128 * kStage * sizeof(float2) <= 2 * kVS * kTileA, "x-result staging must fit over the operand tiles");

template <typename K>
int resident_grid(K kernel, int threads, size_t smem, int work) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  const int g = std::max(1, sms) * std::max(1, per_sm);
  return std::max(1, std::min(work, g));
}

uint16_t half_bits(float x) {  // FP16 bits of a small integer (|x| <= 2048: exact)
  const __half h = __float2half_rn(x);
  uint16_t u;
  std::memcpy(&u, &h, 2);
  return u;
}

}  // namespace

// Fixed-point FP16 slices of an n x n kinetic matrix: T = 2^(e_t - 7) (b1 + 2^-8 b2
// + 2^-16 b3 + 2^-24 b4) + O(2^(e_t - 32)), each b an integer in [-128, 128], as
// zero-padded [kTS][64][64] tiles (row = output index, column = contraction index).
void kinetic_f16_slices(const std::vector<double>& T, int n, std::vector<uint16_t>* slices, int* e_t) {
  double m = 0.0;
  for (double x : T) m = std::max(m, std::fabs(x));
  int e = 0;
  if (m > 0.0) std::frexp(m, &e);  // m = f 2^e, f in [0.5, 1)
  *e_t = e;
  slices->assign((size_t)kTS * 64 * 64, half_bits(0.f));
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < n; ++q) {
      double r = std::ldexp(T[(size_t)i * n + q], 7 - e);
      for (int l = 0; l < kTS; ++l) {
        const double b = std::nearbyint(r);
        (*slices)[((size_t)l * 64 + i) * 64 + q] = half_bits((float)b);
        r = (r - b) * 256.0;
      }
    }
}

bool kinetic_tc_supported(const Tables& t) { return t.nx <= 64 && t.ny <= 64 && t.nz <= 64 && t.tx == t.ty; }

int launch_kin_xy_tc(bsl_handle* h, const float* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  cudaFuncSetAttribute(k_kin_xy_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemXY);
  KinTC a{d.kxy_slices, d.e_txy, v, reinterpret_cast<float2*>(d.ukin), t.nx, t.ny, t.nz, t.nz * t.nn, d.status};
  k_kin_xy_tc<<<resident_grid(k_kin_xy_tc, 256, kSmemXY, (a.nplanes + 1) / 2), 256, kSmemXY, s>>>(a);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int launch_kin_z_tc(bsl_handle* h, const float* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  cudaFuncSetAttribute(k_kin_z_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemZ);
  KinTC a{d.kz_slices, d.e_tz, v, reinterpret_cast<float2*>(d.ukin), t.nx, t.ny, t.nz, t.ny * t.nn, d.status};
  k_kin_z_tc<<<resident_grid(k_kin_z_tc, 128, kSmemZ, (a.nplanes + 1) / 2), 128, kSmemZ, s>>>(a);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace bsl
