// Sinc-DVR kinetic contractions on the fifth-generation tensor cores
// (tcgen05.mma kind::f16, accumulators in tensor memory), sm_103a, with
// exact accumulation.
//
// Reference: Tv_5D_oneCompositeIndex / Mv_5D_oneCompositeIndex,
// Hv-calculators/linRotor/cartSphBasis/HvCalc/linRotCartSphHvRoutines.cpp:1807-1969.
//
// Products (M = 128 rows, N = 64 output columns, K = 64):
//   x and y, one (y, x) plane of fixed (s, z) per batch: rows 0-63 are the rows of
//   the plane (D[y][x] = sum_q v(y, q) Tx[x][q]) and rows 64-127 its columns
//   (D[64 + x][y] = sum_q v(q, x) Ty[y][q]), so both directions of one plane
//   come out of one set of accumulators (the y part is transposed through
//   shared memory before the coalesced store);
//   z, two (z, x) planes of fixed (s, y) per batch: rows (p, x) are the columns
//   of the planes (D[(p, x)][z] = sum_q v(p, q, x) Tz[z][q]).
//
// Exactness (error-free slicing after Ozaki, Ogita, Oishi and Rump,
// Numer. Algorithms 59, 2012, here with 9-bit fixed-point slices): the values of
// the double-float Lanczos vector are scaled by a power of two to below 1 in
// magnitude -- one scale per (y, x) plane for x and y, one per operand row for
// z -- and cut into four 9-bit signed integer slices,
// v = 2^(e - 8) (a1 + 2^-9 a2 + 2^-18 a3 + 2^-27 a4) (36 bits relative to the
// scale's maximum: far below the FP32 noise of the potential apply); T is
// scaled from its largest element and cut into four slices the same way,
// rounded to nearest so that the symmetric T stays exactly symmetric (a
// Lanczos recurrence on a non-symmetric H scatters the converged copies of a
// level).  The slices are
// integers in [-256, 256], exact in FP16, their products are exact, and every
// partial sum of one product class (at most 4 products of 64 terms) is an
// integer of magnitude at most 2^24: the FP32 accumulation in tensor memory is
// exact whatever its internal rounding, so the result carries no accumulation
// bias.  The products of each scale class k + l <= 3 share one accumulator and
// the four classes are combined on the CUDA cores into a double-float pair.
// The rounding of T is the same along each Toeplitz diagonal and adds up
// coherently for smooth states: with 36 bits it shifts levels by ~1e-7 kJ/mol
// per axis.
//
// Pipeline: persistent CTAs, two per SM with 256 tensor-memory columns each, so
// that one CTA slices or finishes its epilogue while the other's products run.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "bsl_internal.h"
#include "bsl_tc.cuh"

namespace bsl {
namespace {

constexpr int kVS = 4;                       // slices of v
constexpr int kTS = 4;                       // slices of T
constexpr uint32_t kTileA = 128 * 128;       // 16 KiB: 128 rows x 64 FP16 (one 128-byte swizzle atom per row)
constexpr uint32_t kTileB = 64 * 128;        // 8 KiB
constexpr uint32_t kBatchA = kVS * kTileA;   // operand slices of one batch
constexpr uint32_t kCols = 4 * 64;           // accumulator columns of one batch (classes 0..3)
constexpr int kTcThreads = 256;       // threads per CTA
constexpr int kPairs = 10;                   // slice products (k, l) with k + l <= 3, by class
__constant__ int8_t c_pk[kPairs] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};
__constant__ int8_t c_pl[kPairs] = {0, 1, 0, 2, 1, 0, 3, 2, 1, 0};
__constant__ int8_t c_first[kPairs] = {1, 1, 0, 1, 0, 0, 1, 0, 0, 0};

struct KinTC {
  const uint16_t* tslices;  // [kTS][64][64] FP16 bits, row = output index, column = q, zero padded
  int e_t;                  // T = 2^(e_t - 8) (b1 + 2^-9 b2 + 2^-18 b3 + 2^-27 b4)
  const float2* v;          // the Lanczos v as double-float pairs
  float2* out;
  int nx, ny, nz, nplanes;
  int* status;
};

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~(uintptr_t)1023);
}

// byte offset of element k (a multiple of 4) of row r in an SW128 K-major tile with K = 64 FP16
__device__ __forceinline__ uint32_t quad_offset(int r, int k) {
  return (uint32_t)(r * 128 + (((k >> 3) ^ (r & 7)) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// exponent e with max|x| 2^-e in [0.5, 1]; 0 for an all-zero plane
__device__ __forceinline__ int plane_exponent(float maxabs) {
  if (!(maxabs > 0.f)) return 0;
  return max(-100, ilogbf(maxabs) + 1);
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((min(max(e, -126), 127) + 127) << 23); }

// Four 9-bit slices of a double-float value already scaled to |y| < 256 (hi and
// lo multiplied by the same power of two): y = a1 + 2^-9 a2 + 2^-18 a3 +
// 2^-27 a4 + O(2^-28), each a an integer in [-256, 256].  Every step is exact
// except the last rounding.
__device__ __forceinline__ void slice4(float yh, float yl, float (&a)[kVS]) {
  a[0] = rintf(yh);
  float r = __fmul_rn(__fadd_rn(__fsub_rn(yh, a[0]), yl), 512.f);
  a[1] = rintf(r);
  r = __fmul_rn(__fsub_rn(r, a[1]), 512.f);
  a[2] = rintf(r);
  r = __fmul_rn(__fsub_rn(r, a[2]), 512.f);
  a[3] = rintf(r);
}

// D_c += A_k B_l^T for the slice products, class c in accumulator columns [64 c, 64 c + 64)
__device__ __forceinline__ void issue_products(uint32_t d, uint32_t a, uint32_t b) {
  const uint32_t idesc = tc::idesc_f16(128, 64);
#pragma unroll 1
  for (int pr = 0; pr < kPairs; ++pr) {
    const int k = c_pk[pr], l = c_pl[pr];
    const uint32_t dc = d + (uint32_t)(k + l) * 64u;
    const bool first = c_first[pr] != 0;
#pragma unroll
    for (int s = 0; s < 4; ++s)
      tc::mma_f16(dc, tc::sw128_desc(a + (uint32_t)k * kTileA + (uint32_t)s * 32u),
                  tc::sw128_desc(b + (uint32_t)l * kTileB + (uint32_t)s * 32u), idesc, (first && s == 0) ? 0u : 1u);
  }
}

// the four class accumulators of 8 consecutive columns combined into
// double-float pairs and multiplied by `scale` (a power of two).  The classes
// are exact integers below 2^24: the head is c0 + 2^-9 c1 with its rounding
// error, the tail collects that error and the two smaller classes (its own
// rounding is ~2^-33 of the head); the pair is left unnormalised (|lo| may
// slightly exceed half an ulp of hi), which the double-float additions accept.
__device__ __forceinline__ void load_pairs8(uint32_t taddr, float scale, float2 (&out)[8]) {
  float c0[8], c1[8], c2[8], c3[8];
  tc::tmem_ld8_nowait(taddr, c0);
  tc::tmem_ld8_nowait(taddr + 64u, c1);
  tc::tmem_ld8_nowait(taddr + 128u, c2);
  tc::tmem_ld8_nowait(taddr + 192u, c3);
  tc::tmem_wait_ld();
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    float h, e;
    two_sum(c0[u], __fmul_rn(c1[u], 0x1p-9f), h, e);
    const float l = __fmaf_rn(c3[u], 0x1p-27f, __fmaf_rn(c2[u], 0x1p-18f, e));
    out[u] = make_float2(__fmul_rn(h, scale), __fmul_rn(l, scale));
  }
}

__device__ __forceinline__ void load_b(uint8_t* B, const uint16_t* src) {
  for (int e = threadIdx.x; e < kTS * 64 * 16; e += kTcThreads) {  // kTS tiles of 64 rows x 16 quads
    const int l = e >> 10, r = (e >> 4) & 63, q = (e & 15) * 4;
    *reinterpret_cast<uint2*>(B + l * kTileB + quad_offset(r, q)) =
        *reinterpret_cast<const uint2*>(src + ((size_t)l * 64 + r) * 64 + q);
  }
}

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }



// Column maxima of the same blocks through shared memory (part: [16][64]
// partials, then [64] maxima).  Contains two __syncthreads.
__device__ __forceinline__ void block_col_max(const float2 (&x)[4][4], float* part, int bj, int bi, float (&cm)[4]) {
#pragma unroll
  for (int c = 0; c < 4; ++c)
    part[bj * 64 + 4 * bi + c] =
        fmaxf(fmaxf(fabsf(x[0][c].x), fabsf(x[1][c].x)), fmaxf(fabsf(x[2][c].x), fabsf(x[3][c].x)));
  __syncthreads();
  if (threadIdx.x < 64) {
    float m = 0.f;
#pragma unroll
    for (int q = 0; q < 16; ++q) m = fmaxf(m, part[q * 64 + threadIdx.x]);
    part[16 * 64 + threadIdx.x] = m;
  }
  __syncthreads();
  const float4 m4 = *reinterpret_cast<const float4*>(part + 16 * 64 + 4 * bi);
  cm[0] = m4.x;
  cm[1] = m4.y;
  cm[2] = m4.z;
  cm[3] = m4.w;
}

// Slices of a 4 x 4 block, each row r scaled by sc[r] and written as row row0 + r
// with K = k0.. (by_rows), or each column c scaled by sc[c] and written as row
// row0 + c with K = k0.. (columns).
template <bool by_rows>
__device__ __forceinline__ void write_block(uint8_t* A, const float2 (&x)[4][4], const float (&sc)[4], int row0,
                                            int k0) {
#pragma unroll
  for (int o = 0; o < 4; ++o) {  // output row
    float s[4][kVS];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float2 v = by_rows ? x[o][u] : x[u][o];
      slice4(__fmul_rn(v.x, sc[o]), __fmul_rn(v.y, sc[o]), s[u]);
    }
#pragma unroll
    for (int k = 0; k < kVS; ++k)
      *reinterpret_cast<uint2*>(A + k * kTileA + quad_offset(row0 + o, k0)) =
          make_uint2(pack_h2(s[0][k], s[1][k]), pack_h2(s[2][k], s[3][k]));
  }
}

// Slices of a 4 x 4 block with one scale, written both as rows row_a + r (K =
// c0..) and as rows row_b + c (K = r0..).
__device__ __forceinline__ void write_block_both(uint8_t* A, const float2 (&x)[4][4], float sc, int row_a, int row_b,
                                                 int r0, int c0) {
  float s[4][4][kVS];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) slice4(__fmul_rn(x[r][c].x, sc), __fmul_rn(x[r][c].y, sc), s[r][c]);
#pragma unroll
  for (int k = 0; k < kVS; ++k) {
#pragma unroll
    for (int r = 0; r < 4; ++r)
      *reinterpret_cast<uint2*>(A + k * kTileA + quad_offset(row_a + r, c0)) =
          make_uint2(pack_h2(s[r][0][k], s[r][1][k]), pack_h2(s[r][2][k], s[r][3][k]));
#pragma unroll
    for (int c = 0; c < 4; ++c)
      *reinterpret_cast<uint2*>(A + k * kTileA + quad_offset(row_b + c, r0)) =
          make_uint2(pack_h2(s[0][c][k], s[1][c][k]), pack_h2(s[2][c][k], s[3][c][k]));
  }
}

// maximum over the CTA (red: one float per warp); contains a __syncthreads
__device__ __forceinline__ float cta_max(float m, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  m = red[0];
#pragma unroll
  for (int w = 1; w < kTcThreads / 32; ++w) m = fmaxf(m, red[w]);
  return m;
}

// x and y contractions; out(y, x) = (Tx v + Ty v) as double-float pairs.  One
// plane per batch: operand rows 0-63 are the plane's rows, rows 64-127 its
// columns, all with one scale per plane (each value is sliced once).  Two CTAs
// per SM, 256 tensor-memory columns each.
__global__ void __launch_bounds__(kTcThreads, 2) k_kin_xy_tc(KinTC a) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = align1024(smraw);
  uint8_t* A = sm;                                        // kVS tiles
  uint8_t* B = sm + kBatchA;                              // kTS tiles
  float* part = reinterpret_cast<float*>(B + kTS * kTileB);  // [16][64] column-maximum partials
  float2* Xs = reinterpret_cast<float2*>(sm);             // [64][64] x part, column swizzled, over A
  float2* Ys = Xs + 64 * 64;                              // [64][64] y part, over A
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  __shared__ int e_plane;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nx = a.nx, ny = a.ny;
  const long long psz = (long long)ny * nx;
  int plane_parity = 0;  // alternates the reduction slots of consecutive planes
  load_b(B, a.tslices);
  if (tid == 0) {
    failed = 0;
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, kCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const int lrow = (warp & 3) * 32 + (tid & 31);  // tensor-memory lane of this thread in the epilogue
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  const int half = warp >> 2;
  const int bj = tid >> 4, bi = tid & 15;  // 4 x 4 block of the plane sliced by this thread
  // this thread's 4 x 4 block of a plane, loaded one plane ahead (software pipeline)
  auto load_block = [&](int plane, float2 (&x)[4][4]) {
    const float2* src = a.v + (long long)plane * psz;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int j = 4 * bj + r, i = 4 * bi + c;
        x[r][c] = (j < ny && i < nx) ? __ldg(src + (long long)j * nx + i) : make_float2(0.f, 0.f);
      }
  };
  float2 xn[4][4];
  if ((int)blockIdx.x < a.nplanes) load_block(blockIdx.x, xn);
  uint32_t phase = 0;
  for (int plane = blockIdx.x; plane < a.nplanes; plane += gridDim.x) {
    float2 x[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) x[r][c] = xn[r][c];
    const int nxt = plane + (int)gridDim.x;
    {  // the plane after next into L2
      const int far = nxt + (int)gridDim.x;
      if (far < a.nplanes)
        for (long long o = (long long)tid * 4; o < psz; o += kTcThreads * 4) prefetch_l2(a.v + (long long)far * psz + o);
    }
    // one scale per plane: every operand row keeps 36 bits relative to the plane maximum
    float m = 0.f;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) m = fmaxf(m, fabsf(x[r][c].x));
    const int e = plane_exponent(cta_max(m, part + 16 * 64 + (plane_parity ? 8 : 0)));
    plane_parity ^= 1;
    if (tid == 0) e_plane = e;
    write_block_both(A, x, pow2f(8 - e), 4 * bj, 64 + 4 * bi, 4 * bj, 4 * bi);
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && !failed) {
      issue_products(tmem, tc::smem_u32(A), tc::smem_u32(B));
      tc::mma_commit(&bar);
    }
    if (nxt < a.nplanes) load_block(nxt, xn);  // in flight during the products and the epilogue
    if (!failed && !tc::mbar_wait(&bar, phase)) failed = 1;
    phase ^= 1u;
    tc::fence_after_sync();
    __syncthreads();
    if (failed) break;
    // epilogue: rows 0-63 (x part) and 64-127 (y part) to shared memory over A
    const float scale = pow2f(e_plane + a.e_t - 16);
#pragma unroll 1
    for (int c0 = half * 32; c0 < half * 32 + 32; c0 += 8) {
      float2 v[8];
      load_pairs8(tmem + lane_base + (uint32_t)c0, scale, v);
      if (lrow < 64) {  // x part: row y = lrow, columns x
#pragma unroll
        for (int u = 0; u < 8; ++u) Xs[lrow * 64 + ((c0 + u) ^ (lrow & 31))] = v[u];
      } else {          // y part: x = lrow - 64, columns y
#pragma unroll
        for (int u = 0; u < 8; ++u) Ys[(c0 + u) * 64 + (lrow - 64)] = v[u];
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    const int i = tid & 63;
    float2* dst = a.out + (long long)plane * psz;
    if (i < nx)
#pragma unroll 2
      for (int j = tid >> 6; j < ny; j += kTcThreads / 64)
        dst[(long long)j * nx + i] = df_add_fast(Xs[j * 64 + (i ^ (j & 31))], Ys[j * 64 + i]);
    __syncthreads();  // A (under Xs, Ys) is sliced again next
  }
  if (failed && tid == 0) a.status[3] = 1;
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// z contraction added into the pairs: out(z, x) += Tz v, two (z, x) planes of
// fixed (s, y) per batch, operand rows (p, x) each scaled by its own maximum.
// Two CTAs per SM, 256 tensor-memory columns each.
__global__ void __launch_bounds__(kTcThreads, 2) k_kin_z_tc(KinTC a) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = align1024(smraw);
  uint8_t* A = sm;                                           // kVS tiles
  uint8_t* B = sm + kBatchA;                                 // kTS tiles
  float* part = reinterpret_cast<float*>(B + kTS * kTileB);  // [16][64] column-maximum partials
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  __shared__ int e_row[128];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const long long pstride = (long long)ny * nx;
  load_b(B, a.tslices);
  if (tid == 0) {
    failed = 0;
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, kCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const int lrow = (warp & 3) * 32 + (tid & 31);
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  const int half = warp >> 2;
  const int bk = tid >> 4, bi = tid & 15;  // 4 x 4 block of each of the two planes
  const int npairs = (a.nplanes + 1) / 2;
  auto plane_base = [&](int plane) {  // plane = s * ny + y
    return (long long)(plane / ny) * nz * pstride + (long long)(plane % ny) * nx;
  };
  // this thread's 4 x 4 block of one plane (zeros beyond the planes)
  auto load_block = [&](int plane, float2 (&x)[4][4]) {
    const bool pv = plane < a.nplanes;
    const float2* src = a.v + (pv ? plane_base(plane) : 0);
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int k = 4 * bk + r, i = 4 * bi + c;
        x[r][c] = (pv && k < nz && i < nx) ? __ldg(src + k * pstride + i) : make_float2(0.f, 0.f);
      }
  };
  auto slice_plane = [&](int pl, const float2 (&x)[4][4]) {
    float cm[4], scl[4];
    block_col_max(x, part, bk, bi, cm);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int ec = plane_exponent(cm[u]);
      scl[u] = pow2f(8 - ec);
      if (bk == 0) e_row[pl * 64 + 4 * bi + u] = ec;
    }
    write_block<false>(A, x, scl, pl * 64 + 4 * bi, 4 * bk);
    __syncthreads();  // part[] is reused by the next plane
  };
  float2 xn[4][4];  // first plane of the next pair, loaded during the products (software pipeline)
  if ((int)blockIdx.x < npairs) load_block(2 * blockIdx.x, xn);
  uint32_t phase = 0;
  for (int pair = blockIdx.x; pair < npairs; pair += gridDim.x) {
    {
      float2 x0[4][4], x1[4][4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) x0[r][c] = xn[r][c];
      load_block(2 * pair + 1, x1);  // in flight while the first plane is sliced
      slice_plane(0, x0);
      slice_plane(1, x1);
    }
    const int nxt = pair + (int)gridDim.x;
    {  // the pair after next into L2
      const int far = nxt + (int)gridDim.x;
      if (far < npairs) {
        const int plane = 2 * far + (tid >> 7);
        const int i = (tid & 127) * 4;
        if (plane < a.nplanes && i < nx)
          for (int k = 0; k < nz; ++k) prefetch_l2(a.v + plane_base(plane) + k * pstride + i);
      }
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && !failed) {
      issue_products(tmem, tc::smem_u32(A), tc::smem_u32(B));
      tc::mma_commit(&bar);
    }
    if (nxt < npairs) load_block(2 * nxt, xn);
    {  // this thread's epilogue targets into L1 while the products run
      const int pl = lrow >> 6, i = lrow & 63;
      const int plane = 2 * pair + pl;
      if (plane < a.nplanes && i < nx) {
        const long long ob = plane_base(plane) + i;
        for (int k = half * 32; k < half * 32 + 32 && k < nz; ++k)
          asm volatile("prefetch.global.L1 [%0];" ::"l"(a.out + ob + k * pstride));
      }
    }
    if (!failed && !tc::mbar_wait(&bar, phase)) failed = 1;
    phase ^= 1u;
    tc::fence_after_sync();
    __syncthreads();
    if (failed) break;
    const int pl = lrow >> 6, i = lrow & 63;
    const int plane = 2 * pair + pl;
    const bool cv = plane < a.nplanes && i < nx;
    const long long ob = cv ? plane_base(plane) + i : 0;
    const float scale = pow2f(e_row[lrow] + a.e_t - 16);
#pragma unroll 1
    for (int c0 = half * 32; c0 < half * 32 + 32; c0 += 8) {
      float2 v[8], u0[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        u0[u] = (cv && c0 + u < nz) ? a.out[ob + (c0 + u) * pstride] : make_float2(0.f, 0.f);
      load_pairs8(tmem + lane_base + (uint32_t)c0, scale, v);
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (cv && c0 + u < nz) a.out[ob + (c0 + u) * pstride] = df_add_fast(u0[u], v[u]);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (failed && tid == 0) a.status[3] = 1;
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

constexpr size_t kSmemXY = kBatchA + kTS * kTileB + 17 * 64 * sizeof(float) + 1024;
constexpr size_t kSmemZ = kSmemXY;
static_assert(2 * 64 * 64 * sizeof(float2) <= kBatchA, "x and y staging must fit over the operand tiles");
static_assert(2 * (kSmemXY + 1024) <= 228 * 1024, "two CTAs per SM");
static_assert(2 * kCols <= 512, "the accumulators of two CTAs must fit in tensor memory");

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, sms);
}

uint16_t half_bits(float x) {  // FP16 bits of a small integer (|x| <= 2048: exact)
  const __half h = __float2half_rn(x);
  uint16_t u;
  std::memcpy(&u, &h, 2);
  return u;
}

}  // namespace

// Fixed-point FP16 slices of an n x n kinetic matrix: T = 2^(e_t - 8) (b1 + 2^-9 b2
// + 2^-18 b3 + 2^-27 b4) + O(2^(e_t - 36)), each b an integer in [-256, 256]
// rounded to nearest (a symmetric T stays symmetric), as zero-padded
// [kTS][64][64] tiles (row = output index, column = contraction index).
void kinetic_f16_slices(const std::vector<double>& T, int n, std::vector<uint16_t>* slices, int* e_t) {
  double m = 0.0;
  for (double x : T) m = std::max(m, std::fabs(x));
  int e = 0;
  if (m > 0.0) std::frexp(m, &e);  // m = f 2^e, f in [0.5, 1)
  *e_t = e;
  slices->assign((size_t)kTS * 64 * 64, half_bits(0.f));
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < n; ++q) {
      double r = std::ldexp(T[(size_t)i * n + q], 8 - e);
      for (int l = 0; l < kTS; ++l) {
        const double b = std::nearbyint(r);
        (*slices)[((size_t)l * 64 + i) * 64 + q] = half_bits((float)b);
        r = (r - b) * 512.0;
      }
    }
}

bool kinetic_tc_supported(const Tables& t) { return t.nx <= 64 && t.ny <= 64 && t.nz <= 64 && t.tx == t.ty; }

int launch_kin_xy_tc(bsl_handle* h, const float2* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  cudaFuncSetAttribute(k_kin_xy_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemXY);
  KinTC a{d.kxy_slices, d.e_txy, v, reinterpret_cast<float2*>(d.ukin), t.nx, t.ny, t.nz, t.nz * t.nn, d.status};
  k_kin_xy_tc<<<std::min(a.nplanes, 2 * sm_count()), kTcThreads, kSmemXY, s>>>(a);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int launch_kin_z_tc(bsl_handle* h, const float2* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  cudaFuncSetAttribute(k_kin_z_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemZ);
  KinTC a{d.kz_slices, d.e_tz, v, reinterpret_cast<float2*>(d.ukin), t.nx, t.ny, t.nz, t.ny * t.nn, d.status};
  k_kin_z_tc<<<std::min((a.nplanes + 1) / 2, 2 * sm_count()), kTcThreads, kSmemZ, s>>>(a);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace bsl
