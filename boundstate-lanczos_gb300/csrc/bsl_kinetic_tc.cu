// Sinc-DVR kinetic contractions on the fifth-generation tensor cores
// (tcgen05.mma kind::tf32, accumulators in tensor memory), sm_103a.
//
// Reference: Tv_5D_oneCompositeIndex / Mv_5D_oneCompositeIndex,
// Hv-calculators/linRotor/cartSphBasis/HvCalc/linRotCartSphHvRoutines.cpp:1807-1969.
//
// Each CTA takes two grid planes at a time (planes padded to 64 x 64) and
// forms D[(plane, row)][col] = sum_q A[(plane, row)][q] T[col][q] as one
// M = 128, N = 64, K = 64 product per split term:
//   x (plane (y, x) of fixed (s, z)):  A[(p, y)][q] = v(p, y, q),  out(y, x) += sum_q v(y, q) Tx[x][q]
//   y (same plane, transposed):        A[(p, x)][q] = v(p, q, x),  out(y, x) += sum_q Ty[y][q] v(q, x)
//   z (plane (z, x) of fixed (s, y)):  A[(p, x)][q] = v(p, q, x),  out(z, x) += sum_q Tz[z][q] v(q, x)
// Precision: v = v1 + v2 and T = T1 + T2 + T3 in TF32 (10 explicit mantissa
// bits each; T carries 33 bits, so the coefficients' rounding is ~1e-10
// relative).  The head D_h = T1 v1 + T1 v2 + T2 v1 and the tail
// D_l = T2 v2 + T3 v1 accumulate separately in FP32 tensor memory and are
// combined into an FP32 (hi, lo) pair with error-free sums, as the SIMT
// kernels do.  Both operands are K-major with the 128-byte swizzle; the
// coefficient tiles stay in shared memory for the CTA's lifetime.
#include <algorithm>
#include <cstring>

#include "bsl_internal.h"
#include "bsl_tc.cuh"

namespace bsl {
namespace {

constexpr uint32_t kTileA = 128 * 64 * 4;  // 32 KiB: 128 rows x 64 TF32
constexpr uint32_t kTileB = 64 * 64 * 4;   // 16 KiB
constexpr int kStage = 65;                 // padded row of the y staging buffer

struct KinTC {
  const float *b1, *b2, *b3;  // T splits, row-major [64][64] (row = output index, col = q), zero padded
  const float* v32;
  float2* out;
  int nx, ny, nz, nplanes;
  int* status;
};

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~(uintptr_t)1023);
}

__device__ __forceinline__ void load_b(uint8_t* B, const float* src, int tid) {
  for (int e = tid; e < 64 * 64; e += 128) *reinterpret_cast<float*>(B + tc::sw128_offset(e >> 6, e & 63, 64)) = src[e];
}

// the five split products of one K = 64 contraction (8 MMAs of K = 8 each)
__device__ __forceinline__ void issue_split_products(uint32_t d_h, uint32_t d_l, uint32_t a1, uint32_t a2, uint32_t b1,
                                                     uint32_t b2, uint32_t b3) {
  const uint32_t idesc = tc::idesc_tf32(128, 64);
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const uint32_t ka = (uint32_t)((s >> 2) * 128 * 128 + (s & 3) * 32);
    const uint32_t kb = (uint32_t)((s >> 2) * 64 * 128 + (s & 3) * 32);
    const uint32_t acc = s > 0 ? 1u : 0u;
    const uint64_t A1 = tc::sw128_desc(a1 + ka), A2 = tc::sw128_desc(a2 + ka);
    const uint64_t B1 = tc::sw128_desc(b1 + kb), B2 = tc::sw128_desc(b2 + kb), B3 = tc::sw128_desc(b3 + kb);
    tc::mma_tf32(d_h, A1, B1, idesc, acc);
    tc::mma_tf32(d_h, A2, B1, idesc, 1u);
    tc::mma_tf32(d_h, A1, B2, idesc, 1u);
    tc::mma_tf32(d_l, A2, B2, idesc, acc);
    tc::mma_tf32(d_l, A1, B3, idesc, 1u);
  }
}

__device__ __forceinline__ void split_tf32(float x, float& h, float& l) {
  h = tc::tf32_round(x);
  l = tc::tf32_round(x - h);
}

__device__ __forceinline__ float2 pair_sum(float xh, float xl, float yh, float yl) {
  float s, e, hi, lo;
  two_sum(xh, yh, s, e);
  two_sum(s, e + (xl + yl), hi, lo);
  return make_float2(hi, lo);
}

// x and y contractions; out(y, x) = (Tx v + Ty v) as (hi, lo) pairs
__global__ void __launch_bounds__(128, 1) k_kin_xy_tc(KinTC a) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = align1024(smraw);
  uint8_t* A1x = sm;
  uint8_t* A2x = sm + kTileA;
  uint8_t* A1y = sm + 2 * kTileA;
  uint8_t* A2y = sm + 3 * kTileA;
  uint8_t* B1 = sm + 4 * kTileA;
  uint8_t* B2 = B1 + kTileB;
  uint8_t* B3 = B2 + kTileB;
  // staging of the x results once the products are complete: [128][65] each,
  // over the (then free) operand tiles
  float* Xh = reinterpret_cast<float*>(sm);
  float* Xl = reinterpret_cast<float*>(sm + 2 * kTileA);
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  load_b(B1, a.b1, tid);
  load_b(B2, a.b2, tid);
  load_b(B3, a.b3, tid);
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
  const uint32_t Dhx = tmem, Dlx = tmem + 64, Dhy = tmem + 128, Dly = tmem + 192;
  const int npairs = (a.nplanes + 1) / 2;
  uint32_t phase = 0;
  for (int pair = blockIdx.x; pair < npairs; pair += gridDim.x) {
    // stage both planes as TF32 splits, natural (x) and transposed (y) orientation
    for (int pl = 0; pl < 2; ++pl) {
      const int plane = 2 * pair + pl;
      const bool pv = plane < a.nplanes;
      const long long base = pv ? (long long)plane * ny * nx : 0;
      for (int e = tid; e < 64 * 64; e += 128) {
        const int j = e >> 6, i = e & 63;
        const float x = (pv && j < ny && i < nx) ? a.v32[base + (long long)j * nx + i] : 0.f;
        float h, l;
        split_tf32(x, h, l);
        *reinterpret_cast<float*>(A1x + tc::sw128_offset(pl * 64 + j, i, 128)) = h;
        *reinterpret_cast<float*>(A2x + tc::sw128_offset(pl * 64 + j, i, 128)) = l;
        *reinterpret_cast<float*>(A1y + tc::sw128_offset(pl * 64 + i, j, 128)) = h;
        *reinterpret_cast<float*>(A2y + tc::sw128_offset(pl * 64 + i, j, 128)) = l;
      }
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && !failed) {
      const uint32_t b1 = tc::smem_u32(B1), b2 = tc::smem_u32(B2), b3 = tc::smem_u32(B3);
      issue_split_products(Dhx, Dlx, tc::smem_u32(A1x), tc::smem_u32(A2x), b1, b2, b3);
      issue_split_products(Dhy, Dly, tc::smem_u32(A1y), tc::smem_u32(A2y), b1, b2, b3);
      tc::mma_commit(&bar);
    }
    if (!failed && !tc::mbar_wait(&bar, phase)) failed = 1;
    phase ^= 1u;
    tc::fence_after_sync();
    __syncthreads();
    if (failed) break;
    // x results (lane = (plane, y), column = x) to shared memory
#pragma unroll 1
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float dh[16], dl[16];
      tc::tmem_ld16(Dhx + lane_base + (uint32_t)c0, dh);
      tc::tmem_ld16(Dlx + lane_base + (uint32_t)c0, dl);
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        Xh[tid * kStage + c0 + c] = dh[c];
        Xl[tid * kStage + c0 + c] = dl[c];
      }
    }
    __syncthreads();
    // y results (lane = (plane, x), column = y) combined with the staged x
    // results; consecutive lanes write consecutive x of one row
    const int pl = tid >> 6, i = tid & 63;
    const int plane = 2 * pair + pl;
    const bool colv = plane < a.nplanes && i < nx;
    const long long base = colv ? (long long)plane * ny * nx + i : 0;
#pragma unroll 1
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float yh[16], yl[16];
      tc::tmem_ld16(Dhy + lane_base + (uint32_t)c0, yh);
      tc::tmem_ld16(Dly + lane_base + (uint32_t)c0, yl);
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int j = c0 + c;
        if (colv && j < ny) {
          const int xrow = pl * 64 + j;
          a.out[base + (long long)j * nx] = pair_sum(Xh[xrow * kStage + i], Xl[xrow * kStage + i], yh[c], yl[c]);
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

// z contraction, added into the (hi, lo) pairs: out(z, x) += Tz v
__global__ void __launch_bounds__(128, 2) k_kin_z_tc(KinTC a) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = align1024(smraw);
  uint8_t* A1 = sm;
  uint8_t* A2 = sm + kTileA;
  uint8_t* B1 = sm + 2 * kTileA;
  uint8_t* B2 = B1 + kTileB;
  uint8_t* B3 = B2 + kTileB;
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  load_b(B1, a.b1, tid);
  load_b(B2, a.b2, tid);
  load_b(B3, a.b3, tid);
  if (tid == 0) {
    failed = 0;
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 128);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const uint32_t Dh = tmem, Dl = tmem + 64;
  const long long plane_stride = (long long)ny * nx;
  const int npairs = (a.nplanes + 1) / 2;
  uint32_t phase = 0;
  for (int pair = blockIdx.x; pair < npairs; pair += gridDim.x) {
    for (int pl = 0; pl < 2; ++pl) {
      const int plane = 2 * pair + pl;  // plane = s * ny + y
      const bool pv = plane < a.nplanes;
      const long long sb = pv ? (long long)(plane / ny) * nz * plane_stride + (long long)(plane % ny) * nx : 0;
      for (int e = tid; e < 64 * 64; e += 128) {
        const int k = e >> 6, i = e & 63;
        const float x = (pv && k < nz && i < nx) ? a.v32[sb + k * plane_stride + i] : 0.f;
        float h, l;
        split_tf32(x, h, l);
        *reinterpret_cast<float*>(A1 + tc::sw128_offset(pl * 64 + i, k, 128)) = h;
        *reinterpret_cast<float*>(A2 + tc::sw128_offset(pl * 64 + i, k, 128)) = l;
      }
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && !failed) {
      issue_split_products(Dh, Dl, tc::smem_u32(A1), tc::smem_u32(A2), tc::smem_u32(B1), tc::smem_u32(B2),
                           tc::smem_u32(B3));
      tc::mma_commit(&bar);
    }
    if (!failed && !tc::mbar_wait(&bar, phase)) failed = 1;
    phase ^= 1u;
    tc::fence_after_sync();
    __syncthreads();
    if (failed) break;
    const int pl = tid >> 6, i = tid & 63;
    const int plane = 2 * pair + pl;
    const bool colv = plane < a.nplanes && i < nx;
    const long long sb = colv ? (long long)(plane / ny) * nz * plane_stride + (long long)(plane % ny) * nx + i : 0;
#pragma unroll 1
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float zh[16], zl[16];
      tc::tmem_ld16(Dh + lane_base + (uint32_t)c0, zh);
      tc::tmem_ld16(Dl + lane_base + (uint32_t)c0, zl);
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int k = c0 + c;
        if (colv && k < nz) {
          const long long o = sb + k * plane_stride;
          const float2 u = a.out[o];
          a.out[o] = pair_sum(u.x, u.y, zh[c], zl[c]);
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
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

constexpr size_t kSmemXY = 4 * kTileA + 3 * kTileB + 1024;
constexpr size_t kSmemZ = 2 * kTileA + 3 * kTileB + 1024;

// persistent grid: every CTA resident at once
template <typename K>
int resident_grid(K kernel, size_t smem, int work) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, smem);
  const int g = std::max(1, sms) * std::max(1, per_sm);
  return std::max(1, std::min(work, g));
}

}  // namespace

// TF32 splits T = T1 + T2 + T3 of an n x n kinetic matrix as zero-padded
// [64][64] row-major tiles (row = output index, column = contraction index).
void kinetic_tf32_tables(const std::vector<double>& T, int n, std::vector<float>* t1, std::vector<float>* t2,
                         std::vector<float>* t3) {
  auto tf32 = [](double x) {
    float f = (float)x;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    std::memcpy(&f, &u, 4);
    return f;
  };
  t1->assign(64 * 64, 0.f);
  t2->assign(64 * 64, 0.f);
  t3->assign(64 * 64, 0.f);
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < n; ++q) {
      const double t = T[(size_t)i * n + q];
      const float a = tf32(t);
      const float b = tf32(t - (double)a);
      const float c = tf32(t - (double)a - (double)b);
      (*t1)[i * 64 + q] = a;
      (*t2)[i * 64 + q] = b;
      (*t3)[i * 64 + q] = c;
    }
}

bool kinetic_tc_supported(const Tables& t) {
  return t.nx <= 64 && t.ny <= 64 && t.nz <= 64 && t.tx == t.ty;
}

int launch_kin_xy_tc(bsl_handle* h, const float* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  cudaFuncSetAttribute(k_kin_xy_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemXY);
  KinTC a{d.kxy_tf32[0], d.kxy_tf32[1], d.kxy_tf32[2], v, reinterpret_cast<float2*>(d.ukin),
          t.nx, t.ny, t.nz, t.nz * t.nn, d.status};
  k_kin_xy_tc<<<resident_grid(k_kin_xy_tc, kSmemXY, (a.nplanes + 1) / 2), 128, kSmemXY, s>>>(a);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int launch_kin_z_tc(bsl_handle* h, const float* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  cudaFuncSetAttribute(k_kin_z_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemZ);
  KinTC a{d.kz_tf32[0], d.kz_tf32[1], d.kz_tf32[2], v, reinterpret_cast<float2*>(d.ukin),
          t.nx, t.ny, t.nz, t.ny * t.nn, d.status};
  k_kin_z_tc<<<resident_grid(k_kin_z_tc, kSmemZ, (a.nplanes + 1) / 2), 128, kSmemZ, s>>>(a);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace bsl
