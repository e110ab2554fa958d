// Mixed-precision sinc-DVR kinetic contractions (sm_103a).
//
// Reference: Tv_5D_oneCompositeIndex / Mv_5D_oneCompositeIndex,
// Hv-calculators/linRotor/cartSphBasis/HvCalc/linRotCartSphHvRoutines.cpp:1807-1969
// (three dense line contractions with the 1-D kinetic matrices, summed).
//
// Precision: v is rounded to FP32; each kinetic matrix is split into an FP32
// head T_hi = fl32(T) and an FP32 tail T_lo = fl32(T - T_hi).  The head
// contraction and the tail contraction accumulate in separate FP32 registers
// and are combined into an unevaluated FP32 pair (hi + lo, error-free sums;
// no FP64 instruction), so the FP32 rounding of the coefficients (a
// systematic shift of every level, several 1e-3 cm^-1 at dx = 0.015 A) does
// not reach the result; only the random rounding of v and of the FP32 sums
// does.
//
// Work decomposition: persistent CTAs, one plane at a time: the (y, x) plane
// of fixed (s, z) for the x and y contractions and the (z, x) plane of fixed
// (s, y) for the z contraction.  Each plane contraction is a dense GEMM
// (n x n coefficients times an n x n plane) with 4 x 4 register tiles.  Both
// GEMM operands are read from shared memory as float4 along the output
// index they own: the plane is kept row-major (x innermost) and transposed
// (for the x contraction's left operand), the coefficient matrices in the
// orientation each product needs, so a thread issues 6 128-bit shared loads
// per 64 FMAs and the loop is FMA-bound.
#include "bsl_device.cuh"

namespace bsl {
namespace {

__host__ __device__ inline int round4(int n) { return (n + 3) & ~3; }

// plane elements held per thread for the next plane: ceil(64*64 / 256)
constexpr int kPrefetch = 16;

struct KinMixed {
  // x/y kernel: a_hi/a_lo = Tx^T [q][i] (x right operand), b_hi/b_lo = Ty^T [q][j] (y left operand)
  // z kernel:   a_hi/a_lo = Tz^T [q][k]
  const float *a_hi, *a_lo, *b_hi, *b_lo;
};

__device__ __forceinline__ void fma4x4(float (&acc)[4][4], const float4 a, const float4 b) {
  const float av[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    acc[r][0] = fmaf(av[r], b.x, acc[r][0]);
    acc[r][1] = fmaf(av[r], b.y, acc[r][1]);
    acc[r][2] = fmaf(av[r], b.z, acc[r][2]);
    acc[r][3] = fmaf(av[r], b.w, acc[r][3]);
  }
}

__device__ __forceinline__ void zero(float (&acc)[4][4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.f;
}

// x and y: out[s][k][j][i] = (Tx v)(i) + (Ty v)(j) on the plane of fixed (s, k)
__global__ void __launch_bounds__(256) k_kin_xy_split(const float* __restrict__ vec, float2* __restrict__ out,
                                                      KinMixed km, int nx, int ny, int nz, int nplanes) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int nxp = round4(nx), nyp = round4(ny);
  float* P = sm;                  // [nyp][nxp]  P[j][i]
  float* PT = P + nyp * nxp;      // [nxp][nyp]  PT[i][j]
  float* XH = PT + nxp * nyp;     // [nxp][nxp]  XH[q][i] = Tx_hi[i][q]
  float* XL = XH + nxp * nxp;
  float* YH = XL + nxp * nxp;     // [nyp][nyp]  YH[q][j] = Ty_hi[j][q]
  float* YL = YH + nyp * nyp;
  for (int e = threadIdx.x; e < nxp * nxp; e += blockDim.x) {
    XH[e] = km.a_hi[e];
    XL[e] = km.a_lo[e];
  }
  for (int e = threadIdx.x; e < nyp * nyp; e += blockDim.x) {
    YH[e] = km.b_hi[e];
    YL[e] = km.b_lo[e];
  }
  const int tcols = nxp / 4;
  const int tx = threadIdx.x % tcols, ty = threadIdx.x / tcols;
  const bool active = ty < nyp / 4;
  const int i0 = 4 * tx, j0 = 4 * ty;
  const int npl = nyp * nxp;
  // the next plane is loaded into registers while the current one is computed
  float pre[kPrefetch];
  auto load = [&](int plane) {
    const int k = plane % nz, s = plane / nz;
    const long long base = ((long long)s * nz + k) * ny * nx;
#pragma unroll
    for (int u = 0; u < kPrefetch; ++u) {
      const int e = threadIdx.x + u * blockDim.x;
      const int j = e / nxp, i = e - j * nxp;
      pre[u] = (e < npl && j < ny && i < nx) ? vec[base + (long long)j * nx + i] : 0.f;
    }
  };
  if (blockIdx.x < nplanes) load(blockIdx.x);
  for (int plane = blockIdx.x; plane < nplanes; plane += gridDim.x) {
    const int k = plane % nz, s = plane / nz;
    const long long base = ((long long)s * nz + k) * ny * nx;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kPrefetch; ++u) {
      const int e = threadIdx.x + u * blockDim.x;
      if (e < npl) {
        const int j = e / nxp, i = e - j * nxp;
        const float x = pre[u];
        P[e] = x;
        PT[i * nyp + j] = x;
      }
    }
    __syncthreads();
    if (plane + (int)gridDim.x < nplanes) load(plane + gridDim.x);
    if (!active) continue;
    float xh[4][4], xl[4][4], yh[4][4], yl[4][4];
    zero(xh);
    zero(xl);
    zero(yh);
    zero(yl);
    // x: out[j][i] = sum_q P[j][q] Tx[i][q] = sum_q PT[q][j] XH[q][i]
#pragma unroll 2
    for (int q = 0; q < nx; ++q) {
      const float4 a = *reinterpret_cast<const float4*>(PT + q * nyp + j0);
      fma4x4(xh, a, *reinterpret_cast<const float4*>(XH + q * nxp + i0));
      fma4x4(xl, a, *reinterpret_cast<const float4*>(XL + q * nxp + i0));
    }
    // y: out[j][i] = sum_q Ty[j][q] P[q][i] = sum_q YH[q][j] P[q][i]
#pragma unroll 2
    for (int q = 0; q < ny; ++q) {
      const float4 b = *reinterpret_cast<const float4*>(P + q * nxp + i0);
      fma4x4(yh, *reinterpret_cast<const float4*>(YH + q * nyp + j0), b);
      fma4x4(yl, *reinterpret_cast<const float4*>(YL + q * nyp + j0), b);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int j = j0 + r;
      if (j >= ny) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int i = i0 + c;
        if (i < nx) {
          // (hi, lo) pair with hi + lo = xh + yh + xl + yl to ~2^-48: no FP64 instruction
          float sh, se;
          two_sum(xh[r][c], yh[r][c], sh, se);
          float hi, lo;
          two_sum(sh, se + (xl[r][c] + yl[r][c]), hi, lo);
          out[base + (long long)j * nx + i] = make_float2(hi, lo);
        }
      }
    }
  }
}

// z: out[s][k][j][i] += (Tz v)(k) on the plane of fixed (s, j)
__global__ void __launch_bounds__(256) k_kin_z_split(const float* __restrict__ vec, float2* __restrict__ out,
                                                     KinMixed km, int nx, int ny, int nz, int nplanes) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int nxp = round4(nx), nzp = round4(nz);
  float* P = sm;                  // [nzp][nxp]  P[k][i]
  float* ZH = P + nzp * nxp;      // [nzp][nzp]  ZH[q][k] = Tz_hi[k][q]
  float* ZL = ZH + nzp * nzp;
  for (int e = threadIdx.x; e < nzp * nzp; e += blockDim.x) {
    ZH[e] = km.a_hi[e];
    ZL[e] = km.a_lo[e];
  }
  const int tcols = nxp / 4;
  const int tx = threadIdx.x % tcols, ty = threadIdx.x / tcols;
  const bool active = ty < nzp / 4;
  const int i0 = 4 * tx, k0 = 4 * ty;
  const long long plane_stride = (long long)ny * nx;
  const int npl = nzp * nxp;
  float pre[kPrefetch];
  auto load = [&](int plane) {
    const int j = plane % ny, s = plane / ny;
    const long long sb = (long long)s * nz * plane_stride + (long long)j * nx;
#pragma unroll
    for (int u = 0; u < kPrefetch; ++u) {
      const int e = threadIdx.x + u * blockDim.x;
      const int k = e / nxp, i = e - k * nxp;
      pre[u] = (e < npl && k < nz && i < nx) ? vec[sb + k * plane_stride + i] : 0.f;
    }
  };
  if (blockIdx.x < nplanes) load(blockIdx.x);
  for (int plane = blockIdx.x; plane < nplanes; plane += gridDim.x) {
    const int j = plane % ny, s = plane / ny;
    const long long sb = (long long)s * nz * plane_stride + (long long)j * nx;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kPrefetch; ++u) {
      const int e = threadIdx.x + u * blockDim.x;
      if (e < npl) P[e] = pre[u];
    }
    __syncthreads();
    if (plane + (int)gridDim.x < nplanes) load(plane + gridDim.x);
    if (!active) continue;
    float zh[4][4], zl[4][4];
    zero(zh);
    zero(zl);
#pragma unroll 2
    for (int q = 0; q < nz; ++q) {
      const float4 b = *reinterpret_cast<const float4*>(P + q * nxp + i0);
      fma4x4(zh, *reinterpret_cast<const float4*>(ZH + q * nzp + k0), b);
      fma4x4(zl, *reinterpret_cast<const float4*>(ZL + q * nzp + k0), b);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int k = k0 + r;
      if (k >= nz) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int i = i0 + c;
        if (i >= nx) continue;
        const long long o = sb + k * plane_stride + i;
        const float2 u = out[o];
        float sh, se;
        two_sum(u.x, zh[r][c], sh, se);
        float hi, lo;
        two_sum(sh, se + (u.y + zl[r][c]), hi, lo);
        out[o] = make_float2(hi, lo);
      }
    }
  }
}

size_t smem_xy(int nx, int ny) {
  const int nxp = round4(nx), nyp = round4(ny);
  return sizeof(float) * (2 * (size_t)nyp * nxp + 2 * (size_t)nxp * nxp + 2 * (size_t)nyp * nyp);
}
size_t smem_z(int nx, int nz) {
  const int nxp = round4(nx), nzp = round4(nz);
  return sizeof(float) * ((size_t)nzp * nxp + 2 * (size_t)nzp * nzp);
}

int persistent_grid(const void* kernel, int threads, size_t smem, int nplanes) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  const int g = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  return nplanes < g ? nplanes : g;
}

}  // namespace

// Host-side coefficient layouts: transposed FP32 head and tail, [q][i] = T[i][q],
// zero-padded to a multiple of 4.
void kinetic_split_tables(const std::vector<double>& T, int n, bool transpose, std::vector<float>* head,
                          std::vector<float>* tail) {
  (void)transpose;  // every operand above is stored transposed
  const int np = round4(n);
  head->assign((size_t)np * np, 0.f);
  tail->assign((size_t)np * np, 0.f);
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < n; ++q) {
      const double t = T[(size_t)i * n + q];
      const float hi = (float)t;
      (*head)[(size_t)q * np + i] = hi;
      (*tail)[(size_t)q * np + i] = (float)(t - (double)hi);
    }
}

int kinetic_mixed_supported(int nx, int ny, int nz, size_t* sxy, size_t* sz) {
  *sxy = smem_xy(nx, ny);
  *sz = smem_z(nx, nz);
  const int threads_xy = (round4(nx) / 4) * (round4(ny) / 4), threads_z = (round4(nx) / 4) * (round4(nz) / 4);
  const int txy = (threads_xy + 31) / 32 * 32, tz = (threads_z + 31) / 32 * 32;
  const bool covered = (long long)txy * kPrefetch >= (long long)round4(nx) * round4(ny) &&
                       (long long)tz * kPrefetch >= (long long)round4(nx) * round4(nz);
  return (*sxy <= 200 * 1024 && *sz <= 200 * 1024 && threads_xy <= 256 && threads_z <= 256 && covered) ? 1 : 0;
}

int launch_kin_xy_mixed(bsl_handle* h, const float* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  size_t sxy, sz;
  if (!kinetic_mixed_supported(t.nx, t.ny, t.nz, &sxy, &sz))
    return fail(BSL_ERR_UNSUPPORTED, "grid too large for the mixed-precision kinetic kernels (max 64 points/axis)");
  cudaFuncSetAttribute(k_kin_xy_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sxy);
  const int threads = ((round4(t.nx) / 4) * (round4(t.ny) / 4) + 31) / 32 * 32;
  const int nplanes = t.nz * t.nn;
  if (!d.kin_grid_xy) d.kin_grid_xy = persistent_grid((const void*)k_kin_xy_split, threads, sxy, 1 << 30);
  const int grid = d.kin_grid_xy;
  KinMixed km{d.kx_head, d.kx_band, d.ky_head, d.ky_band};
  k_kin_xy_split<<<grid < nplanes ? grid : nplanes, threads, sxy, s>>>(v, reinterpret_cast<float2*>(d.ukin), km,
                                                                       t.nx, t.ny, t.nz, nplanes);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int launch_kin_z_mixed(bsl_handle* h, const float* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  size_t sxy, sz;
  if (!kinetic_mixed_supported(t.nx, t.ny, t.nz, &sxy, &sz))
    return fail(BSL_ERR_UNSUPPORTED, "grid too large for the mixed-precision kinetic kernels (max 64 points/axis)");
  cudaFuncSetAttribute(k_kin_z_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sz);
  const int threads = ((round4(t.nx) / 4) * (round4(t.nz) / 4) + 31) / 32 * 32;
  const int nplanes = t.ny * t.nn;
  if (!d.kin_grid_z) d.kin_grid_z = persistent_grid((const void*)k_kin_z_split, threads, sz, 1 << 30);
  const int grid = d.kin_grid_z;
  KinMixed km{d.kz_head, d.kz_band, nullptr, nullptr};
  k_kin_z_split<<<grid < nplanes ? grid : nplanes, threads, sz, s>>>(v, reinterpret_cast<float2*>(d.ukin), km,
                                                                     t.nx, t.ny, t.nz, nplanes);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace bsl
