// Mixed-precision sinc-DVR kinetic contractions (sm_103a).
//
// Reference: Tv_5D_oneCompositeIndex / Mv_5D_oneCompositeIndex,
// Hv-calculators/linRotor/cartSphBasis/HvCalc/linRotCartSphHvRoutines.cpp:1807-1969
// (three dense line contractions with the 1-D kinetic matrices, summed).
//
// Precision: v is rounded to FP32; each kinetic matrix is split into an FP32
// head T_hi = fl32(T) and an FP32 tail T_lo = fl32(T - T_hi).  The head
// contraction and the tail contraction accumulate in separate FP32 registers
// and are combined in FP64, so the FP32 rounding of the coefficients (a
// systematic shift of every level, several 1e-3 cm^-1 at dx = 0.015 A) does
// not reach the result.  The tail is applied on the band |i - i'| <= kBand;
// beyond it |T_lo| < 2^-24 |T_ii'| with |T_ii'| = c 2/(i-i')^2 <= c/40.
//
// Work decomposition: one CTA owns one plane at a time (persistent over
// planes): the (y, x) plane of fixed (s, z) for the x and y contractions and
// the (z, x) plane of fixed (s, y) for the z contraction.  Each plane
// contraction is a small dense GEMM out = A * B (A or B the plane), done with
// 4 x 4 register tiles from shared memory; the coefficient matrices stay in
// shared memory for the CTA's lifetime.
#include "bsl_device.cuh"

namespace bsl {
namespace {

constexpr int kBand = 8;
constexpr int kBandW = 2 * kBand + 1;

__host__ __device__ inline int round4(int n) { return (n + 3) & ~3; }

struct KinMixed {
  const float* ta;   // x/y kernel: Tx_hi transposed [nxp][nxp]; z kernel: Tz_hi [nzp][nzp]
  const float* tb;   // x/y kernel: Ty_hi [nyp][nyp]
  const float* la;   // tails on the band: [kBandW][n], la[d][i] = T_lo[i][i + d - kBand]
  const float* lb;
};

// x and y: out[s][k][j][i] = (Tx v)(i) + (Ty v)(j) on the plane of fixed (s, k)
__global__ void __launch_bounds__(256) k_kin_xy_split(const double* __restrict__ vec, double* __restrict__ out,
                                                      KinMixed km, int nx, int ny, int nz, int nplanes) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int nxp = round4(nx), nyp = round4(ny);
  const int ps = nxp + 4;  // plane row stride (floats), keeps float4 alignment
  float* P = sm;                    // [nyp][ps]
  float* TX = P + nyp * ps;         // [nxp][nxp]   TX[q][i] = Tx_hi[i][q]
  float* TY = TX + nxp * nxp;       // [nyp][nyp]   TY[j][q] = Ty_hi[j][q]
  float* LX = TY + nyp * nyp;       // [kBandW][nxp]
  float* LY = LX + kBandW * nxp;    // [kBandW][nyp]
  for (int e = threadIdx.x; e < nxp * nxp; e += blockDim.x) TX[e] = km.ta[e];
  for (int e = threadIdx.x; e < nyp * nyp; e += blockDim.x) TY[e] = km.tb[e];
  for (int e = threadIdx.x; e < kBandW * nxp; e += blockDim.x) LX[e] = km.la[e];
  for (int e = threadIdx.x; e < kBandW * nyp; e += blockDim.x) LY[e] = km.lb[e];
  const int tcols = nxp / 4;
  const int tx = threadIdx.x % tcols, ty = threadIdx.x / tcols;
  const bool active = ty < nyp / 4;
  const int i0 = 4 * tx, j0 = 4 * ty;
  for (int plane = blockIdx.x; plane < nplanes; plane += gridDim.x) {
    const int k = plane % nz, s = plane / nz;
    const long long base = ((long long)s * nz + k) * ny * nx;
    __syncthreads();
    for (int e = threadIdx.x; e < nyp * nxp; e += blockDim.x) {
      const int j = e / nxp, i = e - j * nxp;
      P[j * ps + i] = (j < ny && i < nx) ? (float)vec[base + (long long)j * nx + i] : 0.f;
    }
    __syncthreads();
    if (!active) continue;
    float ax[4][4], ay[4][4], al[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) ax[r][c] = ay[r][c] = al[r][c] = 0.f;
    // x: out[j][i] = sum_q P[j][q] TX[q][i]
    for (int q = 0; q < nx; ++q) {
      const float4 b = *reinterpret_cast<const float4*>(TX + q * nxp + i0);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float a = P[(j0 + r) * ps + q];
        ax[r][0] = fmaf(a, b.x, ax[r][0]);
        ax[r][1] = fmaf(a, b.y, ax[r][1]);
        ax[r][2] = fmaf(a, b.z, ax[r][2]);
        ax[r][3] = fmaf(a, b.w, ax[r][3]);
      }
    }
    // y: out[j][i] = sum_q TY[j][q] P[q][i]
    for (int q = 0; q < ny; ++q) {
      const float4 b = *reinterpret_cast<const float4*>(P + q * ps + i0);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float a = TY[(j0 + r) * nyp + q];
        ay[r][0] = fmaf(a, b.x, ay[r][0]);
        ay[r][1] = fmaf(a, b.y, ay[r][1]);
        ay[r][2] = fmaf(a, b.z, ay[r][2]);
        ay[r][3] = fmaf(a, b.w, ay[r][3]);
      }
    }
    // tails on the band (both axes share one accumulator: they are 2^-24 small)
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int j = j0 + r, i = i0 + c;
        float acc = 0.f;
        for (int d = 0; d < kBandW; ++d) {
          const int qi = i + d - kBand, qj = j + d - kBand;
          if (qi >= 0 && qi < nx) acc = fmaf(LX[d * nxp + i], P[j * ps + qi], acc);
          if (qj >= 0 && qj < ny) acc = fmaf(LY[d * nyp + j], P[qj * ps + i], acc);
        }
        al[r][c] = acc;
      }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int j = j0 + r;
      if (j >= ny) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int i = i0 + c;
        if (i < nx) out[base + (long long)j * nx + i] = ((double)ay[r][c] + (double)ax[r][c]) + (double)al[r][c];
      }
    }
  }
}

// z: out[s][k][j][i] += (Tz v)(k) on the plane of fixed (s, j)
__global__ void __launch_bounds__(256) k_kin_z_split(const double* __restrict__ vec, double* __restrict__ out,
                                                     KinMixed km, int nx, int ny, int nz, int nplanes) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int nxp = round4(nx), nzp = round4(nz);
  const int ps = nxp + 4;
  float* P = sm;                  // [nzp][ps]   P[k][i]
  float* TZ = P + nzp * ps;       // [nzp][nzp]  TZ[k][q] = Tz_hi[k][q]
  float* LZ = TZ + nzp * nzp;     // [kBandW][nzp]
  for (int e = threadIdx.x; e < nzp * nzp; e += blockDim.x) TZ[e] = km.ta[e];
  for (int e = threadIdx.x; e < kBandW * nzp; e += blockDim.x) LZ[e] = km.la[e];
  const int tcols = nxp / 4;
  const int tx = threadIdx.x % tcols, ty = threadIdx.x / tcols;
  const bool active = ty < nzp / 4;
  const int i0 = 4 * tx, k0 = 4 * ty;
  const long long plane_stride = (long long)ny * nx;
  for (int plane = blockIdx.x; plane < nplanes; plane += gridDim.x) {
    const int j = plane % ny, s = plane / ny;
    const long long sb = (long long)s * nz * plane_stride + (long long)j * nx;
    __syncthreads();
    for (int e = threadIdx.x; e < nzp * nxp; e += blockDim.x) {
      const int k = e / nxp, i = e - k * nxp;
      P[k * ps + i] = (k < nz && i < nx) ? (float)vec[sb + k * plane_stride + i] : 0.f;
    }
    __syncthreads();
    if (!active) continue;
    float az[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) az[r][c] = 0.f;
    for (int q = 0; q < nz; ++q) {
      const float4 b = *reinterpret_cast<const float4*>(P + q * ps + i0);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float a = TZ[(k0 + r) * nzp + q];
        az[r][0] = fmaf(a, b.x, az[r][0]);
        az[r][1] = fmaf(a, b.y, az[r][1]);
        az[r][2] = fmaf(a, b.z, az[r][2]);
        az[r][3] = fmaf(a, b.w, az[r][3]);
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int k = k0 + r;
      if (k >= nz) continue;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int i = i0 + c;
        if (i >= nx) continue;
        float acc = 0.f;
        for (int d = 0; d < kBandW; ++d) {
          const int qk = k + d - kBand;
          if (qk >= 0 && qk < nz) acc = fmaf(LZ[d * nzp + k], P[qk * ps + i], acc);
        }
        const long long o = sb + k * plane_stride + i;
        out[o] = ((double)az[r][c] + (double)acc) + out[o];
      }
    }
  }
}

size_t smem_xy(int nx, int ny) {
  const int nxp = round4(nx), nyp = round4(ny);
  return sizeof(float) * ((size_t)nyp * (nxp + 4) + (size_t)nxp * nxp + (size_t)nyp * nyp + kBandW * (nxp + nyp));
}
size_t smem_z(int nx, int nz) {
  const int nxp = round4(nx), nzp = round4(nz);
  return sizeof(float) * ((size_t)nzp * (nxp + 4) + (size_t)nzp * nzp + kBandW * nzp);
}

}  // namespace

// Host-side coefficient layouts for the kernels above.
void kinetic_split_tables(const std::vector<double>& T, int n, bool transpose, std::vector<float>* head,
                          std::vector<float>* band) {
  const int np = round4(n);
  head->assign((size_t)np * np, 0.f);
  band->assign((size_t)kBandW * np, 0.f);
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < n; ++q) {
      const double t = T[(size_t)i * n + q];
      const float hi = (float)t;
      if (transpose) (*head)[(size_t)q * np + i] = hi;
      else (*head)[(size_t)i * np + q] = hi;
      const int d = q - i + kBand;
      if (d >= 0 && d < kBandW) (*band)[(size_t)d * np + i] = (float)(t - (double)hi);
    }
}

int kinetic_mixed_supported(int nx, int ny, int nz, size_t* sxy, size_t* sz) {
  *sxy = smem_xy(nx, ny);
  *sz = smem_z(nx, nz);
  const int threads_xy = (round4(nx) / 4) * (round4(ny) / 4), threads_z = (round4(nx) / 4) * (round4(nz) / 4);
  return (*sxy <= 200 * 1024 && *sz <= 200 * 1024 && threads_xy <= 256 && threads_z <= 256) ? 1 : 0;
}

int launch_kin_xy_mixed(bsl_handle* h, const double* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  size_t sxy, sz;
  if (!kinetic_mixed_supported(t.nx, t.ny, t.nz, &sxy, &sz))
    return fail(BSL_ERR_UNSUPPORTED, "grid too large for the mixed-precision kinetic kernels (max 64 points/axis)");
  cudaFuncSetAttribute(k_kin_xy_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sxy);
  const int threads = (round4(t.nx) / 4) * (round4(t.ny) / 4);
  const int nplanes = t.nz * t.nn;
  const int grid = nplanes < 8 * 152 ? nplanes : 8 * 152;
  KinMixed km{d.kx_head, d.ky_head, d.kx_band, d.ky_band};
  k_kin_xy_split<<<grid, ((threads + 31) / 32) * 32, sxy, s>>>(v, d.ukin, km, t.nx, t.ny, t.nz, nplanes);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int launch_kin_z_mixed(bsl_handle* h, const double* v, cudaStream_t s) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  size_t sxy, sz;
  if (!kinetic_mixed_supported(t.nx, t.ny, t.nz, &sxy, &sz))
    return fail(BSL_ERR_UNSUPPORTED, "grid too large for the mixed-precision kinetic kernels (max 64 points/axis)");
  cudaFuncSetAttribute(k_kin_z_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sz);
  const int threads = (round4(t.nx) / 4) * (round4(t.nz) / 4);
  const int nplanes = t.ny * t.nn;
  const int grid = nplanes < 8 * 152 ? nplanes : 8 * 152;
  KinMixed km{d.kz_head, nullptr, d.kz_band, nullptr};
  k_kin_z_split<<<grid, ((threads + 31) / 32) * 32, sz, s>>>(v, d.ukin, km, t.nx, t.ny, t.nz, nplanes);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace bsl
