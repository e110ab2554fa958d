// Potential blocks as coefficients of real spherical harmonics (prep).
//
// Every product of two basis functions is a finite sum of real spherical
// harmonics of degree <= 2 l_max (bsl_gaunt.h, generated), so the quadrature
// blocks of the reference (ContinuousAngularGrid/linRotCartSphHvContGridRoutines.cpp:7-152)
// are, point by point, <s|V|s'>(p) = sum_k G[t][k] c_k(p) with t = (s, s'):
// nc coefficients carry the nn (nn + 1) / 2 block elements exactly.  Here the
// coefficients are recovered from the FP64 blocks by least squares (G has full
// column rank; G^T G is nearly diagonal), the reconstruction residual is
// measured, and the FP32 coefficients are stored tile-major for the potential
// stream ([tile][k][128 points], the layout of the FP32 blocks).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bsl_device.cuh"
#include "bsl_gaunt.h"

namespace bsl {
namespace {

// c(p) = Gp blocks(p); residual = max_t |blocks_t - (G c)_t| over the points,
// written as the bits of a non-negative double (ordered like the values)
__global__ void k_gaunt_coeffs(const double* __restrict__ vb64, long long npts, int ntri, int nc,
                               const double* __restrict__ gp, const gaunt::Term* __restrict__ terms, int nterms,
                               float* __restrict__ vc32, long long tile_pts, unsigned long long* resid,
                               unsigned long long* vmax) {
  extern __shared__ double sh[];  // Gp [nc][ntri]
  for (int e = threadIdx.x; e < nc * ntri; e += blockDim.x) sh[e] = gp[e];
  __syncthreads();
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npts;
       p += (long long)gridDim.x * blockDim.x) {
    double c[128];
    for (int k = 0; k < nc; ++k) {
      double s = 0.0;
      for (int t = 0; t < ntri; ++t) s = fma(sh[k * ntri + t], vb64[(long long)t * npts + p], s);
      c[k] = s;
      vc32[((p / tile_pts) * nc + k) * tile_pts + p % tile_pts] = (float)c[k];
    }
    double r = 0.0, m = 0.0;
    int e = 0;
    for (int t = 0; t < ntri; ++t) {
      double s = 0.0;
      for (; e < nterms && terms[e].t == t; ++e) s = fma(terms[e].g, c[terms[e].k], s);
      const double v = vb64[(long long)t * npts + p];
      r = fmax(r, fabs(v - s));
      m = fmax(m, fabs(v));
    }
    atomicMax(resid, (unsigned long long)__double_as_longlong(r));
    atomicMax(vmax, (unsigned long long)__double_as_longlong(m));
  }
}

// the generated expansion of the handle's basis, or null
const gaunt::Basis* basis_of(const bsl_handle* h) {
  for (const gaunt::Basis& b : gaunt::kBases)
    if (b.l_max == h->t.lmax && b.symmetry == h->p.symmetry && b.nn == h->t.nn) return &b;
  return nullptr;
}

// Gp = (G^T G)^-1 G^T by Cholesky (G: ntri x nc, full column rank)
bool pseudo_inverse(const gaunt::Basis& b, int ntri, std::vector<double>* gp) {
  const int nc = b.nc;
  std::vector<double> G((size_t)ntri * nc, 0.0), A((size_t)nc * nc, 0.0);
  for (int e = 0; e < b.nterms; ++e) G[(size_t)b.terms[e].t * nc + b.terms[e].k] = b.terms[e].g;
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j < nc; ++j) {
      double s = 0.0;
      for (int t = 0; t < ntri; ++t) s += G[(size_t)t * nc + i] * G[(size_t)t * nc + j];
      A[(size_t)i * nc + j] = s;
    }
  for (int j = 0; j < nc; ++j) {  // A = L L^T in place (lower triangle)
    double d = A[(size_t)j * nc + j];
    for (int k = 0; k < j; ++k) d -= A[(size_t)j * nc + k] * A[(size_t)j * nc + k];
    if (!(d > 0.0)) return false;
    d = std::sqrt(d);
    A[(size_t)j * nc + j] = d;
    for (int i = j + 1; i < nc; ++i) {
      double s = A[(size_t)i * nc + j];
      for (int k = 0; k < j; ++k) s -= A[(size_t)i * nc + k] * A[(size_t)j * nc + k];
      A[(size_t)i * nc + j] = s / d;
    }
  }
  gp->assign((size_t)nc * ntri, 0.0);
  std::vector<double> y(nc);
  for (int t = 0; t < ntri; ++t) {  // column t of Gp solves A x = G^T e_t
    for (int i = 0; i < nc; ++i) {
      double s = G[(size_t)t * nc + i];
      for (int k = 0; k < i; ++k) s -= A[(size_t)i * nc + k] * y[k];
      y[i] = s / A[(size_t)i * nc + i];
    }
    for (int i = nc - 1; i >= 0; --i) {
      double s = y[i];
      for (int k = i + 1; k < nc; ++k) s -= A[(size_t)k * nc + i] * y[k];
      y[i] = s / A[(size_t)i * nc + i];
    }
    for (int i = 0; i < nc; ++i) (*gp)[(size_t)i * ntri + t] = y[i];
  }
  return true;
}

}  // namespace

int gaunt_coefficient_count(const bsl_handle* h) {
  const gaunt::Basis* b = basis_of(h);
  return b ? b->nc : 0;
}

int dev_gaunt_coeffs(bsl_handle* h, double* residual, double* vmax_out) {
  const gaunt::Basis* b = basis_of(h);
  if (!b) return fail(BSL_ERR_UNSUPPORTED, "no spherical-harmonic expansion is generated for this basis");
  DeviceState& d = h->d;
  const Tables& t = h->t;
  const int ntri = t.nn * (t.nn + 1) / 2, nc = b->nc;
  const long long N = t.npts, tp = vstream_tile_points(), tiled = (N + tp - 1) / tp * tp;
  std::vector<double> gp;
  if (!pseudo_inverse(*b, ntri, &gp)) return fail(BSL_ERR_UNSUPPORTED, "spherical-harmonic expansion is singular");
  double* dgp = nullptr;
  gaunt::Term* dterms = nullptr;
  unsigned long long* dres = nullptr;
  auto cleanup = [&]() {
    cudaFree(dgp);
    cudaFree(dterms);
    cudaFree(dres);
  };
  cudaError_t e;
  if ((e = cudaMalloc(&dgp, gp.size() * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&dterms, (size_t)b->nterms * sizeof(gaunt::Term))) != cudaSuccess ||
      (e = cudaMalloc(&dres, 2 * sizeof(unsigned long long))) != cudaSuccess ||
      (!d.vc32 && (e = cudaMalloc(&d.vc32, (size_t)nc * tiled * sizeof(float))) != cudaSuccess)) {
    cleanup();
    return fail(BSL_ERR_NOMEM, std::string("spherical-harmonic coefficients: ") + cudaGetErrorString(e));
  }
  cudaStream_t s = d.stream;
  int rc = BSL_OK;
  unsigned long long hres[2] = {0, 0};
  const size_t smem = gp.size() * sizeof(double);
  if ((e = cudaMemcpyAsync(dgp, gp.data(), smem, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(dterms, b->terms, (size_t)b->nterms * sizeof(gaunt::Term), cudaMemcpyHostToDevice, s)) !=
          cudaSuccess ||
      (e = cudaMemsetAsync(dres, 0, 2 * sizeof(unsigned long long), s)) != cudaSuccess ||
      (e = cudaMemsetAsync(d.vc32, 0, (size_t)nc * tiled * sizeof(float), s)) != cudaSuccess) {
    rc = cuda_fail(e, "spherical-harmonic coefficients");
  } else if (smem > 200 * 1024) {
    rc = fail(BSL_ERR_UNSUPPORTED, "spherical-harmonic expansion too large for the prep kernel");
  } else {
    cudaFuncSetAttribute(k_gaunt_coeffs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_gaunt_coeffs<<<grid_for(N), kThreads, smem, s>>>(d.vb64, N, ntri, nc, dgp, dterms, b->nterms, d.vc32, tp,
                                                       dres, dres + 1);
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(hres, dres, sizeof(hres), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      rc = cuda_fail(e, "spherical-harmonic coefficients");
  }
  cleanup();
  if (rc) return rc;
  double r, m;
  std::memcpy(&r, &hres[0], sizeof(double));
  std::memcpy(&m, &hres[1], sizeof(double));
  if (residual) *residual = r;
  if (vmax_out) *vmax_out = m;
  return BSL_OK;
}

}  // namespace bsl
