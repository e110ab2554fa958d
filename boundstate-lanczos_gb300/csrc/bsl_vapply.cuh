// Potential-block apply kernels (templated on the block size), shared by the
// FP32 and FP64 instantiation units.
#pragma once

#include "bsl_device.cuh"

namespace bsl {
namespace {

// ---------------------------------------------------------------------------
// potential apply + rotor + (optionally) the first Lanczos step
//   mode 0: u = T v + rot v + V v          (u = out)
//   mode 1: r += T v + rot v + V v; partial alpha = v . r   (r = out, in place)
// ---------------------------------------------------------------------------
template <int NN, typename VT>
__global__ void __launch_bounds__(kThreads) k_vapply(const VT* __restrict__ vb, const double* __restrict__ vec,
                                                     const double* __restrict__ ukin, const double* __restrict__ rot,
                                                     double* __restrict__ out, long long npts, int mode,
                                                     double* partials, unsigned int* counter, double* scalars,
                                                     double* hist, int j, long long dpk) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  // logical Lanczos vectors are v = sv vec and r = sr out; r + H v is kept as
  // sr (out + (sv/sr) H vec): out' = out + c H vec, alpha = sv sr (vec . out')
  const double c = mode ? scalars[6] : 1.0;
  double dot = 0.0;
  if (p < npts) {
    double v[NN], acc[NN];
    VT vv[NN], va[NN];
#pragma unroll
    for (int s = 0; s < NN; ++s) {
      v[s] = vec[s * npts + p];
      vv[s] = (VT)v[s];
      va[s] = (VT)0;
      acc[s] = ukin[s * npts + p] + __ldg(rot + s) * v[s];
    }
    int t = 0;
#pragma unroll
    for (int s = 0; s < NN; ++s) {
#pragma unroll
      for (int q = s; q < NN; ++q, ++t) {
        const VT x = vb[(long long)t * npts + p];
        va[s] += x * vv[q];
        if (q != s) va[q] += x * vv[s];
      }
    }
#pragma unroll
    for (int s = 0; s < NN; ++s) {
      const double hv = acc[s] + (double)va[s];
      if (mode == 0) {
        out[s * npts + p] = hv;
      } else {
        const double r = fma(c, hv, out[s * npts + p]);
        out[s * npts + p] = r;
        dot += v[s] * r;
      }
    }
  }
  if (mode == 1) {
    if (p == 0) dot += vec[dpk] * out[dpk];  // the coordinate outside the symmetry block (H acts on it as 0)
    double total;
    if (reduce_grid(dot, partials, counter, &total) && threadIdx.x == 0) {
      scalars[0] = scalars[7] * total;
      hist[j - 1] = scalars[7] * total;
    }
  }
}

// generic fallback (local-memory arrays) for block sizes without an instantiation
__global__ void __launch_bounds__(kThreads) k_vapply_generic(const double* __restrict__ vb,
                                                             const double* __restrict__ vec,
                                                             const double* __restrict__ ukin,
                                                             const double* __restrict__ rot, double* __restrict__ out,
                                                             long long npts, int nn, int mode, double* partials,
                                                             unsigned int* counter, double* scalars, double* hist,
                                                             int j, long long dpk) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  // logical Lanczos vectors are v = sv vec and r = sr out; r + H v is kept as
  // sr (out + (sv/sr) H vec): out' = out + c H vec, alpha = sv sr (vec . out')
  const double c = mode ? scalars[6] : 1.0;
  double dot = 0.0;
  if (p < npts) {
    double v[kMaxNN], acc[kMaxNN];
    for (int s = 0; s < nn; ++s) {
      v[s] = vec[s * npts + p];
      acc[s] = ukin[s * npts + p] + __ldg(rot + s) * v[s];
    }
    int t = 0;
    for (int s = 0; s < nn; ++s)
      for (int q = s; q < nn; ++q, ++t) {
        const double x = vb[(long long)t * npts + p];
        acc[s] += x * v[q];
        if (q != s) acc[q] += x * v[s];
      }
    for (int s = 0; s < nn; ++s) {
      if (mode == 0) {
        out[s * npts + p] = acc[s];
      } else {
        const double r = fma(c, acc[s], out[s * npts + p]);
        out[s * npts + p] = r;
        dot += v[s] * r;
      }
    }
  }
  if (mode == 1) {
    if (p == 0) dot += vec[dpk] * out[dpk];
    double total;
    if (reduce_grid(dot, partials, counter, &total) && threadIdx.x == 0) {
      scalars[0] = scalars[7] * total;
      hist[j - 1] = scalars[7] * total;
    }
  }
}

}  // namespace
}  // namespace bsl
