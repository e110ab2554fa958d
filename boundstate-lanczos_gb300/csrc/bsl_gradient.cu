// Hellmann-Feynman derivatives of the levels with respect to the cage: site
// charges, site positions and the two Alavi H2 charges.
//
// The levels are eigenvalues of the matrix H(theta) in a basis that does not
// depend on theta, so dE_n/dtheta = <psi_n| dH/dtheta |psi_n>, and only the
// potential blocks depend on theta:
//   <psi|dV|psi> = sum_p sum_{a,b,half} w_a w_b psi(p, a, b, half)^2 dV_half(p, a, b)/dtheta,
//   psi(p, a, b, half) = sum_s psi_s(p) L_s(a) T^half_{m_s}(b)
// (the quadrature of the potential blocks, ContinuousAngularGrid/
// linRotCartSphHvContGridRoutines.cpp:7-152), with V the Alavi SPC/E potential
// of Alavi_ContGrid_H2_Routines.cpp:6-147 with SPC/E or TIP4P water: the two H
// charges at p +- d u(a, b) and the centre-of-mass charge at p interact with
// every site by Coulomb, the centre of mass with every oxygen by Lennard-Jones, and V is clipped at the
// ceiling (no derivative where the ceiling applies).
//
// One CTA per grid point (persistent over points), one thread per site.  The
// angular densities of all levels are formed in shared memory, chunk by chunk
// of (a, b, half) nodes, FP32 (the derivative is a weighted sum; FP32 terms
// folded into FP64 totals per chunk); distances and the centre-of-mass terms
// are FP64.  Each CTA writes its per-site totals; a second kernel adds the CTAs.
#include <vector>

#include "bsl_device.cuh"

namespace bsl {
namespace {

constexpr int kGThreads = 64;     // sites per pass
constexpr int kChunk = 256;       // (a, b, half) nodes per chunk
constexpr int kMaxLev = 8;        // levels per pass
constexpr int kVals = 6;          // per (level, site): dE/dq, dE/dr (3), q_H part, q_CM part

struct GradArgs {
  const float* psi;       // [lev][nn][N] packed eigenvectors (normalised), FP32
  const float* Y;         // [C][nn] sqrt(w_a w_b) L_s(a) T^half_{m_s}(b), C = 2 na nb, node c = (a nb + b) 2 + half
  const double* v1;       // potential grid [N][na][nb], phi_b
  const double* v2;       // potential grid, 2 pi - phi_b
  const double* hdir;     // [na][nb][3] H offset for phi_b (y flips for 2 pi - phi_b)
  const double *xg, *yg, *zg;
  const double* xyz;      // [natoms][3]
  const double* q;        // [natoms]
  const int* is_o;
  int natoms, nx, ny, nn, na, nb, nlev;
  long long npts;
  double ceiling, q_h, q_cm, lj_a, lj_b;
  double* part;           // [gridDim][nlev][natoms][kVals]
};

__global__ void __launch_bounds__(kGThreads) k_hf_gradient(GradArgs g) {
  __shared__ float psi_s[kMaxLev][kMaxNN];
  __shared__ float omega[kMaxLev][kChunk];
  __shared__ float hpos[kChunk][3];       // H offset of node c (for the + atom; the - atom is its negative)
  __shared__ float red[kMaxLev][kGThreads / 32];
  __shared__ float Omega[kMaxLev];
  const int tid = threadIdx.x;
  const int C = 2 * g.na * g.nb;
  const int L = g.nlev;
  // per-(site, level) totals, for sites tid, tid + 64, ... (up to 8 sites per thread)
  for (int w0 = 0; w0 < g.natoms; w0 += kGThreads) {
    const int w = w0 + tid;
    const bool site = w < g.natoms;
    const double rwx = site ? g.xyz[3 * w] : 0.0, rwy = site ? g.xyz[3 * w + 1] : 0.0,
                 rwz = site ? g.xyz[3 * w + 2] : 0.0;
    const double qw = site ? g.q[w] : 0.0;
    const bool oxy = site && g.is_o[w];
    double tot[kMaxLev][kVals];
#pragma unroll
    for (int n = 0; n < kMaxLev; ++n)
#pragma unroll
      for (int k = 0; k < kVals; ++k) tot[n][k] = 0.0;
    for (long long p = blockIdx.x; p < g.npts; p += gridDim.x) {
      const int i = (int)(p % g.nx), j = (int)((p / g.nx) % g.ny), kz = (int)(p / ((long long)g.nx * g.ny));
      const double px = g.xg[i], py = g.yg[j], pz = g.zg[kz];
      __syncthreads();  // psi_s, omega, Omega of the previous point are no longer read
      for (int e = tid; e < L * g.nn; e += kGThreads) psi_s[e / g.nn][e % g.nn] = g.psi[(size_t)e * g.npts + p];
      if (tid < kMaxLev) Omega[tid] = 0.f;
      __syncthreads();
      float om_loc[kMaxLev];
#pragma unroll
      for (int n = 0; n < kMaxLev; ++n) om_loc[n] = 0.f;
      for (int c0 = 0; c0 < C; c0 += kChunk) {
        const int cn = min(kChunk, C - c0);
        // angular densities of the chunk's nodes (0 where the ceiling clips V)
        for (int cc = tid; cc < cn; cc += kGThreads) {
          const int c = c0 + cc;
          const int ab = c >> 1, half = c & 1;
          const double v = (half ? g.v2 : g.v1)[p * (g.na * g.nb) + ab];
          const bool active = v < g.ceiling;
          const float* y = g.Y + (size_t)c * g.nn;
#pragma unroll
          for (int n = 0; n < kMaxLev; ++n) {
            if (n < L) {
              float s = 0.f;
              for (int q = 0; q < g.nn; ++q) s = fmaf(psi_s[n][q], __ldg(y + q), s);
              const float o = active ? s * s : 0.f;
              omega[n][cc] = o;
              om_loc[n] += o;
            }
          }
          hpos[cc][0] = (float)g.hdir[3 * ab];
          hpos[cc][1] = (float)(half ? -g.hdir[3 * ab + 1] : g.hdir[3 * ab + 1]);
          hpos[cc][2] = (float)g.hdir[3 * ab + 2];
        }
        __syncthreads();
        if (site) {
          // H charges at p +- h: dV/dq_w = K q_H / r, dV/dr_w = K q_H q_w (x - r_w) / r^3
          const float dx0 = (float)(px - rwx), dy0 = (float)(py - rwy), dz0 = (float)(pz - rwz);
          float aq[kMaxLev], ax[kMaxLev], ay[kMaxLev], az[kMaxLev];
#pragma unroll
          for (int n = 0; n < kMaxLev; ++n) aq[n] = ax[n] = ay[n] = az[n] = 0.f;
          for (int cc = 0; cc < cn; ++cc) {
            const float hx = hpos[cc][0], hy = hpos[cc][1], hz = hpos[cc][2];
#pragma unroll
            for (int sgn = 0; sgn < 2; ++sgn) {
              const float ex = sgn ? dx0 - hx : dx0 + hx, ey = sgn ? dy0 - hy : dy0 + hy, ez = sgn ? dz0 - hz : dz0 + hz;
              const float inv = rsqrtf(ex * ex + ey * ey + ez * ez);
              const float inv3 = inv * inv * inv;
#pragma unroll
              for (int n = 0; n < kMaxLev; ++n) {
                if (n < L) {
                  const float o = omega[n][cc];
                  aq[n] = fmaf(o, inv, aq[n]);
                  const float oi3 = o * inv3;
                  ax[n] = fmaf(oi3, ex, ax[n]);
                  ay[n] = fmaf(oi3, ey, ay[n]);
                  az[n] = fmaf(oi3, ez, az[n]);
                }
              }
            }
          }
          const double kh = kCoulombK * g.q_h;
#pragma unroll
          for (int n = 0; n < kMaxLev; ++n) {
            tot[n][0] += kh * aq[n];
            tot[n][1] += kh * qw * ax[n];
            tot[n][2] += kh * qw * ay[n];
            tot[n][3] += kh * qw * az[n];
            tot[n][4] += kCoulombK * qw * aq[n];
          }
        }
        __syncthreads();  // omega and hpos are rewritten by the next chunk
      }
      // Omega_n(p): sum of the active densities (the centre-of-mass terms do not depend on a, b)
#pragma unroll
      for (int n = 0; n < kMaxLev; ++n) {
        float v = om_loc[n];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) red[n][tid >> 5] = v;
      }
      __syncthreads();
      if (tid < kMaxLev) {
        float v = 0.f;
        for (int k = 0; k < kGThreads / 32; ++k) v += red[tid][k];
        Omega[tid] = v;
      }
      __syncthreads();
      if (site) {
        const double dx = px - rwx, dy = py - rwy, dz = pz - rwz;
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double inv = 1.0 / sqrt(r2), inv3 = inv * inv * inv;
        double f = kCoulombK * g.q_cm * qw * inv3;  // dV/dr_w = f (p - r_w)
        if (oxy) {
          const double i2 = inv * inv, i6 = i2 * i2 * i2, i8 = i6 * i2, i14 = i6 * i6 * i2;
          f += 12.0 * g.lj_a * i14 - 6.0 * g.lj_b * i8;
        }
#pragma unroll
        for (int n = 0; n < kMaxLev; ++n) {
          const double O = n < L ? Omega[n] : 0.f;
          tot[n][0] += kCoulombK * g.q_cm * O * inv;
          tot[n][1] += O * f * dx;
          tot[n][2] += O * f * dy;
          tot[n][3] += O * f * dz;
          tot[n][5] += kCoulombK * qw * O * inv;
        }
      }
    }
    if (site) {
#pragma unroll
      for (int n = 0; n < kMaxLev; ++n)
        if (n < L)
#pragma unroll
          for (int k = 0; k < kVals; ++k)
            g.part[(((size_t)blockIdx.x * L + n) * g.natoms + w) * kVals + k] = tot[n][k];
    }
  }
}

// sum over the CTAs: out[lev][natoms][kVals]
__global__ void k_hf_reduce(const double* part, int nblocks, int count, double* out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= count) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * count + e];
  out[e] = s;
}

}  // namespace
}  // namespace bsl

using namespace bsl;

extern "C" int bsl_hf_gradient(bsl_handle* h, int nlev, const double* psi, double* dq_site, double* dr_site,
                               double* dq_alavi) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (nlev < 1 || !psi || !dq_site || !dr_site || !dq_alavi) return fail(BSL_ERR_INPUT, "bad arguments");
  if (h->p.potential != BSL_POT_ALAVI_SPCE && h->p.potential != BSL_POT_ALAVI_TIP4P)
    return fail(BSL_ERR_UNSUPPORTED,
                "derivatives need a continuous-grid Alavi potential (the point-grid lookups are piecewise constant)");
  if (!h->d.v1) return fail(BSL_ERR_STATE, "the potential grid was released after HvPrep (keep_potential_grid = 0)");
  cudaSetDevice(h->p.device);
  const Tables& t = h->t;
  const long long N = t.npts, Df = bsl_basis_size(h);
  const int nn = t.nn, natoms = (int)h->cage.q.size();
  // packed, normalised FP32 eigenvectors
  std::vector<float> ps((size_t)nlev * nn * N);
  for (int n = 0; n < nlev; ++n) {
    double nrm = 0.0;
    for (int s = 0; s < nn; ++s)
      for (long long p = 0; p < N; ++p) {
        const double x = psi[(size_t)n * Df + (size_t)t.full_of[s] * N + p];
        nrm += x * x;
      }
    if (!(nrm > 0.0)) return fail(BSL_ERR_INPUT, "an eigenvector has no component in the symmetry block");
    const double sc = 1.0 / std::sqrt(nrm);
    for (int s = 0; s < nn; ++s)
      for (long long p = 0; p < N; ++p)
        ps[((size_t)n * nn + s) * N + p] = (float)(psi[(size_t)n * Df + (size_t)t.full_of[s] * N + p] * sc);
  }
  // Y[c][s] with the quadrature weights, node c = (a nb + b) 2 + half
  const int C = 2 * t.na * t.nb;
  std::vector<float> Y((size_t)C * nn);
  for (int a = 0; a < t.na; ++a)
    for (int b = 0; b < t.nb; ++b)
      for (int half = 0; half < 2; ++half)
        for (int s = 0; s < nn; ++s) {
          const int m = t.m_of[t.full_of[s]];
          const double tr = (half ? t.trig2 : t.trig1)[(size_t)(m + t.lmax) * t.nb + b];
          Y[(((size_t)a * t.nb + b) * 2 + half) * nn + s] =
              (float)(std::sqrt(t.gl_w[a] * t.gc_w[b]) * t.leg[(size_t)s * t.na + a] * tr);
        }
  std::vector<double> hdir((size_t)t.na * t.nb * 3);
  const double hz = 0.03707;  // Alavi_Parameters.h:10, nm
  for (int a = 0; a < t.na; ++a)
    for (int b = 0; b < t.nb; ++b) {
      double* o = &hdir[((size_t)a * t.nb + b) * 3];
      o[0] = hz * sin(t.theta[a]) * t.gc_x[b];
      o[1] = hz * sin(t.theta[a]) * sin(t.phi[b]);
      o[2] = hz * t.gl_x[a];
    }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = (int)std::min<long long>(N, 16LL * std::max(1, sms));
  std::vector<void*> bufs;
  auto up = [&](const void* src, size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    bufs.push_back(p);
    if (src && cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return p;
  };
  auto cleanup = [&]() {
    for (void* p : bufs) cudaFree(p);
  };
  const float* dY = (const float*)up(Y.data(), Y.size() * 4);
  const double* dh = (const double*)up(hdir.data(), hdir.size() * 8);
  const double* dx = (const double*)up(t.xg.data(), t.xg.size() * 8);
  const double* dy = (const double*)up(t.yg.data(), t.yg.size() * 8);
  const double* dz = (const double*)up(t.zg.data(), t.zg.size() * 8);
  const double* dxyz = (const double*)up(h->cage.xyz.data(), h->cage.xyz.size() * 8);
  const double* dq = (const double*)up(h->cage.q.data(), h->cage.q.size() * 8);
  const int* dio = (const int*)up(h->cage.is_o.data(), h->cage.is_o.size() * 4);
  const int per_pass = std::min(nlev, kMaxLev);
  double* dpart = (double*)up(nullptr, (size_t)blocks * per_pass * natoms * kVals * 8);
  double* dout = (double*)up(nullptr, (size_t)per_pass * natoms * kVals * 8);
  float* dpsi = (float*)up(nullptr, (size_t)per_pass * nn * N * 4);
  if (!dY || !dh || !dx || !dy || !dz || !dxyz || !dq || !dio || !dpart || !dout || !dpsi) {
    cleanup();
    return fail(BSL_ERR_NOMEM, "derivative buffers");
  }
  std::vector<double> out((size_t)per_pass * natoms * kVals);
  for (int n0 = 0; n0 < nlev; n0 += per_pass) {
    const int L = std::min(per_pass, nlev - n0);
    cudaError_t e = cudaMemcpy(dpsi, ps.data() + (size_t)n0 * nn * N, (size_t)L * nn * N * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cleanup();
      return cuda_fail(e, "eigenvector upload");
    }
    GradArgs g{dpsi, dY, h->d.v1, h->d.v2, dh, dx, dy, dz, dxyz, dq, dio, natoms, t.nx, t.ny, nn, t.na, t.nb, L, N,
               h->p.ceiling_potential, h->cage.q_h2_h, h->cage.q_h2_cm, h->cage.lj_a, h->cage.lj_b, dpart};
    k_hf_gradient<<<blocks, kGThreads>>>(g);
    const int count = L * natoms * kVals;
    k_hf_reduce<<<(count + 255) / 256, 256>>>(dpart, blocks, count, dout);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out.data(), dout, (size_t)count * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      cleanup();
      return cuda_fail(e, "derivative kernels");
    }
    for (int n = 0; n < L; ++n) {
      double qh = 0.0, qcm = 0.0;
      for (int w = 0; w < natoms; ++w) {
        const double* o = &out[((size_t)n * natoms + w) * kVals];
        dq_site[(size_t)(n0 + n) * natoms + w] = o[0];
        for (int k = 0; k < 3; ++k) dr_site[((size_t)(n0 + n) * natoms + w) * 3 + k] = o[1 + k];
        qh += o[4];
        qcm += o[5];
      }
      dq_alavi[2 * (n0 + n)] = qh;
      dq_alavi[2 * (n0 + n) + 1] = qcm;
    }
  }
  cleanup();
  return BSL_OK;
}
