// CUDA kernels (sm_103a) of the boundstate-lanczos GB300 library.
//
//   potential grid     V(x,y,z,theta,phi) for the Alavi H2 model in an SPC/E cage
//                      (reference: potentialCalc/Alavi/AlaviGeneric/Alavi_ContGrid_H2_Routines.cpp:6-147)
//                      or the isotropic oscillator (IsoHarmOsc_Routines.cpp:6-31), FP64;
//                      the point-grid Alavi H2 (Alavi_H2_Routines.cpp:5-276) and the
//                      origin point charge (Coulomb_Routines.cpp:6-33)
//   potential blocks   <lm|V|l'm'>(x,y,z) by the angular quadrature, sum-factorised over phi
//                      (reference: HvCalc/NoQuadOnTheFly/ContinuousAngularGrid/linRotCartSphHvContGridRoutines.cpp:7-152)
//   kinetic            sinc-DVR contractions along x, y (one plane per CTA) and z
//                      (reference: HvCalc/linRotCartSphHvRoutines.cpp:1807-1969)
//   potential apply    per-point symmetric block times the local (l,m) coefficients, fused
//                      with the rotor diagonal and the first Lanczos update and dot product
//                      (reference: HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:675-796)
//   Lanczos            fused axpy/dot/norm kernels with deterministic last-block reductions
//                      (reference: headLoop/LanczosCode/lanczosEigenValuesVectors.cpp:191-238)
//
// Vectors use the packed layout: element (s, p) at s*N + p with p = (k*ny + j)*nx + i.
// Potential blocks use [t][p] with t enumerating s <= s' row by row, so that
// consecutive threads (consecutive p) read consecutive addresses.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "bsl_device.cuh"

namespace bsl {
namespace {


// ---------------------------------------------------------------------------
// potential grid (FP64, no contraction: the reference evaluates each product
// and sum separately)
// ---------------------------------------------------------------------------
struct AtomSet {
  const double* xyz;  // [natoms][3]
  const double* q;
  const int* is_o;
  int n;
  double q_h, q_cm;   // Alavi H2 charges: each H, centre of mass
  double lj_a, lj_b;  // centre of mass - O Lennard-Jones A / r^12 - B / r^6 of the water model
};

constexpr int kMaxAtoms = 512;

__device__ __forceinline__ double dist(const double* a, double x, double y, double z) {
  const double d0 = __dsub_rn(a[0], x), d1 = __dsub_rn(a[1], y), d2 = __dsub_rn(a[2], z);
  double s = __dmul_rn(d0, d0);
  s = __dadd_rn(s, __dmul_rn(d1, d1));
  s = __dadd_rn(s, __dmul_rn(d2, d2));
  return __dsqrt_rn(s);
}

__device__ __forceinline__ double coulomb(const double* sxyz, const double* sq, int n, double qsite, double x,
                                          double y, double z) {
  double e = 0.0;
  const double kq = __dmul_rn(kCoulombK, qsite);
  for (int i = 0; i < n; ++i) e = __dadd_rn(e, __ddiv_rn(__dmul_rn(kq, sq[i]), dist(sxyz + 3 * i, x, y, z)));
  return e;
}

// Energy of one Alavi H2 charge site at every point of a grid (x fastest):
// Coulomb with the site charge qsite, plus the Lennard-Jones term to the
// oxygens for the centre of mass (with_lj).  The continuous-grid calculators
// evaluate it at the basis grid (the centre of mass), the point-grid ones at
// every point of the potential universe for both the centre of mass and the
// H atoms (Alavi_SiteSite_Eng, Alavi_H2_Routines.cpp:197-276).
__global__ void k_site_energy(AtomSet atoms, const double* xg, const double* yg, const double* zg, int nx, int ny,
                              long long npts, double qsite, int with_lj, double* out) {
  __shared__ double sxyz[3 * kMaxAtoms], sq[kMaxAtoms];
  __shared__ int so[kMaxAtoms];
  for (int i = threadIdx.x; i < atoms.n; i += blockDim.x) {
    sxyz[3 * i] = atoms.xyz[3 * i];
    sxyz[3 * i + 1] = atoms.xyz[3 * i + 1];
    sxyz[3 * i + 2] = atoms.xyz[3 * i + 2];
    sq[i] = atoms.q[i];
    so[i] = atoms.is_o[i];
  }
  __syncthreads();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int i = (int)(p % nx), j = (int)((p / nx) % ny), k = (int)(p / ((long long)nx * ny));
  const double x = xg[i], y = yg[j], z = zg[k];
  double e = coulomb(sxyz, sq, atoms.n, qsite, x, y, z);
  if (with_lj) {
    double lj = 0.0;
    for (int a = 0; a < atoms.n; ++a) {
      if (!so[a]) continue;
      const double r = dist(sxyz + 3 * a, x, y, z);
      lj = __dadd_rn(lj, __dsub_rn(__ddiv_rn(atoms.lj_a, pow(r, 12.0)), __ddiv_rn(atoms.lj_b, pow(r, 6.0))));
    }
    e = __dadd_rn(e, lj);
  }
  out[p] = e;
}

// The potential universe of the point-grid calculators (generateGrid,
// potentialCalc/CommonRoutines/gridFcns.cpp:6-56): n[j] points with spacing
// d[j] = grid_max / (n - 1) from gmin[j] = -grid_max / 2, x fastest (disp, :58-84).
struct PointGrid {
  int n[3];
  double d[3], gmin[3];
};

// index of the universe point nearest to the numerator's coordinate: C round
// (halves away from zero) of numerator / d, kept inside the universe
// (AlaviMapH2GridToHGrid, Alavi_H2_Routines.cpp:5-52)
__device__ __forceinline__ int nearest_index(double numerator, double d, int n) {
  const int i = (int)round(__ddiv_rn(numerator, d));
  return i <= 0 ? 0 : (i >= n ? n - 1 : i);
}

// Point-grid Alavi H2 (Alavi_H2_Eng_Point, Alavi_H2_Routines.cpp:136-195, in
// calc_Vlmlpmp_NoQuad, HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:126-177):
// V = CM(nearest to the centre) + H(nearest to centre + d e) + H(nearest to
// centre - d e), clipped at the ceiling; e = (sin t cos p, sin t sin p, cos t)
// of each quadrature direction, both phi halves (edir: [half][a*nb+b][3]).
// One thread per (point, theta_a, phi_b).
__global__ void k_potential_point(const double* xg, const double* yg, const double* zg, int nx, int ny,
                                  long long npts, int nab, PointGrid u, const double* edir, const double* cmpot,
                                  const double* hpot, double hz, double ceiling, double* v1, double* v2) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npts * nab) return;
  const long long p = t / nab;
  const int ab = (int)(t % nab);
  const int i = (int)(p % nx), j = (int)((p / nx) % ny), k = (int)(p / ((long long)nx * ny));
  const double c[3] = {xg[i], yg[j], zg[k]};
  int icm[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) icm[q] = nearest_index(__dsub_rn(c[q], u.gmin[q]), u.d[q], u.n[q]);
  const double vcm = cmpot[icm[0] + (long long)u.n[0] * (icm[1] + (long long)u.n[1] * icm[2])];
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const double* e = edir + ((long long)half * nab + ab) * 3;
    double v = vcm;
#pragma unroll
    for (int site = 0; site < 2; ++site) {  // H1 at +d, H2 at -d along the axis
      const double dist_h = site ? -hz : hz;
      int ih[3];
#pragma unroll
      for (int q = 0; q < 3; ++q)
        ih[q] = nearest_index(__dsub_rn(__dadd_rn(c[q], __dmul_rn(e[q], dist_h)), u.gmin[q]), u.d[q], u.n[q]);
      v = __dadd_rn(v, hpot[ih[0] + (long long)u.n[0] * (ih[1] + (long long)u.n[1] * ih[2])]);
    }
    if (v >= ceiling) v = ceiling;
    (half ? v2 : v1)[t] = v;
  }
}

// Point charge at the origin seen by one on the H2 centre of mass
// (CoulombPotential, potentialCalc/CoulombPotential/Coulomb_Routines.cpp:6-33,
// CoulombEng, CommonRoutines/energyRoutines.cpp:5-26): V = (K q_c q_m) / |r|,
// |V| > |c_ceil| -> c_ceil, then the HvInputFile ceiling; orientation
// independent.
__global__ void k_potential_coulomb(const double* xg, const double* yg, const double* zg, int nx, int ny,
                                    long long npts, int nab, double kqq, double coulomb_ceiling, double ceiling,
                                    double* v1, double* v2) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npts * nab) return;
  const long long p = t / nab;
  const int i = (int)(p % nx), j = (int)((p / nx) % ny), k = (int)(p / ((long long)nx * ny));
  const double x = xg[i], y = yg[j], z = zg[k];
  double s = __dmul_rn(x, x);
  s = __dadd_rn(s, __dmul_rn(y, y));
  s = __dadd_rn(s, __dmul_rn(z, z));
  double v = __ddiv_rn(kqq, __dsqrt_rn(s));
  if (fabs(v) > fabs(coulomb_ceiling)) v = coulomb_ceiling;
  if (v >= ceiling) v = ceiling;
  v1[t] = v;
  v2[t] = v;
}

// one thread per (point, theta_a, phi_b): both phi halves
__global__ void k_potential_alavi(AtomSet atoms, const double* xg, const double* yg, const double* zg, int nx, int ny,
                                  long long npts, int nab, const double* hdir, const double* cm, double ceiling,
                                  double* v1, double* v2) {
  __shared__ double sxyz[3 * kMaxAtoms], sq[kMaxAtoms];
  for (int i = threadIdx.x; i < atoms.n; i += blockDim.x) {
    sxyz[3 * i] = atoms.xyz[3 * i];
    sxyz[3 * i + 1] = atoms.xyz[3 * i + 1];
    sxyz[3 * i + 2] = atoms.xyz[3 * i + 2];
    sq[i] = atoms.q[i];
  }
  __syncthreads();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npts * nab) return;
  const long long p = t / nab;
  const int ab = (int)(t % nab);
  const int i = (int)(p % nx), j = (int)((p / nx) % ny), k = (int)(p / ((long long)nx * ny));
  const double x = xg[i], y = yg[j], z = zg[k];
  const double hx = hdir[3 * ab], hy = hdir[3 * ab + 1], hz = hdir[3 * ab + 2];
  const double c = cm[p];
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const double hyh = half ? -1.0 * hy : hy;
    double v = coulomb(sxyz, sq, atoms.n, atoms.q_h, __dadd_rn(x, hx), __dadd_rn(y, hyh), __dadd_rn(z, hz));
    v = __dadd_rn(v, coulomb(sxyz, sq, atoms.n, atoms.q_h, __dsub_rn(x, hx), __dsub_rn(y, hyh), __dsub_rn(z, hz)));
    v = __dadd_rn(v, c);
    if (v >= ceiling) v = ceiling;
    (half ? v2 : v1)[t] = v;
  }
}

__global__ void k_potential_iso(const double* xg, const double* yg, const double* zg, int nx, int ny, long long npts,
                                int nab, double factor, double iso_ceiling, double ceiling, double* v1, double* v2) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npts * nab) return;
  const long long p = t / nab;
  const int i = (int)(p % nx), j = (int)((p / nx) % ny), k = (int)(p / ((long long)nx * ny));
  const double x = xg[i], y = yg[j], z = zg[k];
  double d2 = __dmul_rn(x, x);
  d2 = __dadd_rn(d2, __dmul_rn(y, y));
  d2 = __dadd_rn(d2, __dmul_rn(z, z));
  double v = __dmul_rn(factor, d2);
  if (fabs(v) > fabs(iso_ceiling)) v = iso_ceiling;
  if (v >= ceiling) v = ceiling;
  v1[t] = v;
  v2[t] = v;
}

// ---------------------------------------------------------------------------
// potential blocks: one CTA per grid point.
//   F[a][m,m'] = sum_b w_b (T1_m(b) T1_m'(b) V1(a,b) + T2_m(b) T2_m'(b) V2(a,b))
//   B[s,s']   = sum_a w_a L_s(a) L_s'(a) F[a][m_s, m_s']
// ---------------------------------------------------------------------------
struct BlockTables {
  const double* trig1;  // [nm][nb]
  const double* trig2;
  const double* leg;    // [nn][na]
  const double* wa;     // [na]
  const double* wb;     // [nb]
  const int2* mpair;    // [nmtri] (mi, mj), mi <= mj
  const int2* spair;    // [ntri] (s, s')
  const int* fidx;      // [ntri] index into the mpair list of (m_s, m_s') sorted
  int na, nb, nm, nmtri, nn, ntri;
};

__global__ void k_vblocks(BlockTables bt, const double* v1, const double* v2, long long npts, double* vb64,
                          float* vb32, long long tile_pts) {
  extern __shared__ double smem[];
  const int na = bt.na, nb = bt.nb, nab = na * nb;
  double* sV1 = smem;
  double* sV2 = sV1 + nab;
  double* sT1 = sV2 + nab;
  double* sT2 = sT1 + bt.nm * nb;
  double* sL = sT2 + bt.nm * nb;
  double* sF = sL + bt.nn * na;
  const long long p = blockIdx.x;
  for (int e = threadIdx.x; e < nab; e += blockDim.x) {
    sV1[e] = v1[p * nab + e];
    sV2[e] = v2[p * nab + e];
  }
  for (int e = threadIdx.x; e < bt.nm * nb; e += blockDim.x) {
    const int b = e % nb;
    sT1[e] = bt.trig1[e] * sqrt(bt.wb[b]);
    sT2[e] = bt.trig2[e] * sqrt(bt.wb[b]);
  }
  for (int e = threadIdx.x; e < bt.nn * na; e += blockDim.x) sL[e] = bt.leg[e];
  __syncthreads();
  for (int e = threadIdx.x; e < na * bt.nmtri; e += blockDim.x) {
    const int a = e / bt.nmtri;
    const int2 mm = bt.mpair[e % bt.nmtri];
    const double* t1a = sT1 + mm.x * nb;
    const double* t1b = sT1 + mm.y * nb;
    const double* t2a = sT2 + mm.x * nb;
    const double* t2b = sT2 + mm.y * nb;
    const double* va = sV1 + a * nb;
    const double* vb = sV2 + a * nb;
    double f = 0.0;
    for (int b = 0; b < nb; ++b) f += t1a[b] * t1b[b] * va[b] + t2a[b] * t2b[b] * vb[b];
    sF[e] = f;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < bt.ntri; t += blockDim.x) {
    const int2 ss = bt.spair[t];
    const int fi = bt.fidx[t];
    const double* la = sL + ss.x * na;
    const double* lb = sL + ss.y * na;
    double acc = 0.0;
    for (int a = 0; a < na; ++a) acc += bt.wa[a] * la[a] * lb[a] * sF[a * bt.nmtri + fi];
    vb64[(long long)t * npts + p] = acc;
    vb32[((p / tile_pts) * bt.ntri + t) * tile_pts + p % tile_pts] = (float)acc;
  }
}

// ---------------------------------------------------------------------------
// kinetic
// ---------------------------------------------------------------------------
// x and y contractions of one (s, k) plane; out = Tx.v + Ty.v (overwrites)
__global__ void k_kin_xy_f64(const double* __restrict__ vec, double* __restrict__ out, const double* __restrict__ tx,
                             const double* __restrict__ ty, int nx, int ny, int nz) {
  extern __shared__ double plane[];
  const int k = blockIdx.x, s = blockIdx.y;
  const long long base = ((long long)s * nz + k) * ny * nx;
  const int np = nx * ny;
  for (int e = threadIdx.x; e < np; e += blockDim.x) plane[e] = vec[base + e];
  __syncthreads();
  for (int e = threadIdx.x; e < np; e += blockDim.x) {
    const int j = e / nx, i = e - j * nx;
    const double* tr = tx + (long long)i * nx;
    const double* row = plane + j * nx;
    double ax = 0.0;
    for (int q = 0; q < nx; ++q) ax += __ldg(tr + q) * row[q];
    const double* tc = ty + (long long)j * ny;
    double ay = 0.0;
    for (int q = 0; q < ny; ++q) ay += __ldg(tc + q) * plane[q * nx + i];
    out[base + e] = ay + ax;
  }
}

// z contraction of one (s, j) plane, added: out += Tz.v
__global__ void k_kin_z_f64(const double* __restrict__ vec, double* __restrict__ out, const double* __restrict__ tz,
                            int nx, int ny, int nz) {
  extern __shared__ double plane[];  // [k][i]
  const int j = blockIdx.x, s = blockIdx.y;
  const long long sb = (long long)s * nz * ny * nx;
  const int np = nx * nz;
  for (int e = threadIdx.x; e < np; e += blockDim.x) {
    const int k = e / nx, i = e - k * nx;
    plane[e] = vec[sb + ((long long)k * ny + j) * nx + i];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < np; e += blockDim.x) {
    const int k = e / nx, i = e - k * nx;
    const double* tr = tz + (long long)k * nz;
    double az = 0.0;
    for (int q = 0; q < nz; ++q) az += __ldg(tr + q) * plane[q * nx + i];
    const long long o = sb + ((long long)k * ny + j) * nx + i;
    out[o] = az + out[o];
  }
}

// Full-layout step of the host-state loop body (lanczosEigenValuesVectors.cpp:
// 195-238), three passes in the reference's per-element FP64 arithmetic:
//   1. r_i += (H v)_i on the symmetry block (packed_of: full function -> packed, -1
//      outside), alpha = v . r
//   2. beta^2 = |r - alpha v|^2 (nothing written)
//   3. v <- (r - alpha v) / beta, r <- -beta v
__global__ void k_scatter_dot(const double* __restrict__ v, double* __restrict__ r, long long L,
                              const double* __restrict__ hv, const int* __restrict__ packed_of, long long npts,
                              int nfull, double* partials, unsigned int* counter, double* scalars, double* hist,
                              int j) {
  __shared__ int pof[1024];
  for (int f = threadIdx.x; f < nfull && f < 1024; f += blockDim.x) pof[f] = packed_of[f];
  __syncthreads();
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += (long long)gridDim.x * blockDim.x) {
    const long long f = i / npts;
    const int s = pof[f];
    double ri = r[i];
    if (s >= 0) {
      ri = ri + hv[(long long)s * npts + (i - f * npts)];
      r[i] = ri;
    }
    acc += v[i] * ri;
  }
  double total;
  if (reduce_grid(acc, partials, counter, &total) && threadIdx.x == 0) {
    scalars[0] = total;
    hist[j - 1] = total;
  }
}

__global__ void k_beta_only(const double* __restrict__ v, const double* __restrict__ r, long long L, double* partials,
                            unsigned int* counter, double* scalars, double* hist, int hist_stride, int j,
                            int* status) {
  const double alpha = scalars[0];
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += (long long)gridDim.x * blockDim.x) {
    const double x = r[i] - alpha * v[i];
    acc += x * x;
  }
  double total;
  if (reduce_grid(acc, partials, counter, &total) && threadIdx.x == 0) {
    const double b = sqrt(total);
    scalars[1] = b;
    scalars[2] = total;
    scalars[3] = 1. / b;
    hist[hist_stride + j] = b;
    hist[2 * hist_stride + j] = total;
    if (!(b > 0.0) || !isfinite(b) || !isfinite(alpha)) {
      if (status[0] == 0) status[1] = j;
      status[0] = 1;
    }
  }
}

__global__ void k_normalize_fused(double* __restrict__ v, double* __restrict__ r, long long L,
                                  const double* __restrict__ scalars) {
  const double alpha = scalars[0], b = scalars[1], inv = scalars[3];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += (long long)gridDim.x * blockDim.x) {
    const double vi = v[i];
    const double x = r[i] - alpha * vi;
    v[i] = inv * x;
    r[i] = (-b) * vi;
  }
}

// the same, written to other buffers (the caller's host vec and rvec, mapped
// into the device address space, so the results cross the host link once)
__global__ void k_normalize_to(const double* __restrict__ v, const double* __restrict__ r, long long L,
                               const double* __restrict__ scalars, double* __restrict__ v_out,
                               double* __restrict__ r_out) {
  const double alpha = scalars[0], b = scalars[1], inv = scalars[3];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += (long long)gridDim.x * blockDim.x) {
    const double vi = v[i];
    const double x = r[i] - alpha * vi;
    v_out[i] = inv * x;
    r_out[i] = (-b) * vi;
  }
}

// packed FP32 copy and double-float pairs of a full-layout FP64 vector
__global__ void k_gather_mixed(const double* __restrict__ full, float* __restrict__ v32, float2* __restrict__ vpair,
                               const int* __restrict__ full_of, long long npts, int nn) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= npts * nn) return;
  const int s = (int)(e / npts);
  const long long p = e - (long long)s * npts;
  const double x = full[(long long)full_of[s] * npts + p];
  const float2 d = df_of(x);
  v32[e] = d.x;
  if (vpair) vpair[e] = d;
}

// Folded-scale update of the packed loop.  The logical vectors are v = sv V and
// r = sr R, and R already holds R + (sv/sr) H V.  This kernel forms
// r - alpha v = sr (R - alpha (sv/sr) V), beta^2 = sr^2 |R|^2, and the scales of
// the next iteration, whose V is this R (v_{j+1} = (sr/beta) R) and whose R is
// this V (r_{j+1} = -beta v_j = (-beta sv) V): no pass rescales or swaps memory.
// It also writes the FP32 copy of the next v's buffer for the mixed kernels.
__global__ void k_update_fold(const double* __restrict__ V, double* __restrict__ R, long long L,
                              float* __restrict__ v32_next, long long D, double* partials, unsigned int* counter,
                              double* scalars, double* hist, int hist_stride, int j, int* status) {
  const double alpha = scalars[0], sv = scalars[4], sr = scalars[5], c = scalars[6];
  const double a = alpha * c;
  double acc = 0.0;
  const long long L2 = L / 2;
  const double2* V2 = reinterpret_cast<const double2*>(V);
  double2* R2 = reinterpret_cast<double2*>(R);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L2; i += (long long)gridDim.x * blockDim.x) {
    const double2 v = V2[i];
    double2 r = R2[i];
    r.x = fma(-a, v.x, r.x);
    r.y = fma(-a, v.y, r.y);
    R2[i] = r;
    acc = fma(r.x, r.x, acc);
    acc = fma(r.y, r.y, acc);
    const long long e = 2 * i;
    if (e + 1 < D) {
      reinterpret_cast<float2*>(v32_next)[i] = make_float2(f32_round(r.x), f32_round(r.y));
    } else if (e < D) {
      v32_next[e] = f32_round(r.x);
    }
  }
  if ((L & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const double x = fma(-a, V[L - 1], R[L - 1]);
    R[L - 1] = x;
    acc = fma(x, x, acc);
    if (L - 1 < D) v32_next[L - 1] = f32_round(x);
  }
  double total;
  if (reduce_grid(acc, partials, counter, &total) && threadIdx.x == 0) {
    const double b2 = sr * sr * total;
    const double b = sqrt(b2);
    scalars[1] = b;
    scalars[2] = b2;
    scalars[3] = 1. / b;
    hist[hist_stride + j] = b;
    hist[2 * hist_stride + j] = b2;
    const double sv_n = sr / b, sr_n = -b * sv;
    scalars[4] = sv_n;
    scalars[5] = sr_n;
    scalars[6] = sv_n / sr_n;
    scalars[7] = sv_n * sr_n;
    if (!(b > 0.0) || !isfinite(b) || !isfinite(alpha)) {
      if (status[0] == 0) status[1] = j;
      status[0] = 1;
    }
  }
}

// k_update_fold for Lanczos buffers stored as double-float pairs (mixed
// precision): every per-element operation runs on the FP32 pipe.  The new R
// buffer is also multiplied by a power of two g (exact) chosen from the
// previous beta so that its norm stays near 1 whatever the scales sv, sr do
// over many iterations: the FP32 exponent range of the pairs (and of the FP32
// copy the kinetic reads) is never approached.  The logical r keeps its value
// through sr / g.
__global__ void __launch_bounds__(256, 3) k_update_pair(const float2* __restrict__ V, float2* __restrict__ R,
                                                        long long L, float* __restrict__ v32_next, long long D,
                                                        double* partials, unsigned int* counter, double* scalars,
                                                        double* hist, int hist_stride, int j, int* status) {
  pdl_launch_dependents();
  pdl_wait();  // alpha and R come from the potential stream
  // per-thread constants prepared by the previous kernels' last blocks (no FP64 work per thread)
  const float2 na = reinterpret_cast<const float2*>(scalars)[9];  // -alpha c
  const int e = reinterpret_cast<const int*>(scalars)[20];         // g = 2^e, e = ilogb(sr) - ilogb(beta_{j-1})
  const float g = ldexpf(1.f, e);
  float2 acc = make_float2(0.f, 0.f);
  // two elements per 16-byte access, kUnroll accesses in flight per thread
  constexpr int kUnroll = 4;
  const long long L2 = L / 2;
  const float4* V4 = reinterpret_cast<const float4*>(V);
  float4* R4 = reinterpret_cast<float4*>(R);
  const long long stride = (long long)gridDim.x * blockDim.x * kUnroll;
  for (long long base = (long long)blockIdx.x * blockDim.x * kUnroll + threadIdx.x; base < L2; base += stride) {
    float4 v[kUnroll], r[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const long long q = base + (long long)u * blockDim.x;
      if (q < L2) {
        v[u] = V4[q];
        r[u] = R4[q];
      }
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const long long q = base + (long long)u * blockDim.x;
      if (q < L2) {
        const float2 r0 = df_scale2(df_fma_fast(na, make_float2(v[u].x, v[u].y), make_float2(r[u].x, r[u].y)), g);
        const float2 r1 = df_scale2(df_fma_fast(na, make_float2(v[u].z, v[u].w), make_float2(r[u].z, r[u].w)), g);
        R4[q] = make_float4(r0.x, r0.y, r1.x, r1.y);
        acc = df_add_fast(df_sqr(r0), acc);
        acc = df_add_fast(df_sqr(r1), acc);
        const long long e0 = 2 * q;
        if (v32_next) {  // only the CUDA-core kinetic reads the FP32 copy
          if (e0 + 1 < D)
            reinterpret_cast<float2*>(v32_next)[q] = make_float2(r0.x, r1.x);
          else if (e0 < D)
            v32_next[e0] = r0.x;
        }
      }
    }
  }
  if ((L & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const long long i = L - 1;
    const float2 r = df_scale2(df_fma_fast(na, V[i], R[i]), g);
    R[i] = r;
    acc = df_add_fast(df_sqr(r), acc);
    if (v32_next && i < D) v32_next[i] = r.x;
  }
  double total;
  if (reduce_grid_df(acc, partials, counter, &total) && threadIdx.x == 0)
    finish_update_pair(total, e, scalars, hist, hist_stride, j, status);
}

// double-float pairs of an FP64 vector
__global__ void k_pair_copy(const double* __restrict__ x, float2* __restrict__ y, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = df_of(x[i]);
}

// FP64 vector to double-float pairs in place (same 8 bytes per element)
__global__ void k_to_pair(double* x, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    reinterpret_cast<float2*>(x)[i] = df_of(x[i]);
}

// FP32 copy (rounded to nearest, integer pipe) of an FP64 vector
__global__ void k_to_f32(const double* __restrict__ x, float* __restrict__ y, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = f32_round(x[i]);
}

__global__ void k_fill(double* x, long long L, double val) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += (long long)gridDim.x * blockDim.x)
    x[i] = val;
}

// packed[s*N + p] = full[full_of[s]*N + p]
__global__ void k_gather(const double* __restrict__ full, double* __restrict__ packed, const int* __restrict__ full_of,
                         long long npts, int nn) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= npts * nn) return;
  const int s = (int)(e / npts);
  const long long p = e - (long long)s * npts;
  packed[e] = full[(long long)full_of[s] * npts + p];
}

// full[full_of[s]*N + p] += packed[s*N + p]
__global__ void k_scatter_add(const double* __restrict__ packed, double* __restrict__ full,
                              const int* __restrict__ full_of, long long npts, int nn) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= npts * nn) return;
  const int s = (int)(e / npts);
  const long long p = e - (long long)s * npts;
  const long long o = (long long)full_of[s] * npts + p;
  full[o] = full[o] + packed[e];
}

// ritz[n*D + i] += coef[n] * v[i] for active n, v = scalars[4] * V
__global__ void k_ritz(const double* __restrict__ V, long long D, const double* __restrict__ coef,
                       const int* __restrict__ active, int ngood, double* __restrict__ ritz,
                       const double* __restrict__ scalars, int pairs) {
  const double sv = scalars[4];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (long long)gridDim.x * blockDim.x) {
    const double vi = sv * (pairs ? f64_of_df(reinterpret_cast<const float2*>(V)[i]) : V[i]);
    for (int n = 0; n < ngood; ++n)
      if (active[n]) ritz[(long long)n * D + i] += coef[n] * vi;
  }
}

int launch_vapply(bsl_handle* h, const double* v, double* out, int mode, int j, cudaStream_t s) {
  DeviceState& d = h->d;
  const Tables& t = h->t;
  const long long N = t.npts;
  const dim3 g(grid_for(N));
  const long long dpk = N * t.nn;
  if (h->precision == BSL_PREC_MIXED) {
    StreamArgs a = vstream_args(h, v, out);
    a.mode = mode;
    a.j = j;
    a.defer = mode == 2 ? h->defer_reductions : 0;
    return launch_vapply_f32(a, t.nn, s);
  }
  return launch_vapply_f64(d.vb64, g, s, t.nn, v, d.ukin, d.rot, out, N, mode, d.partials, d.counter, d.scalars,
                           d.hist, j, dpk);
}

// mixed-precision kinetic stages by the selected engine: the tensor-core engine
// reads v as double-float pairs, the CUDA-core engine its FP32 copy
int launch_kin_xy(bsl_handle* h, const float2* vpair, cudaStream_t s) {
  return h->kinetic_engine == BSL_KIN_TENSOR ? launch_kin_xy_tc(h, vpair, s) : launch_kin_xy_mixed(h, h->d.v32, s);
}
int launch_kin_z(bsl_handle* h, const float2* vpair, cudaStream_t s) {
  return h->kinetic_engine == BSL_KIN_TENSOR ? launch_kin_z_tc(h, vpair, s) : launch_kin_z_mixed(h, h->d.v32, s);
}

int launch_kinetic(bsl_handle* h, const double* v, const float2* vpair, cudaStream_t s) {
  DeviceState& d = h->d;
  const Tables& t = h->t;
  const bool mixed = h->precision == BSL_PREC_MIXED;
  const size_t esz = mixed ? sizeof(float) : sizeof(double);
  const size_t sm_xy = esz * t.nx * t.ny, sm_z = esz * t.nx * t.nz;
  if (sm_xy > 200 * 1024 || sm_z > 200 * 1024) return fail(BSL_ERR_UNSUPPORTED, "grid plane too large for one CTA");
  const dim3 gxy(t.nz, t.nn), gz(t.ny, t.nn);
  if (mixed) {
    int rc = launch_kin_xy(h, vpair, s);
    if (!rc) rc = launch_kin_z(h, vpair, s);
    return rc;
  } else {
    cudaFuncSetAttribute(k_kin_xy_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_xy);
    cudaFuncSetAttribute(k_kin_z_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_z);
    k_kin_xy_f64<<<gxy, kThreads, sm_xy, s>>>(v, d.ukin, d.tx, d.ty, t.nx, t.ny, t.nz);
    k_kin_z_f64<<<gz, kThreads, sm_z, s>>>(v, d.ukin, d.tz, t.nx, t.ny, t.nz);
  }
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
StreamArgs vstream_args(bsl_handle* h, const double* v, double* out) {
  DeviceState& d = h->d;
  const Tables& t = h->t;
  StreamArgs a{};
  a.vb = d.vb32;
  a.v32 = d.v32;
  a.vec = v;
  a.ukin = reinterpret_cast<const float2*>(d.ukin);
  a.rot_hi = d.rot_hi;
  a.rot_lo = d.rot_lo;
  a.out = out;
  a.npts = t.npts;
  a.dpk = t.npts * t.nn;
  a.mode = 2;
  a.j = 0;
  a.jdev = d.jdev;
  a.partials = d.partials;
  a.scalars = d.scalars;
  a.hist = d.hist;
  a.counter = d.counter;
  a.status = d.status;
  a.vb16 = d.vb16;
  a.vscale = d.vscale;
  a.vc = d.vc32;
  a.vprod = d.vprod;
  a.vformat = h->vformat;
  a.nn = t.nn;
  a.red_count = 0;
  a.ctas_per_sm = h->tune_vs;
  return a;
}

int dev_potential_alavi(bsl_handle* h) {
  DeviceState& d = h->d;
  const Tables& t = h->t;
  const int natoms = (int)h->cage.q.size();
  if (natoms > kMaxAtoms) return fail(BSL_ERR_UNSUPPORTED, "cage has more than 512 atoms");
  std::vector<double> hdir((size_t)t.na * t.nb * 3);
  const double hz = 0.03707;  // Alavi_Parameters.h:10, nm
  for (int a = 0; a < t.na; ++a)
    for (int b = 0; b < t.nb; ++b) {
      double* o = &hdir[((size_t)a * t.nb + b) * 3];
      o[0] = hz * sin(t.theta[a]) * t.gc_x[b];
      o[1] = hz * sin(t.theta[a]) * sin(t.phi[b]);
      o[2] = hz * t.gl_x[a];
    }
  double *dxyz = nullptr, *dq = nullptr, *dh = nullptr, *dx = nullptr, *dy = nullptr, *dz = nullptr;
  int* dis_o = nullptr;
  auto cleanup = [&]() {
    cudaFree(dxyz); cudaFree(dq); cudaFree(dh); cudaFree(dis_o); cudaFree(dx); cudaFree(dy); cudaFree(dz);
  };
  auto up = [&](void** p, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*p, src, bytes, cudaMemcpyHostToDevice);
  };
  cudaError_t e;
  if ((e = up((void**)&dxyz, h->cage.xyz.data(), h->cage.xyz.size() * 8)) != cudaSuccess ||
      (e = up((void**)&dq, h->cage.q.data(), h->cage.q.size() * 8)) != cudaSuccess ||
      (e = up((void**)&dis_o, h->cage.is_o.data(), h->cage.is_o.size() * 4)) != cudaSuccess ||
      (e = up((void**)&dh, hdir.data(), hdir.size() * 8)) != cudaSuccess ||
      (e = up((void**)&dx, t.xg.data(), t.xg.size() * 8)) != cudaSuccess ||
      (e = up((void**)&dy, t.yg.data(), t.yg.size() * 8)) != cudaSuccess ||
      (e = up((void**)&dz, t.zg.data(), t.zg.size() * 8)) != cudaSuccess) {
    cleanup();
    return cuda_fail(e, "potential upload");
  }
  AtomSet atoms{dxyz, dq, dis_o, natoms, h->cage.q_h2_h, h->cage.q_h2_cm, h->cage.lj_a, h->cage.lj_b};
  const long long N = t.npts;
  const int nab = t.na * t.nb;
  double* cm = d.ukin;  // scratch of >= N doubles
  k_site_energy<<<grid_for(N), kThreads, 0, d.stream>>>(atoms, dx, dy, dz, t.nx, t.ny, N, atoms.q_cm, 1, cm);
  k_potential_alavi<<<grid_for(N * nab), kThreads, 0, d.stream>>>(atoms, dx, dy, dz, t.nx, t.ny, N, nab, dh, cm,
                                                                  h->p.ceiling_potential, d.v1, d.v2);
  e = cudaGetLastError();
  cudaError_t e2 = cudaStreamSynchronize(d.stream);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "potential kernel launch");
  if (e2 != cudaSuccess) return cuda_fail(e2, "potential kernel");
  return BSL_OK;
}

int dev_potential_iso(bsl_handle* h) {
  DeviceState& d = h->d;
  const Tables& t = h->t;
  double *dx = nullptr, *dy = nullptr, *dz = nullptr;
  BSL_CUDA(cudaMalloc(&dx, t.xg.size() * 8));
  BSL_CUDA(cudaMalloc(&dy, t.yg.size() * 8));
  BSL_CUDA(cudaMalloc(&dz, t.zg.size() * 8));
  BSL_CUDA(cudaMemcpy(dx, t.xg.data(), t.xg.size() * 8, cudaMemcpyHostToDevice));
  BSL_CUDA(cudaMemcpy(dy, t.yg.data(), t.yg.size() * 8, cudaMemcpyHostToDevice));
  BSL_CUDA(cudaMemcpy(dz, t.zg.data(), t.zg.size() * 8, cudaMemcpyHostToDevice));
  const double factor = 0.5 * h->p.iso_mass * h->p.iso_frequency * h->p.iso_frequency;
  const long long N = t.npts;
  const int nab = t.na * t.nb;
  k_potential_iso<<<grid_for(N * nab), kThreads, 0, d.stream>>>(dx, dy, dz, t.nx, t.ny, N, nab, factor,
                                                                h->p.iso_ceiling, h->p.ceiling_potential, d.v1, d.v2);
  cudaError_t e = cudaGetLastError();
  cudaError_t e2 = cudaStreamSynchronize(d.stream);
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dz);
  if (e != cudaSuccess) return cuda_fail(e, "isotropic oscillator kernel launch");
  if (e2 != cudaSuccess) return cuda_fail(e2, "isotropic oscillator kernel");
  return BSL_OK;
}

namespace {
// device copies of host arrays, freed together
struct Uploads {
  std::vector<void*> ptrs;
  ~Uploads() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t put(T** dst, const std::vector<T>& src) {
    *dst = nullptr;
    cudaError_t e = cudaMalloc((void**)dst, std::max<size_t>(1, src.size()) * sizeof(T));
    if (e != cudaSuccess) return e;
    ptrs.push_back(*dst);
    return src.empty() ? cudaSuccess : cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
  }
};
}  // namespace

int dev_potential_point_alavi(bsl_handle* h) {
  DeviceState& d = h->d;
  const Tables& t = h->t;
  const bsl_hv_params& p = h->p;
  const int natoms = (int)h->cage.q.size();
  if (natoms > kMaxAtoms) return fail(BSL_ERR_UNSUPPORTED, "cage has more than 512 atoms");
  // the potential universe (generateGrid, gridFcns.cpp:6-56)
  PointGrid u;
  const int un[3] = {p.pnx, p.pny, p.pnz};
  const double umax[3] = {p.px_max, p.py_max, p.pz_max};
  std::vector<double> ucoord[3];
  long long usize = 1;
  for (int q = 0; q < 3; ++q) {
    u.n[q] = un[q];
    u.d[q] = umax[q] / double(un[q] - 1);
    u.gmin[q] = (-0.5) * umax[q];
    usize *= un[q];
    ucoord[q].resize(un[q]);
    for (int i = 0; i < un[q]; ++i) ucoord[q][i] = (double(i) * u.d[q]) - (umax[q] / 2.0);
  }
  // H-H axis of every quadrature direction, phi in [0, pi) then [pi, 2 pi)
  const int nab = t.na * t.nb;
  std::vector<double> edir((size_t)2 * nab * 3);
  for (int half = 0; half < 2; ++half)
    for (int a = 0; a < t.na; ++a)
      for (int b = 0; b < t.nb; ++b) {
        const double ph = half ? t.phi2[b] : t.phi[b];
        double* o = &edir[(((size_t)half * t.na + a) * t.nb + b) * 3];
        o[0] = sin(t.theta[a]) * cos(ph);
        o[1] = sin(t.theta[a]) * sin(ph);
        o[2] = cos(t.theta[a]);
      }
  Uploads up;
  double *dxyz, *dq, *de, *dx, *dy, *dz, *ux, *uy, *uz, *cm, *hp;
  int* dis_o;
  cudaError_t e;
  if ((e = up.put(&dxyz, h->cage.xyz)) != cudaSuccess || (e = up.put(&dq, h->cage.q)) != cudaSuccess ||
      (e = up.put(&dis_o, h->cage.is_o)) != cudaSuccess || (e = up.put(&de, edir)) != cudaSuccess ||
      (e = up.put(&dx, t.xg)) != cudaSuccess || (e = up.put(&dy, t.yg)) != cudaSuccess ||
      (e = up.put(&dz, t.zg)) != cudaSuccess || (e = up.put(&ux, ucoord[0])) != cudaSuccess ||
      (e = up.put(&uy, ucoord[1])) != cudaSuccess || (e = up.put(&uz, ucoord[2])) != cudaSuccess ||
      (e = up.put(&cm, std::vector<double>((size_t)usize))) != cudaSuccess ||
      (e = up.put(&hp, std::vector<double>((size_t)usize))) != cudaSuccess)
    return cuda_fail(e, "point-grid potential upload");
  AtomSet atoms{dxyz, dq, dis_o, natoms, h->cage.q_h2_h, h->cage.q_h2_cm, h->cage.lj_a, h->cage.lj_b};
  k_site_energy<<<grid_for(usize), kThreads, 0, d.stream>>>(atoms, ux, uy, uz, u.n[0], u.n[1], usize, atoms.q_cm, 1,
                                                            cm);
  k_site_energy<<<grid_for(usize), kThreads, 0, d.stream>>>(atoms, ux, uy, uz, u.n[0], u.n[1], usize, atoms.q_h, 0,
                                                            hp);
  const long long N = t.npts;
  const double hz = 0.03707;  // H2_H1_Z = -H2_H2_Z, Alavi_Parameters.h:10-14, nm
  k_potential_point<<<grid_for(N * nab), kThreads, 0, d.stream>>>(dx, dy, dz, t.nx, t.ny, N, nab, u, de, cm, hp, hz,
                                                                  p.ceiling_potential, d.v1, d.v2);
  e = cudaGetLastError();
  const cudaError_t e2 = cudaStreamSynchronize(d.stream);
  if (e != cudaSuccess) return cuda_fail(e, "point-grid potential launch");
  if (e2 != cudaSuccess) return cuda_fail(e2, "point-grid potential kernel");
  return BSL_OK;
}

int dev_potential_coulomb(bsl_handle* h) {
  DeviceState& d = h->d;
  const Tables& t = h->t;
  Uploads up;
  double *dx, *dy, *dz;
  cudaError_t e;
  if ((e = up.put(&dx, t.xg)) != cudaSuccess || (e = up.put(&dy, t.yg)) != cudaSuccess ||
      (e = up.put(&dz, t.zg)) != cudaSuccess)
    return cuda_fail(e, "Coulomb potential upload");
  const double kqq = kCoulombK * h->p.coulomb_centre_charge * h->p.coulomb_mol_charge;
  const long long N = t.npts;
  const int nab = t.na * t.nb;
  k_potential_coulomb<<<grid_for(N * nab), kThreads, 0, d.stream>>>(dx, dy, dz, t.nx, t.ny, N, nab, kqq,
                                                                    h->p.coulomb_ceiling, h->p.ceiling_potential,
                                                                    d.v1, d.v2);
  e = cudaGetLastError();
  const cudaError_t e2 = cudaStreamSynchronize(d.stream);
  if (e != cudaSuccess) return cuda_fail(e, "Coulomb potential launch");
  if (e2 != cudaSuccess) return cuda_fail(e2, "Coulomb potential kernel");
  return BSL_OK;
}

int dev_vblocks(bsl_handle* h) {
  DeviceState& d = h->d;
  const Tables& t = h->t;
  const int nm = 2 * t.lmax + 1, nmtri = nm * (nm + 1) / 2, ntri = t.nn * (t.nn + 1) / 2;
  std::vector<int2> mpair, spair;
  std::vector<int> fidx;
  std::vector<int> mindex((size_t)nm * nm, -1);
  for (int a = 0; a < nm; ++a)
    for (int b = a; b < nm; ++b) {
      mindex[(size_t)a * nm + b] = (int)mpair.size();
      mpair.push_back(make_int2(a, b));
    }
  for (int s = 0; s < t.nn; ++s)
    for (int q = s; q < t.nn; ++q) {
      spair.push_back(make_int2(s, q));
      int ma = t.m_of[t.full_of[s]] + t.lmax, mb = t.m_of[t.full_of[q]] + t.lmax;
      if (ma > mb) std::swap(ma, mb);
      fidx.push_back(mindex[(size_t)ma * nm + mb]);
    }
  double *dt1, *dt2, *dleg, *dwa, *dwb;
  int2 *dmp, *dsp;
  int* dfi;
  BSL_CUDA(cudaMalloc(&dt1, t.trig1.size() * 8));
  BSL_CUDA(cudaMalloc(&dt2, t.trig2.size() * 8));
  BSL_CUDA(cudaMalloc(&dleg, t.leg.size() * 8));
  BSL_CUDA(cudaMalloc(&dwa, t.gl_w.size() * 8));
  BSL_CUDA(cudaMalloc(&dwb, t.gc_w.size() * 8));
  BSL_CUDA(cudaMalloc(&dmp, mpair.size() * sizeof(int2)));
  BSL_CUDA(cudaMalloc(&dsp, spair.size() * sizeof(int2)));
  BSL_CUDA(cudaMalloc(&dfi, fidx.size() * sizeof(int)));
  BSL_CUDA(cudaMemcpy(dt1, t.trig1.data(), t.trig1.size() * 8, cudaMemcpyHostToDevice));
  BSL_CUDA(cudaMemcpy(dt2, t.trig2.data(), t.trig2.size() * 8, cudaMemcpyHostToDevice));
  BSL_CUDA(cudaMemcpy(dleg, t.leg.data(), t.leg.size() * 8, cudaMemcpyHostToDevice));
  BSL_CUDA(cudaMemcpy(dwa, t.gl_w.data(), t.gl_w.size() * 8, cudaMemcpyHostToDevice));
  BSL_CUDA(cudaMemcpy(dwb, t.gc_w.data(), t.gc_w.size() * 8, cudaMemcpyHostToDevice));
  BSL_CUDA(cudaMemcpy(dmp, mpair.data(), mpair.size() * sizeof(int2), cudaMemcpyHostToDevice));
  BSL_CUDA(cudaMemcpy(dsp, spair.data(), spair.size() * sizeof(int2), cudaMemcpyHostToDevice));
  BSL_CUDA(cudaMemcpy(dfi, fidx.data(), fidx.size() * sizeof(int), cudaMemcpyHostToDevice));
  BlockTables bt{dt1, dt2, dleg, dwa, dwb, dmp, dsp, dfi, t.na, t.nb, nm, nmtri, t.nn, ntri};
  const size_t smem = 8 * ((size_t)2 * t.na * t.nb + (size_t)2 * nm * t.nb + (size_t)t.nn * t.na +
                           (size_t)t.na * nmtri);
  int rc = BSL_OK;
  if (smem > 220 * 1024) {
    rc = fail(BSL_ERR_UNSUPPORTED, "angular quadrature too large for the block assembly kernel");
  } else {
    cudaFuncSetAttribute(k_vblocks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_vblocks<<<(unsigned)t.npts, kThreads, smem, d.stream>>>(bt, d.v1, d.v2, t.npts, d.vb64, d.vb32,
                                                               vstream_tile_points());
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(d.stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "potential block assembly");
  }
  cudaFree(dt1); cudaFree(dt2); cudaFree(dleg); cudaFree(dwa); cudaFree(dwb);
  cudaFree(dmp); cudaFree(dsp); cudaFree(dfi);
  return rc;
}

int dev_hv(bsl_handle* h, const double* v, double* u, cudaStream_t s) {
  DeviceState& d = h->d;
  const long long D = bsl_packed_size(h);
  if (h->precision == BSL_PREC_MIXED) {
    k_to_f32<<<1024, kThreads, 0, s>>>(v, d.v32, D);
    if (h->kinetic_engine == BSL_KIN_TENSOR) {
      if (!d.vpair) BSL_CUDA(cudaMalloc(&d.vpair, (size_t)D * sizeof(float2)));
      k_pair_copy<<<1024, kThreads, 0, s>>>(v, d.vpair, D);
    }
    BSL_CUDA(cudaGetLastError());
  }
  int rc = launch_kinetic(h, v, d.vpair, s);
  if (rc) return rc;
  return launch_vapply(h, v, u, 0, 0, s);
}

// r -= alpha v, beta and the next scales, on FP64 or double-float buffers
int launch_update(bsl_handle* h, double* V, double* R, long long L, int j, cudaStream_t s) {
  DeviceState& d = h->d;
  if (h->state_pairs == 1 && h->kinetic_engine == BSL_KIN_TENSOR)  // nothing reads an FP32 copy of v
    return launch_update_stream(reinterpret_cast<const float2*>(V), reinterpret_cast<float2*>(R), L, d.partials,
                                d.counter, d.scalars, d.hist, d.hist_cap, j, d.jdev, d.status, s, h->tune_upd,
                                h->defer_reductions);
  if (h->state_pairs == 1)
    BSL_CUDA(launch_pdl(k_update_pair, dim3(d.pair_blocks), dim3(kThreads), 0, s, reinterpret_cast<const float2*>(V),
                        reinterpret_cast<float2*>(R), L, h->kinetic_engine == BSL_KIN_TENSOR ? nullptr : d.v32, L - 1,
                        d.partials, d.counter, d.scalars, d.hist, d.hist_cap, j, d.status));
  else
    k_update_fold<<<d.red_blocks, kThreads, 0, s>>>(V, R, L, d.v32, L - 1, d.partials, d.counter, d.scalars, d.hist,
                                                    d.hist_cap, j, d.status);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

namespace {
__global__ void k_set_iteration(int* jdev, int j, double* scalars) {
  *jdev = j;
  reinterpret_cast<int*>(scalars)[kPendingSlot] = 0;
}
}  // namespace

// the iteration counter read by the kernels of an iteration launched with j = 0
// (and no deferred beta pending)
int dev_set_iteration(bsl_handle* h, int j, cudaStream_t s) {
  k_set_iteration<<<1, 1, 0, s>>>(h->d.jdev, j, h->d.scalars);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

// Iterations whose kernels take j from the device counter (and so can be
// captured once and replayed): the double-float path with the tensor-core
// kinetic and the streamed update.
bool device_counted_iterations(const bsl_handle* h) {
  return h->precision == BSL_PREC_MIXED && h->state_pairs == 1 && h->kinetic_engine == BSL_KIN_TENSOR;
}

// Device-counted iterations (j = 0) defer their reductions: alpha's block
// totals are summed by the update's CTAs, beta's by the next iteration's x/y
// kinetic or dev_finish_iterations.
int dev_lanczos_iteration(bsl_handle* h, int j, cudaStream_t s) {
  DeviceState& d = h->d;
  const long long L = bsl_packed_size(h) + 1;  // + the coordinate outside the symmetry block
  double* V = h->lanczos_flip ? d.rvec : d.vec;
  double* R = h->lanczos_flip ? d.vec : d.rvec;
  h->defer_reductions = j == 0 && device_counted_iterations(h) ? 1 : 0;
  int rc = launch_kinetic(h, V, reinterpret_cast<const float2*>(V), s);
  if (h->defer_reductions && fused_iterations(h)) {
    // the block product of V was formed by the previous update (or
    // dev_begin_iterations); this update forms the next one
    StreamArgs a = vstream_args(h, V, R);
    if (!rc) rc = launch_vapply_light(a, h->t.nn, s);
    if (!rc) rc = launch_update_fused(a, h->t.nn, 1, s);
  } else {
    if (!rc) rc = launch_vapply(h, V, R, h->state_pairs == 1 ? 2 : 1, j, s);
    if (!rc) rc = launch_update(h, V, R, L, j, s);
  }
  h->defer_reductions = 0;
  if (rc) return rc;
  h->lanczos_flip ^= 1;
  return BSL_OK;
}

bool fused_iterations(const bsl_handle* h) {
  return device_counted_iterations(h) && fused_update_supported(h->vformat, h->t.nn);
}

int deferred_beta_count(bsl_handle* h) {
  if (fused_iterations(h)) return fused_update_ctas(vstream_args(h, h->d.vec, h->d.rvec), h->t.nn);
  return update_stream_ctas(h->tune_upd);
}

int ensure_product_buffer(bsl_handle* h) {
  DeviceState& d = h->d;
  if (!fused_iterations(h) || d.vprod) return BSL_OK;
  const size_t n = (size_t)h->t.npts * h->t.nn;
  const cudaError_t e = cudaMalloc(&d.vprod, n * sizeof(float));
  if (e != cudaSuccess) {
    d.vprod = nullptr;
    return fail(BSL_ERR_NOMEM, std::string("block product buffer: ") + cudaGetErrorString(e));
  }
  release_iteration_graph(d);  // no captured launch may hold the missing buffer
  return BSL_OK;
}

int dev_begin_iterations(bsl_handle* h, cudaStream_t s) {
  DeviceState& d = h->d;
  if (!fused_iterations(h)) return BSL_OK;
  if (int rc = ensure_product_buffer(h)) return rc;
  double* V = h->lanczos_flip ? d.rvec : d.vec;
  double* R = h->lanczos_flip ? d.vec : d.rvec;
  return launch_update_fused(vstream_args(h, V, R), h->t.nn, 2, s);
}

// the beta left pending by the last device-counted iteration
int dev_finish_iterations(bsl_handle* h, cudaStream_t s) {
  DeviceState& d = h->d;
  return launch_finish_beta(d.partials, deferred_beta_count(h), d.scalars, d.hist, d.hist_cap, d.jdev, d.status,
                            s);
}

// The same iteration with an event recorded after every kernel (ev[0] before).
int dev_lanczos_iteration_timed(bsl_handle* h, int j, cudaStream_t s, cudaEvent_t* ev) {
  DeviceState& d = h->d;
  struct Reset {
    bsl_handle* h;
    ~Reset() { h->defer_reductions = 0; }
  } reset{h};
  h->defer_reductions = j == 0 && device_counted_iterations(h) ? 1 : 0;
  const Tables& t = h->t;
  const long long L = bsl_packed_size(h) + 1;
  const bool mixed = h->precision == BSL_PREC_MIXED;
  double* V = h->lanczos_flip ? d.rvec : d.vec;
  double* R = h->lanczos_flip ? d.vec : d.rvec;
  const size_t sm_xy = sizeof(double) * t.nx * t.ny, sm_z = sizeof(double) * t.nx * t.nz;
  const dim3 gxy(t.nz, t.nn), gz(t.ny, t.nn);
  if (!mixed) {
    cudaFuncSetAttribute(k_kin_xy_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_xy);
    cudaFuncSetAttribute(k_kin_z_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_z);
  }
  int rc;
  cudaEventRecord(ev[0], s);
  if (mixed) {
    if ((rc = launch_kin_xy(h, reinterpret_cast<const float2*>(V), s))) return rc;
  } else {
    k_kin_xy_f64<<<gxy, kThreads, sm_xy, s>>>(V, d.ukin, d.tx, d.ty, t.nx, t.ny, t.nz);
  }
  cudaEventRecord(ev[1], s);
  if (mixed) {
    if ((rc = launch_kin_z(h, reinterpret_cast<const float2*>(V), s))) return rc;
  } else {
    k_kin_z_f64<<<gz, kThreads, sm_z, s>>>(V, d.ukin, d.tz, t.nx, t.ny, t.nz);
  }
  cudaEventRecord(ev[2], s);
  const bool fused = h->defer_reductions && fused_iterations(h);
  const StreamArgs fa = vstream_args(h, V, R);
  if ((rc = fused ? launch_vapply_light(fa, t.nn, s) : launch_vapply(h, V, R, h->state_pairs == 1 ? 2 : 1, j, s)))
    return rc;
  cudaEventRecord(ev[3], s);
  if ((rc = fused ? launch_update_fused(fa, t.nn, 1, s) : launch_update(h, V, R, L, j, s))) return rc;
  cudaEventRecord(ev[4], s);
  BSL_CUDA(cudaGetLastError());
  h->lanczos_flip ^= 1;
  return BSL_OK;
}

const char* dev_stage_name(bsl_handle* h, int i) {
  const bool mixed = h->precision == BSL_PREC_MIXED;
  static const char* n64[4] = {"k_kin_xy_f64", "k_kin_z_f64", "k_vapply<NN,double>", "k_update_fold"};
  static const char* nmx[4] = {"k_kin_xy_split", "k_kin_z_split", "k_vstream<NN>", "k_update_pair"};
  static const char* ntc[4] = {"k_kin_xy_tc", "k_kin_z_tc", "k_vstream<NN>", "k_update_stream"};
  if (!mixed) return n64[i];
  if (fused_iterations(h) && i >= 2)
    return i == 2 ? "k_vapply_light<NN>" : h->vformat == BSL_VFMT_GAUNT ? "k_vstream<NN,coefficients,update>"
                                                                        : "k_vstream<NN,fp32,update>";
  if (i == 2 && h->vformat == BSL_VFMT_GAUNT) return "k_vstream<NN,coefficients>";
  if (i == 2 && h->vformat == BSL_VFMT_BF16) return "k_vstream<NN,bf16>";
  return h->kinetic_engine == BSL_KIN_TENSOR ? ntc[i] : nmx[i];
}

int dev_to_pair(double* x, long long n, cudaStream_t s) {
  k_to_pair<<<1024, kThreads, 0, s>>>(x, n);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int dev_to_f32(const double* x, float* y, long long n, cudaStream_t s) {
  k_to_f32<<<1024, kThreads, 0, s>>>(x, y, n);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int dev_fill(double* x, long long L, double val, cudaStream_t s) {
  k_fill<<<1024, kThreads, 0, s>>>(x, L, val);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int dev_gather_packed(bsl_handle* h, const double* full, double* packed, cudaStream_t s) {
  const long long N = h->t.npts;
  k_gather<<<grid_for(N * h->t.nn), kThreads, 0, s>>>(full, packed, h->d.full_of, N, h->t.nn);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int dev_scatter_full(bsl_handle* h, const double* packed, double* full_accum, cudaStream_t s) {
  const long long N = h->t.npts;
  k_scatter_add<<<grid_for(N * h->t.nn), kThreads, 0, s>>>(packed, full_accum, h->d.full_of, N, h->t.nn);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

// H v of a full-layout FP64 vector into packed FP64 `out` (mode 0), without a
// packed FP64 copy on the mixed path.
int dev_hv_full(bsl_handle* h, const double* full, double* out, cudaStream_t s) {
  DeviceState& d = h->d;
  const long long N = h->t.npts, D = bsl_packed_size(h);
  if (h->precision != BSL_PREC_MIXED) {
    k_gather<<<grid_for(N * h->t.nn), kThreads, 0, s>>>(full, d.vec, d.full_of, N, h->t.nn);
    BSL_CUDA(cudaGetLastError());
    return dev_hv(h, d.vec, out, s);
  }
  const bool tc = h->kinetic_engine == BSL_KIN_TENSOR;
  if (tc && !d.vpair) BSL_CUDA(cudaMalloc(&d.vpair, (size_t)D * sizeof(float2)));
  k_gather_mixed<<<grid_for(D), kThreads, 0, s>>>(full, d.v32, tc ? d.vpair : nullptr, d.full_of, N, h->t.nn);
  BSL_CUDA(cudaGetLastError());
  int rc = launch_kinetic(h, nullptr, d.vpair, s);
  if (rc) return rc;
  return launch_vapply(h, nullptr, out, 0, 0, s);
}

// The full-layout host step after H v: r += S H v, alpha, beta, normalise and swap.
int dev_full_step_fused(bsl_handle* h, double* v, double* r, long long L, const double* hv, int j, cudaStream_t s,
                        double* v_out, double* r_out) {
  DeviceState& d = h->d;
  const int g = d.red_blocks;
  k_scatter_dot<<<g, kThreads, 0, s>>>(v, r, L, hv, d.packed_of, h->t.npts, h->t.nn_full, d.partials, d.counter,
                                       d.scalars, d.hist, j);
  k_beta_only<<<g, kThreads, 0, s>>>(v, r, L, d.partials, d.counter, d.scalars, d.hist, d.hist_cap, j, d.status);
  if (v_out)
    k_normalize_to<<<g, kThreads, 0, s>>>(v, r, L, d.scalars, v_out, r_out);
  else
    k_normalize_fused<<<g, kThreads, 0, s>>>(v, r, L, d.scalars);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int dev_ritz_accumulate(bsl_handle* h, const double* coef, const int* active, int ngood, double* ritz,
                        cudaStream_t s, bool previous) {
  const long long L = bsl_packed_size(h) + 1;  // with the coordinate outside the symmetry block
  const double* V = (h->lanczos_flip ^ (previous ? 1 : 0)) ? h->d.rvec : h->d.vec;
  k_ritz<<<1024, kThreads, 0, s>>>(V, L, coef, active, ngood, ritz, h->d.scalars, h->state_pairs == 1);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace bsl
