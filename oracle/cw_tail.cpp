// ORACLE — test infrastructure only. Never linked into the product library.
//
// CPU restatement (C++, FP64) of the Cullum–Willoughby tridiagonal tail that the
// reference keeps in Fortran 77 (gfortran is not available here):
//   BISEC   headLoop/LanczosCode/supportingRoutines/bisec.f:4-225
//   ISOEV   headLoop/LanczosCode/supportingRoutines/isoev.f:4-55
//   INVERR  headLoop/LanczosCode/supportingRoutines/inverr.f:4-167
//   TRIVEC  headLoop/LanczosCode/supportingRoutines/trivec.f:4-95
//   STURMI  headLoop/LanczosCode/supportingRoutines/sturmi.f:4-116
//   INVERM  headLoop/LanczosCode/supportingRoutines/inverm.f:4-142
//   GENRAN  headLoop/LanczosCode/supportingRoutines/genran.f:4-32
//   SCALAR  headLoop/LanczosCode/supportingRoutines/scalar.f:4-21
//
// The entry points carry the gfortran ABI names (trailing underscore, every
// argument by reference, arrays 1-based in the Fortran text and 0-based here)
// so that the unmodified reference driver (lanczosEigenValuesVectors.cpp,
// lancbis.cpp) links against them.  The arithmetic follows the Fortran
// statement by statement so that the bisection results are bit-identical for
// identical alpha/beta input.
//
// Third-party algorithms restated here (not in the reference tree):
//  * LAPACK DLAMCH('E') (relative machine epsilon, rounding mode) = 2^-53.
//  * GNU Fortran runtime SRAND/RAND (libgfortran, linked by the reference
//    makefile's -lgfortran; the GCC version used in 2013 is not recorded).
//    Published algorithm: the Park–Miller "minimal standard" multiplicative
//    congruential generator x <- 16807 x mod (2^31-1) (Park & Miller, CACM 31,
//    1988), seed 0 replaced by 123459876; RAND returns the REAL(4) value
//    ((x-1) with its 9 low bits cleared) / 2^32.  Only ratios of these values
//    are used (INVERR/INVERM rescale the vector by EPS4/sum|G|), so the
//    overall power-of-two scale is immaterial.  The values affect only the
//    inverse-iteration start vectors (error estimates and Tm eigenvectors),
//    never the eigenvalues.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <vector>
#include <algorithm>

namespace {

const double kEps2 = 2.0 * 1.1102230246251565e-16;  // 2*DLAMCH('E')

void genran(int seed, double* r, int n) {
  uint64_t x = seed ? (uint64_t)seed : 123459876ull;
  for (int i = 0; i < n; ++i) {
    x = (16807ull * x) % 2147483647ull;
    uint32_t v = (uint32_t)(x - 1) & ~(uint32_t)511u;
    float f = (float)v / 4294967296.0f;
    r[i] = (double)f;
  }
}

double scalar(const double* a, const double* b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s = s + a[i] * b[i];
  return s;
}

// Sturm count below x1 with the forward recurrence (bisec.f:187-198).
// a: alpha[0..mev-1], b/b2: beta/beta2[0..mev] (Fortran BETA(1) == b[0]).
int sturm_forward(const double* a, const double* b, const double* b2, int mev,
                  double x1, int na, double eps) {
  int nev = -na;
  double yu = 1.0, yv;
  for (int i = 0; i < mev; ++i) {
    if (yu == 0.0) yv = b[i] / eps; else yv = b2[i] / yu;
    yu = x1 - a[i] - yv;
    if (yu < 0.0) nev++;
  }
  return nev;
}

// Backward recurrence (bisec.f:199-215): returns kev and jev (count without
// the last step) for the matrix with the first row and column deleted.
void sturm_backward(const double* a, const double* b, const double* b2, int mev,
                    double x1, int na, double eps, int* kev_out, int* jev_out) {
  int kev = -na, jev = 0;
  double yu = 1.0, yv;
  for (int i = mev - 1; i >= 0; --i) {
    if (yu == 0.0) yv = b[i + 1] / eps; else yv = b2[i + 1] / yu;
    yu = x1 - a[i] - yv;
    jev = 0;
    if (yu < 0.0) { kev++; jev = 1; }
  }
  *kev_out = kev;
  *jev_out = kev - jev;
}

}  // namespace

extern "C" {

double dlamch_(const char* cmach) {
  (void)cmach;
  return 1.1102230246251565e-16;
}

// BISEC (bisec.f:4-225).  vb has 2*nmax entries.
void bisec_(double* alpha, double* beta, double* beta2, int* mev_p, double* vs,
            int* mp, double* vb, int* nmax_p, double* bb_p, double* ub_p, int* ndis_p) {
  const int mev = *mev_p;
  (void)nmax_p;
  const double bb = *bb_p, ub = *ub_p;
  const double eps = kEps2;
  double tkmax = 0.0;
  for (int i = 0; i < mev; ++i) tkmax = std::max(std::max(std::fabs(alpha[i]), beta[i]), tkmax);
  const double ttol = eps * tkmax;
  const int mxstur = 100 * mev;
  int ndis = 0;
  const double betam = beta[mev];
  beta[mev] = 0.0;
  for (int i = 0; i <= mev; ++i) beta2[i] = beta[i] * beta[i];
  const double temp = (double)(mev + 1000);
  const double ep0 = temp * ttol;
  const double ep1 = std::sqrt(temp) * ttol;
  int na = 0;
  // counts at the interval ends
  int nev = sturm_forward(alpha, beta, beta2, mev, ub, na, eps);
  na = nev;
  nev = sturm_forward(alpha, beta, beta2, mev, bb, na, eps);
  const int mt = nev;
  if (30 * mt >= mxstur) {
    std::fprintf(stderr, "estimated number of Sturms exceeds limit in BISEC\n");
    std::exit(1);
  }
  if (mt != 0) {
    // vb[0..mt-1] lower bounds, vb[mt..2mt-1] upper bounds (Fortran VB(I), VB(MT+I))
    for (int i = 0; i < mt; ++i) { vb[i] = bb; vb[mt + i] = ub; }
    int k = mt;
    while (true) {
      double xl = vb[k - 1];
      double xu = vb[mt + k - 1];
      double x1 = xu;
      nev = sturm_forward(alpha, beta, beta2, mev, x1, na, eps);
      int nu = nev;
      // bisection (labels 170-220)
      while (true) {
        x1 = (xl + xu) * 0.5;
        double xs = std::fabs(xl) + std::fabs(xu);
        double x0 = xu - xl;
        double ept = eps * xs + ep1;
        if (x0 <= ept) break;
        nev = sturm_forward(alpha, beta, beta2, mev, x1, na, eps);
        if (nev < k) {
          xu = x1;
          nu = nev;
          for (int i = 0; i < nev; ++i) vb[i] = std::max(x1, vb[i]);
          for (int ii = nev + 1; ii <= k; ++ii) vb[mt + ii - 1] = std::min(x1, vb[mt + ii - 1]);
        } else {
          xl = x1;
        }
      }
      // label 230: converged eigenvalue x1; multiplicity / spurious test
      ndis++;
      vs[ndis - 1] = x1;
      int kl, jl, ku, ju;
      sturm_backward(alpha, beta, beta2, mev, xl - ep0, na, eps, &kl, &jl);
      x1 = xu + ep0;
      sturm_backward(alpha, beta, beta2, mev, x1, na, eps, &ku, &ju);
      int mpev, knew;
      if (kl - ku - 1 == 0) {
        mpev = 1;
        if (ju < jl) mpev = 0;
        knew = k - 1;
      } else {
        if (ku != nu) {
          while (true) {  // labels 260-270
            x1 = x1 + ep0;
            nev = sturm_forward(alpha, beta, beta2, mev, x1, na, eps);
            int kne = ku - nev;
            ku = nev;
            if (kne == 0) break;
          }
        }
        mpev = kl - ku;  // label 280
        knew = ku;
      }
      k = knew;  // label 300
      mp[ndis - 1] = mpev;
      if (k <= 0) break;
      for (int i = 0; i < knew; ++i) vb[i] = std::max(x1, vb[i]);
    }
  }
  beta[mev] = betam;
  *ndis_p = ndis;
}

// ISOEV (isoev.f:4-55)
void isoev_(double* vs, int* mp, int* ndis_p) {
  const int ndis = *ndis_p;
  const double gaptol = 1.0e-8;
  double t0 = 0.0, t1 = 0.0, g = 0.0;
  for (int j = 1; j <= ndis; ++j) {
    if (mp[j - 1] != 1) continue;
    if (j != ndis) t1 = vs[j] - vs[j - 1];
    if (j != 1) t0 = vs[j - 1] - vs[j - 2];
    if (j != 1 && j != ndis) {
      g = (t0 < t1) ? -t0 : t1;
    } else {
      if (j == 1) g = vs[1] - vs[0];
      if (j == ndis) g = vs[ndis - 2] - vs[ndis - 1];
    }
    int i = (g >= 0.0) ? j + 1 : j - 1;
    if (mp[i - 1] == 0) {
      double gap = std::fabs(g);
      double temp = std::max(gaptol, gaptol * std::fabs(vs[j - 1]));
      if (gap <= temp) mp[j - 1] = -mp[j - 1];
    }
  }
}

// Inverse iteration on T - x1 with partial pivoting, shared by INVERR
// (inverr.f:173-215) and INVERM (inverm.f:284-326).  v2 holds the start
// vector on entry; beta[mev] must be zero.  Returns the iteration count.
static int inverse_iterate(const double* alpha, double* beta, double* v1, double* v2,
                           int mev, double x1, double eps3, double eps4, int iter_max) {
  int it = 1;
  while (true) {
    double u = alpha[0] - x1;
    double z = beta[1];
    for (int i = 2; i <= mev; ++i) {
      if (beta[i - 1] > std::fabs(u)) {
        double ratio = u / beta[i - 1];
        beta[i - 1] = -beta[i - 1];
        v1[i - 2] = alpha[i - 1] - x1;
        u = z - ratio * v1[i - 2];
        z = -ratio * beta[i];
        double temp = v2[i - 2];
        v2[i - 2] = v2[i - 1];
        v2[i - 1] = temp - ratio * v2[i - 1];
      } else {
        v1[i - 2] = z / u;
        v2[i - 2] = v2[i - 2] / u;
        v2[i - 1] = v2[i - 1] - beta[i - 1] * v2[i - 2];
        double ratio = beta[i - 1] / u;
        u = alpha[i - 1] - x1 - z * ratio;
        z = beta[i];
      }
    }
    if (u == 0.0) u = eps3;
    v2[mev - 1] = v2[mev - 1] / u;
    for (int ii = 1; ii <= mev - 1; ++ii) {
      int i = mev - ii;
      if (beta[i] < 0.0) {
        beta[i] = -beta[i];
        v2[i - 1] = (v2[i - 1] - v1[i - 1] * v2[i] - beta[i + 1] * v2[i + 1]) / beta[i];
      } else {
        v2[i - 1] = v2[i - 1] - v1[i - 1] * v2[i];
      }
    }
    double xnorm = std::fabs(v2[mev - 1]);
    for (int ii = 1; ii <= mev - 1; ++ii) xnorm = xnorm + std::fabs(v2[mev - ii - 1]);
    if (xnorm >= 1.0) break;
    it++;
    if (it > iter_max) break;
    double xu = eps4 / xnorm;
    for (int i = 0; i < mev; ++i) v2[i] = v2[i] * xu;
  }
  return it;
}

// INVERR (inverr.f:70-233).  beta has mev+1 entries, v2 has mev+1.
void inverr_(double* alpha, double* beta, double* v1, double* v2, double* g, int* mev_p,
             double* vs, int* mp, double* err, int* ndis_p) {
  const int mev = *mev_p, ndis = *ndis_p;
  for (int i = 0; i < ndis; ++i) err[i] = 0.0;
  const double eps = kEps2;
  const int iter_max = 10;
  const double betam = beta[mev];
  beta[mev] = 0.0;
  double tsum = std::fabs(alpha[0]);
  for (int i = 2; i <= mev; ++i) tsum = tsum + std::fabs(alpha[i - 1]) + beta[i - 1];
  const double eps3 = eps * tsum;
  const double eps4 = (double)mev * eps3;
  genran(1, g, mev);
  double gsum = 0.0;
  for (int i = 0; i < mev; ++i) gsum = gsum + std::fabs(g[i]);
  gsum = eps4 / gsum;
  for (int i = 0; i < mev; ++i) g[i] = gsum * g[i];
  for (int jev = 0; jev < ndis; ++jev) {
    if (mp[jev] != 1) continue;
    const double x1 = vs[jev];
    for (int i = 0; i < mev; ++i) v2[i] = g[i];
    int it = inverse_iterate(alpha, beta, v1, v2, mev, x1, eps3, eps4, iter_max);
    double sum = scalar(v2, v2, mev);
    sum = 1.0 / std::sqrt(sum);
    for (int ii = 0; ii < mev; ++ii) v2[ii] = sum * v2[ii];
    double est = betam * std::fabs(v2[mev - 1]);
    if (it > iter_max) est = -est;
    err[jev] = est;
  }
  beta[mev] = betam;
}

}  // extern "C"

// STURMI (sturmi.f:99-211)
static void sturmi(const double* alpha, double* beta, const double* beta2, int mmax, double x1,
                   int* mk1, int* mk2) {
  const double epsm = kEps2;
  double tkmax = 0.0;
  for (int i = 0; i < mmax; ++i) tkmax = std::max(std::max(std::fabs(alpha[i]), beta[i]), tkmax);
  const double ttol = epsm * tkmax;
  const double xmltol = (double)(mmax + 1000) * ttol;
  const double stutol = 5.0 * xmltol;
  const double temp = std::fabs(x1) * 1.0e-10;
  const double toln = std::max(temp, stutol);
  *mk1 = 0;
  *mk2 = 0;
  beta[0] = 0.0;
  const double evl = x1 - toln, evu = x1 + toln;
  double u1 = 1.0, u2 = 1.0, v1, v2;
  int ic0 = 0, ic1 = 0, ic2 = 0, icd = 0;
  int i;
  bool jumped = false;
  for (i = 1; i <= mmax; ++i) {
    if (u1 != 0.0) v1 = beta2[i - 1] / u1; else v1 = beta[i - 1] / epsm;
    u1 = evl - alpha[i - 1] - v1;
    if (u1 < 0.0) ic1++;
    if (u2 != 0.0) v2 = beta2[i - 1] / u2; else v2 = beta[i - 1] / epsm;
    u2 = evu - alpha[i - 1] - v2;
    if (u2 < 0.0) ic2++;
    icd = ic1 - ic2;
    int ic = icd - ic0;
    if (ic >= 1) {
      if (ic0 == 0) *mk1 = i;
      ic0++;
      if (ic0 > 1) { jumped = true; break; }
    }
  }
  if (!jumped) {
    i = i - 1;  // Fortran DO variable is MMAX+1 after normal exit
    if (ic0 == 0) *mk1 = mmax;
  }
  *mk2 = i;
  if (icd == 0) {
    std::fprintf(stderr, "eigenvalue not found in STURMI\n");
    std::exit(1);
  }
}

// INVERM (inverm.f:215-353)
static void inverm(const double* alpha, double* beta, double* v1, double* v2, const double* g,
                   int mev, double x1, double* error, bool* qconv) {
  const double eps = kEps2;
  const int iter_max = 10;
  const double betam = beta[mev];
  beta[mev] = 0.0;
  double tsum = std::fabs(alpha[0]);
  for (int i = 2; i <= mev; ++i) tsum = tsum + std::fabs(alpha[i - 1]) + beta[i - 1];
  const double eps3 = eps * tsum;
  const double eps4 = (double)mev * eps3;
  double gsum = 0.0;
  for (int i = 0; i < mev; ++i) gsum = gsum + std::fabs(g[i]);
  gsum = eps4 / gsum;
  for (int i = 0; i < mev; ++i) v2[i] = gsum * g[i];
  int it = inverse_iterate(alpha, beta, v1, v2, mev, x1, eps3, eps4, iter_max);
  double sum = scalar(v2, v2, mev);
  sum = 1.0 / std::sqrt(sum);
  for (int ii = 0; ii < mev; ++ii) v2[ii] = sum * v2[ii];
  *error = std::fabs(v2[mev - 1]);
  // residual vector in v1 (inverm.f:333-339); kept for fidelity, unused by callers
  if (mev >= 2) {
    v1[mev - 1] = alpha[mev - 1] * v2[mev - 1] + beta[mev - 1] * v2[mev - 2] - x1 * v2[mev - 1];
    for (int j = 2; j <= mev - 1; ++j) {
      int jm = mev + 1 - j;
      v1[jm - 1] = alpha[jm - 1] * v2[jm - 1] + beta[jm - 1] * v2[jm - 2] + beta[jm] * v2[jm] - x1 * v2[jm - 1];
    }
    v1[0] = alpha[0] * v2[0] + beta[1] * v2[1] - x1 * v2[0];
  }
  *qconv = !(it > iter_max);
  beta[mev] = betam;
}

extern "C" {

// TRIVEC (trivec.f:4-95).  evtr is column-major [nit x ngood].
void trivec_(double* alpha, double* beta, double* bet2, double* wrk1, double* wrk2, int* nit_p,
             double* eval, int* ngood_p, double* evtr, double* mamin) {
  const int nit = *nit_p, ngood = *ngood_p;
  genran(1, wrk2, nit);
  for (int ig = 0; ig < ngood; ++ig) {
    int mk1, mk2;
    sturmi(alpha, beta, bet2, nit, eval[ig], &mk1, &mk2);
    int ma, ml, idelta;
    if (mk2 == nit) {
      ma = std::min((5 * mk1) / 4 + 1, nit);
      ml = nit;
      idelta = (std::min(nit, (13 * mk1) / 8 + 1) - ma) / 10 + 1;
    } else {
      ma = (3 * mk1 + mk2) / 4 + 1;
      ml = (mk1 + 3 * mk2) / 4;
      idelta = ((3 * mk1 + 5 * mk2) / 8 + 1 - ma) / 10 + 1;
    }
    int icount = 0;
    bool qfind = false;
    double errmin = 1.0;
    double* col = evtr + (size_t)ig * nit;
    // MAMIN is an INTEGER array in trivec.f but the C++ caller passes double*;
    // the reference reinterprets the storage.  Integers are kept here in an
    // int view of the same storage to reproduce that behaviour.
    int* mamin_i = reinterpret_cast<int*>(mamin);
    do {
      icount++;
      double error;
      bool qconv;
      inverm(alpha, beta, wrk1, col, wrk2, ma, eval[ig], &error, &qconv);
      qfind = qfind || qconv;
      if (error <= errmin) {
        errmin = error;
        mamin_i[ig] = ma;
      }
      ma = ma + idelta;
    } while (ma < ml && icount <= 10);
    if (!qfind) {
      std::fprintf(stderr, " IGOOD=%5d\nINVERM never converged in TRIVEC\n", ig + 1);
      std::exit(1);
    }
    double error;
    bool qconv;
    inverm(alpha, beta, wrk1, col, wrk2, mamin_i[ig], eval[ig], &error, &qconv);
    if (errmin > 1e-10)
      std::printf(" vector no. %4d has ERRMIN value > 1D-10: %8.2E\n\n", ig + 1, errmin);
  }
}

}  // extern "C"
