// Cullum-Willoughby tail of the Lanczos method on the host, FP64.
//
// Good eigenvalues of the Lanczos tridiagonal T_m by Sturm-sequence bisection
// with the spurious test against T_m with its first row and column removed,
// isolation flags and inverse-iteration error estimates; T_m eigenvectors for
// Ritz vectors.  Follows the reference's Fortran 77 routines
// (headLoop/LanczosCode/supportingRoutines/):
//   bisec.f:4-225   good/spurious eigenvalues in (emin, emax]
//   isoev.f:4-55    good eigenvalues next to a spurious one
//   inverr.f:4-233  error estimate beta_{m+1} |u_m| by inverse iteration
//   trivec.f:4-95, sturmi.f:99-211, inverm.f:215-353   T_m eigenvectors
// and their C++ driver lancbis.cpp:5-105.  Tolerances use EPS = 2 * 2^-53
// (LAPACK DLAMCH('E') doubled, as the Fortran does).  The inverse iterations
// start from a Park-Miller "minimal standard" sequence (x <- 16807 x mod
// 2^31-1, seed 1), the generator behind the GNU Fortran RAND the reference
// calls; the start vector affects error estimates and eigenvector signs only.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "bsl_internal.h"

namespace bsl {
namespace {

constexpr double kEps = 2.0 * 1.1102230246251565e-16;

void random_start(std::vector<double>* g, int n) {
  g->resize(n);
  uint64_t x = 1;
  for (int i = 0; i < n; ++i) {
    x = (16807ull * x) % 2147483647ull;
    const uint32_t bits = (uint32_t)(x - 1) & ~(uint32_t)511u;
    (*g)[i] = (double)((float)bits / 4294967296.0f);
  }
}

// Tridiagonal T with diagonal a[0..m-1] and off-diagonals b[1..m-1] (b[0] and
// b[m] are zero).  b2 holds the squares.
struct Tri {
  const double* a;
  std::vector<double> b, b2;
  int m;
};

// Number of eigenvalues of T greater than x (forward Sturm recurrence).
int count_above(const Tri& T, double x) {
  int c = 0;
  double u = 1.0;
  for (int i = 0; i < T.m; ++i) {
    const double w = (u == 0.0) ? T.b[i] / kEps : T.b2[i] / u;
    u = x - T.a[i] - w;
    if (u < 0.0) ++c;
  }
  return c;
}

// Backward recurrence: count for T (*all) and for T without its first row and
// column (*hat).
void count_above_backward(const Tri& T, double x, int* all, int* hat) {
  int c = 0, last = 0;
  double u = 1.0;
  for (int i = T.m - 1; i >= 0; --i) {
    const double w = (u == 0.0) ? T.b[i + 1] / kEps : T.b2[i + 1] / u;
    u = x - T.a[i] - w;
    last = (u < 0.0) ? 1 : 0;
    c += last;
  }
  *all = c;
  *hat = c - last;
}

// Distinct eigenvalues in (lo, hi] with multiplicities (0 = spurious).
// `unit` is the unit roundoff behind the multiplicity tolerances: 2^-52 (kEps)
// as in BISEC, or the effective unit roundoff of an inexact H v.
// `noise` (relative to max|T|, 0 for none) is a floor under the multiplicity
// window only: copies of a level closer than noise * max|T| count as one
// (a multiple eigenvalue, good), while an eigenvalue alone in that window is
// still tested against T without its first row in the window built on `unit`.
void bisect(const Tri& T, double lo, double hi, double unit, double noise, std::vector<double>* vs,
            std::vector<int>* mp) {
  const int m = T.m;
  double tkmax = 0.0;
  for (int i = 0; i < m; ++i) tkmax = std::max(std::max(std::fabs(T.a[i]), T.b[i]), tkmax);
  const double ttol = unit * tkmax;
  const double big = double(m + 1000);
  const double ep0 = big * ttol, ep1 = std::sqrt(big) * ttol;
  const double epm = std::max(ep0, noise * tkmax);  // multiplicity window
  const int above_hi = count_above(T, hi);
  const int mt = count_above(T, lo) - above_hi;
  vs->clear();
  mp->clear();
  if (mt <= 0) return;
  std::vector<double> lower(mt, lo), upper(mt, hi);
  int k = mt;
  while (k > 0) {
    double xl = lower[k - 1], xu = upper[k - 1];
    double x = xu;
    int nu = count_above(T, x) - above_hi;
    while (true) {
      x = (xl + xu) * 0.5;
      if (xu - xl <= kEps * (std::fabs(xl) + std::fabs(xu)) + ep1) break;
      const int c = count_above(T, x) - above_hi;
      if (c < k) {
        xu = x;
        nu = c;
        for (int i = 0; i < c; ++i) lower[i] = std::max(x, lower[i]);
        for (int i = c; i < k; ++i) upper[i] = std::min(x, upper[i]);
      } else {
        xl = x;
      }
    }
    vs->push_back(x);
    int kl, jl, ku, ju;
    count_above_backward(T, xl - epm, &kl, &jl);
    kl -= above_hi;
    jl -= above_hi;
    x = xu + epm;
    count_above_backward(T, x, &ku, &ju);
    ku -= above_hi;
    ju -= above_hi;
    int mult, knew;
    if (kl - ku - 1 == 0) {
      if (epm > ep0) {  // alone in the multiplicity window: the spurious test in the unit window
        count_above_backward(T, xl - ep0, &kl, &jl);
        count_above_backward(T, xu + ep0, &ku, &ju);
      }
      mult = (ju < jl) ? 0 : 1;
      knew = k - 1;
    } else {
      if (ku != nu) {
        while (true) {
          x = x + epm;
          const int c = count_above(T, x) - above_hi;
          const int diff = ku - c;
          ku = c;
          if (diff == 0) break;
        }
      }
      mult = kl - ku;
      knew = ku;
    }
    mp->push_back(mult);
    k = knew;
    for (int i = 0; i < knew; ++i) lower[i] = std::max(x, lower[i]);
  }
}

// Flag (-1) good eigenvalues whose nearest neighbour is spurious and closer
// than max(1e-8, 1e-8 |E|).
void flag_isolation(const std::vector<double>& vs, std::vector<int>* mp) {
  const int nd = (int)vs.size();
  if (nd < 2) return;
  double t0 = 0.0, t1 = 0.0, g = 0.0;
  for (int j = 0; j < nd; ++j) {
    if ((*mp)[j] != 1) continue;
    if (j != nd - 1) t1 = vs[j + 1] - vs[j];
    if (j != 0) t0 = vs[j] - vs[j - 1];
    if (j != 0 && j != nd - 1) g = (t0 < t1) ? -t0 : t1;
    else if (j == 0) g = vs[1] - vs[0];
    else g = vs[nd - 2] - vs[nd - 1];
    const int nb = (g >= 0.0) ? j + 1 : j - 1;
    if ((*mp)[nb] == 0) {
      const double tol = std::max(1.0e-8, 1.0e-8 * std::fabs(vs[j]));
      if (std::fabs(g) <= tol) (*mp)[j] = -(*mp)[j];
    }
  }
}

// Inverse iteration for (T_mev - x) u = g with partial pivoting (at most
// 10 steps); b is modified transiently and restored.  Returns the step count.
int inverse_iteration(const double* a, std::vector<double>& b, int mev, double x, double eps3, double eps4,
                      std::vector<double>& w, std::vector<double>& u) {
  int it = 1;
  while (true) {
    double piv = a[0] - x;
    double z = b[1];
    for (int i = 2; i <= mev; ++i) {
      if (b[i - 1] > std::fabs(piv)) {
        const double ratio = piv / b[i - 1];
        b[i - 1] = -b[i - 1];
        w[i - 2] = a[i - 1] - x;
        piv = z - ratio * w[i - 2];
        z = -ratio * b[i];
        const double tmp = u[i - 2];
        u[i - 2] = u[i - 1];
        u[i - 1] = tmp - ratio * u[i - 1];
      } else {
        w[i - 2] = z / piv;
        u[i - 2] = u[i - 2] / piv;
        u[i - 1] = u[i - 1] - b[i - 1] * u[i - 2];
        const double ratio = b[i - 1] / piv;
        piv = a[i - 1] - x - z * ratio;
        z = b[i];
      }
    }
    if (piv == 0.0) piv = eps3;
    u[mev - 1] = u[mev - 1] / piv;
    for (int i = mev - 1; i >= 1; --i) {
      if (b[i] < 0.0) {
        b[i] = -b[i];
        const double far = (i + 1 < mev) ? b[i + 1] * u[i + 1] : 0.0;
        u[i - 1] = (u[i - 1] - w[i - 1] * u[i] - far) / b[i];
      } else {
        u[i - 1] = u[i - 1] - w[i - 1] * u[i];
      }
    }
    double norm = std::fabs(u[mev - 1]);
    for (int i = mev - 2; i >= 0; --i) norm = norm + std::fabs(u[i]);
    if (norm >= 1.0) break;
    ++it;
    if (it > 10) break;
    const double sc = eps4 / norm;
    for (int i = 0; i < mev; ++i) u[i] = u[i] * sc;
  }
  return it;
}

void tolerances(const double* a, const std::vector<double>& b, int mev, double* eps3, double* eps4) {
  double tsum = std::fabs(a[0]);
  for (int i = 2; i <= mev; ++i) tsum = tsum + std::fabs(a[i - 1]) + b[i - 1];
  *eps3 = kEps * tsum;
  *eps4 = double(mev) * (*eps3);
}

void normalise(std::vector<double>& u, int mev) {
  double s = 0.0;
  for (int i = 0; i < mev; ++i) s = s + u[i] * u[i];
  s = 1.0 / std::sqrt(s);
  for (int i = 0; i < mev; ++i) u[i] = s * u[i];
}

}  // namespace

int cw_good_eigenvalues(int niter, const double* alpha, const double* beta, const double* beta2, double emin,
                        double emax, double* eval, double* err, int* ngood, double unit, double noise) {
  if (!(unit > 0.0)) unit = kEps;
  if (!(noise > 0.0)) noise = 0.0;
  (void)beta2;  // recomputed from beta, as BISEC does
  Tri T;
  T.a = alpha;
  T.m = niter;
  T.b.assign(beta, beta + niter + 1);
  const double beta_last = T.b[niter];
  T.b[niter] = 0.0;
  T.b2.resize(niter + 1);
  for (int i = 0; i <= niter; ++i) T.b2[i] = T.b[i] * T.b[i];
  std::vector<double> vs;
  std::vector<int> mp;
  bisect(T, emin, emax, unit, noise, &vs, &mp);
  flag_isolation(vs, &mp);
  // error estimates for isolated good eigenvalues
  const int nd = (int)vs.size();
  std::vector<double> e(nd, 0.0);
  std::vector<double> g, w(niter + 1, 0.0), u(niter + 1, 0.0);
  double eps3, eps4;
  tolerances(alpha, T.b, niter, &eps3, &eps4);
  random_start(&g, niter);
  double gsum = 0.0;
  for (int i = 0; i < niter; ++i) gsum = gsum + std::fabs(g[i]);
  gsum = eps4 / gsum;
  for (int i = 0; i < niter; ++i) g[i] = gsum * g[i];
  for (int jv = 0; jv < nd; ++jv) {
    if (mp[jv] != 1) continue;
    for (int i = 0; i < niter; ++i) u[i] = g[i];
    const int it = inverse_iteration(alpha, T.b, niter, vs[jv], eps3, eps4, w, u);
    normalise(u, niter);
    double est = beta_last * std::fabs(u[niter - 1]);
    if (it > 10) est = -est;
    e[jv] = est;
  }
  int n = 0;
  for (int i = 0; i < nd; ++i)
    if (mp[i] != 0) {
      eval[n] = vs[i];
      err[n] = e[i];
      ++n;
    }
  *ngood = n;
  return BSL_OK;
}

int cw_tm_eigenvectors(int niter, const double* alpha, const double* beta, const double* beta2,
                       const double* eval, int ngood, double* evtr) {
  std::vector<double> b(niter + 1), b2(niter + 1);
  b[0] = 0.0;
  b2[0] = 0.0;
  for (int j = 1; j <= niter; ++j) {
    b[j] = beta[j];
    b2[j] = beta2[j];
  }
  std::vector<double> g;
  random_start(&g, niter);
  std::vector<double> w(niter + 1, 0.0);
  std::fill(evtr, evtr + (size_t)niter * ngood, 0.0);
  for (int ig = 0; ig < ngood; ++ig) {
    const double x = eval[ig];
    // sizes at which x first appears (mk1) and doubles (mk2): two Sturm
    // sequences at x -/+ max(1e-10|x|, 5 (m+1000) EPS tkmax)
    double tkmax = 0.0;
    for (int i = 0; i < niter; ++i) tkmax = std::max(std::max(std::fabs(alpha[i]), b[i]), tkmax);
    const double toln = std::max(std::fabs(x) * 1.0e-10, 5.0 * double(niter + 1000) * kEps * tkmax);
    const double lo = x - toln, hi = x + toln;
    double u1 = 1.0, u2 = 1.0;
    int c1 = 0, c2 = 0, seen = 0, diff = 0, mk1 = 0, mk2 = 0, i;
    bool stopped = false;
    for (i = 1; i <= niter; ++i) {
      const double w1 = (u1 != 0.0) ? b2[i - 1] / u1 : b[i - 1] / kEps;
      u1 = lo - alpha[i - 1] - w1;
      if (u1 < 0.0) ++c1;
      const double w2 = (u2 != 0.0) ? b2[i - 1] / u2 : b[i - 1] / kEps;
      u2 = hi - alpha[i - 1] - w2;
      if (u2 < 0.0) ++c2;
      diff = c1 - c2;
      if (diff - seen >= 1) {
        if (seen == 0) mk1 = i;
        ++seen;
        if (seen > 1) {
          stopped = true;
          break;
        }
      }
    }
    if (!stopped) {
      i = niter;
      if (seen == 0) mk1 = niter;
    }
    mk2 = i;
    if (diff == 0) return fail(BSL_ERR_INPUT, "eigenvalue not found in the Lanczos matrix (STURMI)");
    int ma, ml, step;
    if (mk2 == niter) {
      ma = std::min((5 * mk1) / 4 + 1, niter);
      ml = niter;
      step = (std::min(niter, (13 * mk1) / 8 + 1) - ma) / 10 + 1;
    } else {
      ma = (3 * mk1 + mk2) / 4 + 1;
      ml = (mk1 + 3 * mk2) / 4;
      step = ((3 * mk1 + 5 * mk2) / 8 + 1 - ma) / 10 + 1;
    }
    double* col = evtr + (size_t)ig * niter;
    std::vector<double> u(col, col + niter);
    u.resize(niter + 1, 0.0);
    auto solve = [&](int mev, double* error, bool* conv) {
      const double bm = b[mev];
      b[mev] = 0.0;
      double eps3, eps4;
      tolerances(alpha, b, mev, &eps3, &eps4);
      double gs = 0.0;
      for (int q = 0; q < mev; ++q) gs = gs + std::fabs(g[q]);
      gs = eps4 / gs;
      for (int q = 0; q < mev; ++q) u[q] = gs * g[q];
      const int it = inverse_iteration(alpha, b, mev, x, eps3, eps4, w, u);
      normalise(u, mev);
      *error = std::fabs(u[mev - 1]);
      *conv = !(it > 10);
      b[mev] = bm;
    };
    int count = 0, best = ma;
    bool found = false;
    double errmin = 1.0;
    do {
      ++count;
      double error;
      bool conv;
      solve(ma, &error, &conv);
      for (int q = 0; q < ma; ++q) col[q] = u[q];
      found = found || conv;
      if (error <= errmin) {
        errmin = error;
        best = ma;
      }
      ma += step;
    } while (ma < ml && count <= 10);
    if (!found) return fail(BSL_ERR_INPUT, "inverse iteration never converged for Tm eigenvector " +
                                              std::to_string(ig + 1));
    double error;
    bool conv;
    solve(best, &error, &conv);
    for (int q = 0; q < best; ++q) col[q] = u[q];
  }
  return BSL_OK;
}

}  // namespace bsl
