// Host side of the boundstate-lanczos GB300 library: input formats, basis and
// quadrature tables, cage geometry, device set-up and the C ABI.
//
// Reference behaviour followed (paths relative to the reference repository):
//   HvInputFile reader and checks  Hv-calculators/linRotor/cartSphBasis/HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:246-348
//   lm basis order                 Hv-calculators/linRotor/cartSphBasis/HvCalc/linRotCartSphHvRoutines.cpp:24-68
//   Gauss-Legendre nodes           same file :219-255
//   normalised Legendre functions  same file :293-403
//   tesseral trig factors          same file :405-434
//   uniform phi grid               same file :450-463, 1507-1514
//   sinc-DVR kinetic matrix        same file :484-517
//   rotor energies                 same file :522-538
//   symmetry mask                  HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:530-573
//   SPC/E cage geometry            potentialCalc/Alavi/SPCE/SPCE_AH2_EngRoutines.cpp:5-108, librarySources/matVecClasses/rotmat.cpp:6-32
//   Lanczos loop                   headLoop/LanczosCode/lanczosEigenValuesVectors.cpp:170-242, 371-469
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "bsl_internal.h"

namespace bsl {

namespace {
thread_local std::string g_last_error;

// SPC/E body frame (nm) and charges, SPCE_AH2_EngRoutines.h:17-30
const double kBodyO[3] = {0.0, 0.0, 0.006461408220};
const double kBodyH1[3] = {-8.164965810E-2, 0.0, -0.05127361870};
const double kBodyH2[3] = {8.164965810E-2, 0.0, -0.05127361870};
const double kQO = -0.8476, kQH = 0.4238;
// TIP4P body frame (nm), charges and O-H2 Lennard-Jones, TIP4P_AH2_EngRoutines.h
const double kT4O[3] = {0.0, 0.0, 0.00655538};
const double kT4H1[3] = {-0.075695, 0.0, -0.0520326};
const double kT4H2[3] = {0.075695, 0.0, -0.0520326};
const double kT4M[3] = {0.0, 0.0, -0.00844462};
const double kT4QH = 0.520, kT4QM = -1.040;
const double kT4A = 1.362e-06, kT4B = 1.532e-3;

double factorial(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f *= double(i);
  return f;
}

// Sinc-DVR kinetic matrix on n points spanning [-w/2, w/2] with dx = w/(n-1):
// T_ii' = hbar^2/(2 m dx^2) (-1)^(i-i') {pi^2/3 if i = i', 2/(i-i')^2 otherwise}.
void kinetic_matrix(double width, int n, double mass, std::vector<double>* T, std::vector<double>* grid) {
  const double dx = width / double(n - 1);
  T->resize((size_t)n * n);
  grid->resize(n);
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) {
      const int d = i - j;
      double t = (kHbar * kHbar) / (2.0 * mass * dx * dx) * ((d % 2 == 0) ? 1.0 : -1.0);
      t *= (d == 0) ? (kPi * kPi) / 3.0 : 2.0 / double(d * d);
      (*T)[(size_t)i * n + j] = t;
    }
    (*grid)[i] = double(i) * dx - width / 2.0;
  }
}

// Gauss-Legendre nodes and weights on [-1, 1] by Newton iteration on the
// three-term recurrence, roots filled symmetrically from both ends.
void gauss_legendre(int n, std::vector<double>* x, std::vector<double>* w) {
  x->assign(n, 0.0);
  w->assign(n, 0.0);
  const int half = (n + 1) / 2;
  for (int i = 1; i <= half; ++i) {
    double z = std::cos(M_PI * (double(i) - 0.25) / (double(n) + 0.5));
    double z_prev, dp;
    do {
      double p0 = 1.0, p1 = 0.0;
      for (int j = 1; j <= n; ++j) {
        const double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * double(j) - 1.0) * z * p1 - (double(j) - 1.0) * p2) / double(j);
      }
      // p0 = P_n(z), p1 = P_{n-1}(z)
      dp = double(n) * (z * p0 - p1) / (z * z - 1.0);
      z_prev = z;
      z = z_prev - p0 / dp;
    } while (std::fabs(z - z_prev) > DBL_EPSILON);
    (*x)[i - 1] = -z;
    (*x)[n - i] = z;
    (*w)[i - 1] = 2.0 / ((1.0 - z * z) * dp * dp);
    (*w)[n - i] = (*w)[i - 1];
  }
}

// Normalised associated Legendre values Ptilde_l^|m|(x) for l, m <= lmax:
// column recurrences in l, then N_lm = (-1)^m sqrt((l-m)!(2l+1)/(2(l+m)!)).
void legendre_table(int lmax, double x, std::vector<double>* P) {
  const int w = lmax + 1;
  P->assign((size_t)w * w, 0.0);
  auto at = [&](int l, int m) -> double& { return (*P)[(size_t)l * w + m]; };
  const double s = std::sqrt(1.0 - x * x);
  at(0, 0) = 1.0;
  for (int l = 1; l <= lmax; ++l) at(l, l) = (2.0 * double(l) - 1.0) * at(l - 1, l - 1) * s;
  for (int m = 0; m < lmax; ++m)
    for (int l = m; l < lmax; ++l) {
      const double below = (l - 1 < m) ? 0.0 : at(l - 1, m);
      at(l + 1, m) = (((2.0 * double(l) + 1.0) * x * at(l, m)) - ((double(l) + double(m)) * below)) /
                     (double(l) - double(m) + 1.0);
    }
  for (int l = 0; l <= lmax; ++l) {
    double sign = 1.0;
    for (int m = 0; m <= l; ++m) {
      at(l, m) *= sign * std::sqrt(factorial(l - m) * (2.0 * double(l) + 1.0) / (2.0 * factorial(l + m)));
      sign = -sign;
    }
  }
}

// Real (tesseral) phi factor: 1/sqrt(2 pi) for m = 0, cos(m phi)/sqrt(pi) for
// m > 0, sin(|m| phi)/sqrt(pi) for m < 0.
double trig_factor(int m, double phi) {
  const double r = 1.0 / std::sqrt(kPi);
  if (m == 0) return r / std::sqrt(2.0);
  if (m > 0) return r * std::cos(double(m) * phi);
  return r * std::sin(double(-m) * phi);
}

bool read_token_pairs(std::istream& f, std::vector<std::string>* vals, int count) {
  std::string key, val;
  for (int i = 0; i < count; ++i) {
    if (!(f >> key >> val)) return false;
    vals->push_back(val);
  }
  return true;
}

bool to_int(const std::string& s, int* v) {
  char* e = nullptr;
  long x = std::strtol(s.c_str(), &e, 10);
  if (e == s.c_str()) return false;
  *v = (int)x;
  return true;
}
bool to_double(const std::string& s, double* v) {
  char* e = nullptr;
  double x = std::strtod(s.c_str(), &e);
  if (e == s.c_str()) return false;
  *v = x;
  return true;
}

}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* where) {
  g_last_error = std::string("CUDA error in ") + where + ": " + cudaGetErrorString(e);
  return BSL_ERR_CUDA;
}

int build_tables(const bsl_hv_params& p, Tables* t) {
  t->nx = p.nx;
  t->ny = p.ny;
  t->nz = p.nz;
  t->npts = (long long)p.nx * p.ny * p.nz;
  t->lmax = p.l_max;
  t->nn_full = (p.l_max + 1) * (p.l_max + 1);
  t->na = p.theta_points;
  t->nb = p.phi_points;
  kinetic_matrix(p.x_max, p.nx, p.total_mass, &t->tx, &t->xg);
  kinetic_matrix(p.y_max, p.ny, p.total_mass, &t->ty, &t->yg);
  kinetic_matrix(p.z_max, p.nz, p.total_mass, &t->tz, &t->zg);
  t->l_of.clear();
  t->m_of.clear();
  for (int m = -p.l_max; m <= p.l_max; ++m)
    for (int l = std::abs(m); l <= p.l_max; ++l) {
      t->l_of.push_back(l);
      t->m_of.push_back(m);
    }
  t->full_of.clear();
  t->rot.clear();
  for (int n = 0; n < t->nn_full; ++n) {
    const int l = t->l_of[n];
    const bool keep = p.symmetry == BSL_SYM_ALL || (p.symmetry == BSL_SYM_EVEN && l % 2 == 0) ||
                      (p.symmetry == BSL_SYM_ODD && l % 2 == 1);
    if (!keep) continue;
    t->full_of.push_back(n);
    const double ld = double(l);
    t->rot.push_back(p.rotational_constant * ld * (ld + 1.0));
  }
  t->nn = (int)t->full_of.size();
  gauss_legendre(t->na, &t->gl_x, &t->gl_w);
  t->gc_x.resize(t->nb);
  t->gc_w.resize(t->nb);
  t->theta.resize(t->na);
  t->phi.resize(t->nb);
  t->phi2.resize(t->nb);
  for (int b = 0; b < t->nb; ++b) {
    t->gc_x[b] = std::cos(kPi * (2.0 * double(b + 1) - 1.0) / (2.0 * double(t->nb)));
    t->gc_w[b] = kPi / double(t->nb);
    t->phi[b] = std::acos(t->gc_x[b]);
    t->phi2[b] = 2 * kPi - std::acos(t->gc_x[b]);
  }
  for (int a = 0; a < t->na; ++a) t->theta[a] = std::acos(t->gl_x[a]);
  t->leg.assign((size_t)t->nn * t->na, 0.0);
  std::vector<double> P;
  for (int a = 0; a < t->na; ++a) {
    legendre_table(p.l_max, t->gl_x[a], &P);
    for (int s = 0; s < t->nn; ++s) {
      const int n = t->full_of[s];
      t->leg[(size_t)s * t->na + a] = P[(size_t)t->l_of[n] * (p.l_max + 1) + std::abs(t->m_of[n])];
    }
  }
  const int nm = 2 * p.l_max + 1;
  t->trig1.assign((size_t)nm * t->nb, 0.0);
  t->trig2.assign((size_t)nm * t->nb, 0.0);
  for (int m = -p.l_max; m <= p.l_max; ++m)
    for (int b = 0; b < t->nb; ++b) {
      t->trig1[(size_t)(m + p.l_max) * t->nb + b] = trig_factor(m, std::acos(t->gc_x[b]));
      t->trig2[(size_t)(m + p.l_max) * t->nb + b] = trig_factor(m, 2.0 * kPi - std::acos(t->gc_x[b]));
    }
  return BSL_OK;
}

namespace {
// ZYZ rotation R(phi, theta, chi) and its derivatives with respect to each angle
void zyz(const double* ea, double R[3][3], double dR[3][3][3]) {
  const double cp = std::cos(ea[0]), sp = std::sin(ea[0]), ct = std::cos(ea[1]), st = std::sin(ea[1]),
               cx = std::cos(ea[2]), sx = std::sin(ea[2]);
  const double M[3][3] = {{(cp * ct * cx) - (sp * sx), (-1 * cp * ct * sx) - (sp * cx), cp * st},
                          {(sp * ct * cx) + (cp * sx), (-1 * sp * ct * sx) + (cp * cx), sp * st},
                          {-1 * st * cx, st * sx, ct}};
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) R[r][k] = M[r][k];
  if (!dR) return;
  // d/dphi
  const double Dp[3][3] = {{-sp * ct * cx - cp * sx, sp * ct * sx - cp * cx, -sp * st},
                           {cp * ct * cx - sp * sx, -cp * ct * sx - sp * cx, cp * st},
                           {0.0, 0.0, 0.0}};
  // d/dtheta
  const double Dt[3][3] = {{-cp * st * cx, cp * st * sx, cp * ct}, {-sp * st * cx, sp * st * sx, sp * ct},
                           {-ct * cx, ct * sx, -st}};
  // d/dchi
  const double Dx[3][3] = {{-cp * ct * sx - sp * cx, -cp * ct * cx + sp * sx, 0.0},
                           {-sp * ct * sx + cp * cx, -sp * ct * cx - cp * sx, 0.0},
                           {st * sx, st * cx, 0.0}};
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) {
      dR[0][r][k] = Dp[r][k];
      dR[1][r][k] = Dt[r][k];
      dR[2][r][k] = Dx[r][k];
    }
}
const double* body_site(int model, int a) {
  if (model == BSL_POT_ALAVI_TIP4P) return a == 0 ? kT4O : (a == 1 ? kT4H1 : (a == 2 ? kT4H2 : kT4M));
  return a == 0 ? kBodyO : (a == 1 ? kBodyH1 : kBodyH2);
}
}  // namespace

void build_cage(int model, int nmol, const double* cm_ang, const double* euler, const double* q_site, Cage* c) {
  const bool t4 = cage_model(model) == BSL_POT_ALAVI_TIP4P;
  c->model = t4 ? BSL_POT_ALAVI_TIP4P : BSL_POT_ALAVI_SPCE;
  c->sites = t4 ? 4 : 3;
  c->lj_a = t4 ? kT4A : 1.364e-06;  // SPCE_AH2_EngRoutines.h:37-38
  c->lj_b = t4 ? kT4B : 1.533e-3;
  c->xyz.clear();
  c->q.clear();
  c->is_o.clear();
  c->cm_ang.assign(cm_ang, cm_ang + 3 * (size_t)nmol);
  c->euler.assign(euler, euler + 3 * (size_t)nmol);
  const double qs[4] = {t4 ? 0.0 : kQO, t4 ? kT4QH : kQH, t4 ? kT4QH : kQH, kT4QM};
  for (int i = 0; i < nmol; ++i) {
    double R[3][3];
    zyz(euler + 3 * i, R, nullptr);
    for (int a = 0; a < c->sites; ++a) {
      const double* b = body_site(c->model, a);
      for (int r = 0; r < 3; ++r) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += R[r][k] * b[k];
        c->xyz.push_back(s + kNmPerAngstrom * cm_ang[3 * i + r]);
      }
      c->q.push_back(q_site ? q_site[c->sites * i + a] : qs[a]);
      c->is_o.push_back(a == 0 ? 1 : 0);
    }
  }
}

void site_angle_derivative(const Cage& c, int m, int a, int k, double* out) {
  double R[3][3], dR[3][3][3];
  zyz(&c.euler[3 * (size_t)m], R, dR);
  const double* b = body_site(c.model, a);
  for (int r = 0; r < 3; ++r) out[r] = dR[k][r][0] * b[0] + dR[k][r][1] * b[1] + dR[k][r][2] * b[2];
}

int read_cage(const std::string& path, int model, Cage* c) {
  std::ifstream f(path);
  if (!f.is_open()) return fail(BSL_ERR_INPUT, "Atom geometry file '" + path + "' could not be opened.");
  int nmol = 0;
  std::string line;
  if (!(f >> nmol) || nmol <= 0) return fail(BSL_ERR_INPUT, "geometry file '" + path + "': bad molecule count");
  std::getline(f, line);
  std::getline(f, line);
  std::vector<double> cm(3 * (size_t)nmol), ea(3 * (size_t)nmol);
  for (int i = 0; i < nmol; ++i) {
    std::string name;
    if (!(f >> name >> cm[3 * i] >> ea[3 * i] >> cm[3 * i + 1] >> ea[3 * i + 1] >> cm[3 * i + 2] >> ea[3 * i + 2]))
      return fail(BSL_ERR_INPUT, "geometry file '" + path + "': expected " + std::to_string(nmol) +
                                     " molecules, read " + std::to_string(i));
  }
  build_cage(model, nmol, cm.data(), ea.data(), nullptr, c);
  return BSL_OK;
}

namespace {

void free_device(DeviceState& d) {
  release_iteration_graph(d);
  void* ptrs[] = {d.tx, d.ty, d.tz, d.kx_head, d.ky_head, d.kz_head, d.kx_band, d.ky_band, d.kz_band, d.rot,
                  d.v1, d.v2, d.vb64, d.vb32, d.vec, d.rvec, d.ukin, d.v32, d.rot_hi, d.rot_lo, d.partials,
                  d.counter,
                  d.scalars, d.status, d.hist, d.ref_vec, d.ref_out, d.full_of, d.packed_of, d.ritz};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (d.vpair) cudaFree(d.vpair);
  if (d.kxy_slices) cudaFree(d.kxy_slices);
  if (d.kz_slices) cudaFree(d.kz_slices);
  if (d.jdev) cudaFree(d.jdev);
  if (d.vb16) cudaFree(d.vb16);
  if (d.vscale) cudaFree(d.vscale);
  if (d.vc32) cudaFree(d.vc32);
  if (d.vprod) cudaFree(d.vprod);
  if (d.copy_done) cudaEventDestroy(d.copy_done);
  if (d.vec_in) cudaEventDestroy(d.vec_in);
  if (d.copy_stream) cudaStreamDestroy(d.copy_stream);
  if (d.ev0) cudaEventDestroy(d.ev0);
  if (d.ev1) cudaEventDestroy(d.ev1);
  if (d.stream) cudaStreamDestroy(d.stream);
  d = DeviceState();
}

template <typename T>
int dalloc(T** p, size_t n, const char* what) {
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T) + 16);
  if (e != cudaSuccess) return fail(BSL_ERR_NOMEM, std::string("device allocation failed for ") + what + ": " +
                                                       cudaGetErrorString(e));
  return BSL_OK;
}

template <typename T>
int upload(T** p, const std::vector<T>& host, const char* what) {
  int rc = dalloc(p, host.size(), what);
  if (rc) return rc;
  BSL_CUDA(cudaMemcpy(*p, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice));
  return BSL_OK;
}

int validate(const bsl_hv_params& p) {
  if (p.x_max > p.px_max || p.y_max > p.py_max || p.z_max > p.pz_max)
    return fail(BSL_ERR_INPUT,
                "Error, the system's physical dimensions must be the same size or smaller than the potential "
                "universe dimensions.");
  if (p.x_max * p.px_max * p.y_max * p.py_max * p.z_max * p.pz_max < DBL_EPSILON ||
      (long long)p.nx * p.ny * p.nz * p.pnx * p.pny * p.pnz == 0)
    return fail(BSL_ERR_INPUT, "Error, none of the system dimensions nor the number of points can be zero.");
  if (p.nx < 2 || p.ny < 2 || p.nz < 2) return fail(BSL_ERR_INPUT, "grids need at least 2 points per axis");
  if (p.l_max < 0 || p.theta_points < 1 || p.phi_points < 1)
    return fail(BSL_ERR_INPUT, "l_max, thetaPoints and phiPoints must be positive");
  if (p.symmetry < BSL_SYM_ALL || p.symmetry > BSL_SYM_ODD)
    return fail(BSL_ERR_INPUT, "ERROR: Symmeterizer Flag not recognized.");
  if (p.symmetry == BSL_SYM_ODD && p.l_max < 1) return fail(BSL_ERR_INPUT, "Odd symmetry needs l_max >= 1");
  if (p.potential < BSL_POT_ALAVI_SPCE || p.potential > BSL_POT_COULOMB)
    return fail(BSL_ERR_INPUT, "unknown potential");
  if (p.precision != BSL_PREC_FP64 && p.precision != BSL_PREC_MIXED)
    return fail(BSL_ERR_INPUT, "unknown precision");
  return BSL_OK;
}

}  // namespace
// HvPrep with the cage either from the geometry file (cage == null) or given
int hv_prep(const bsl_hv_params* params, const Cage* cage, bsl_handle** out) {
  if (!params || !out) return fail(BSL_ERR_INPUT, "null argument");
  *out = nullptr;
  int rc = validate(*params);
  if (rc) return rc;
  bsl_handle* h = new bsl_handle();
  h->p = *params;
  h->precision = params->precision;
  rc = build_tables(h->p, &h->t);
  if (rc) { delete h; return rc; }
  if (h->t.nn > kMaxNN) {
    delete h;
    return fail(BSL_ERR_UNSUPPORTED, "symmetry block with " + std::to_string(h->t.nn) + " (l,m) functions exceeds " +
                                         std::to_string(kMaxNN));
  }
  if (has_cage(h->p.potential)) {
    if (cage) {
      h->cage = *cage;
    } else {
      rc = read_cage(h->p.geometry_filename, h->p.potential, &h->cage);
      if (rc) { delete h; return rc; }
    }
  }
  auto bail = [&](int code) {
    free_device(h->d);
    delete h;
    return code;
  };
  cudaError_t e = cudaSetDevice(h->p.device);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaSetDevice"));
  DeviceState& d = h->d;
  if ((e = cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaStreamCreate"));
  if ((e = cudaEventCreate(&d.ev0)) != cudaSuccess || (e = cudaEventCreate(&d.ev1)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaEventCreate"));
  const Tables& t = h->t;
  std::vector<float> hi, lo;
  if ((rc = upload(&d.tx, t.tx, "Tx")) || (rc = upload(&d.ty, t.ty, "Ty")) || (rc = upload(&d.tz, t.tz, "Tz")))
    return bail(rc);
  kinetic_split_tables(t.tx, t.nx, true, &hi, &lo);
  if ((rc = upload(&d.kx_head, hi, "Tx")) || (rc = upload(&d.kx_band, lo, "Tx"))) return bail(rc);
  kinetic_split_tables(t.ty, t.ny, false, &hi, &lo);
  if ((rc = upload(&d.ky_head, hi, "Ty")) || (rc = upload(&d.ky_band, lo, "Ty"))) return bail(rc);
  kinetic_split_tables(t.tz, t.nz, false, &hi, &lo);
  if ((rc = upload(&d.kz_head, hi, "Tz")) || (rc = upload(&d.kz_band, lo, "Tz"))) return bail(rc);
  if (kinetic_tc_supported(t)) {
    std::vector<uint16_t> sl;
    kinetic_smem_image(t.tx, t.nx, true, &sl, &d.e_txy);
    if ((rc = upload(&d.kxy_slices, sl, "Tx"))) return bail(rc);
    kinetic_smem_image(t.tz, t.nz, false, &sl, &d.e_tz);
    if ((rc = upload(&d.kz_slices, sl, "Tz"))) return bail(rc);
    h->kinetic_engine = BSL_KIN_TENSOR;
  }
  if ((rc = upload(&d.rot, t.rot, "rotor"))) return bail(rc);
  {
    std::vector<float> rh(t.rot.size()), rl(t.rot.size());
    for (size_t i = 0; i < t.rot.size(); ++i) {
      rh[i] = (float)t.rot[i];
      rl[i] = (float)(t.rot[i] - (double)rh[i]);
    }
    if ((rc = upload(&d.rot_hi, rh, "rotor")) || (rc = upload(&d.rot_lo, rl, "rotor"))) return bail(rc);
  }
  if ((rc = upload(&d.full_of, t.full_of, "index map"))) return bail(rc);
  {
    std::vector<int> pof(t.nn_full, -1);
    for (int s2 = 0; s2 < t.nn; ++s2) pof[t.full_of[s2]] = s2;
    if ((rc = upload(&d.packed_of, pof, "index map"))) return bail(rc);
  }
  const size_t N = (size_t)t.npts, D = N * t.nn;
  const size_t ngrid = N * t.na * t.nb;
  const size_t ntri = (size_t)t.nn * (t.nn + 1) / 2;
  const size_t tp = (size_t)vstream_tile_points(), tiled = (N + tp - 1) / tp * tp;
  if ((rc = dalloc(&d.v1, ngrid, "potential grid")) || (rc = dalloc(&d.v2, ngrid, "potential grid")) ||
      (rc = dalloc(&d.vb64, ntri * N, "potential blocks")) || (rc = dalloc(&d.vb32, ntri * tiled, "potential blocks")) ||
      (rc = dalloc(&d.vec, D + 1, "Lanczos vector")) || (rc = dalloc(&d.rvec, D + 1, "Lanczos vector")) ||
      (rc = dalloc(&d.ukin, D, "kinetic work")) || (rc = dalloc(&d.v32, D, "FP32 Lanczos copy")))
    return bail(rc);
  d.red_blocks = 1216;
  {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->p.device);
    d.pair_blocks = 3 * (sms > 0 ? sms : 152);  // 3 resident 256-thread blocks per SM (80 registers)
  }
  // one partial per block of the widest reducing launch (the per-point potential
  // apply); deferred beta totals from kBetaPartials on
  const size_t nparts = std::max({(size_t)d.red_blocks, (N + 63) / 64, (size_t)(kBetaPartials + d.red_blocks)}) + 64;
  if ((rc = dalloc(&d.partials, nparts, "reduction scratch")) ||
      (rc = dalloc(&d.counter, 4, "reduction counter")) || (rc = dalloc(&d.scalars, 16, "scalars")) ||
      (rc = dalloc(&d.status, 4, "status")) || (rc = dalloc(&d.jdev, 1, "iteration counter")))
    return bail(rc);
  if ((e = cudaMemset(d.counter, 0, 4 * sizeof(unsigned int))) != cudaSuccess) return bail(cuda_fail(e, "memset"));
  if ((e = cudaMemset(d.status, 0, 4 * sizeof(int))) != cudaSuccess) return bail(cuda_fail(e, "memset"));
  // zero the padding points of the last tile of the streamed FP32 blocks
  if ((e = cudaMemset(d.vb32, 0, ntri * tiled * sizeof(float))) != cudaSuccess) return bail(cuda_fail(e, "memset"));
  switch (h->p.potential) {
    case BSL_POT_ISOHARMOSC: rc = dev_potential_iso(h); break;
    case BSL_POT_COULOMB: rc = dev_potential_coulomb(h); break;
    case BSL_POT_POINT_ALAVI_SPCE:
    case BSL_POT_POINT_ALAVI_TIP4P: rc = dev_potential_point_alavi(h); break;
    default: rc = dev_potential_alavi(h);
  }
  if (rc) return bail(rc);
  if ((rc = dev_vblocks(h))) return bail(rc);
  // the mixed path streams the blocks as spherical-harmonic coefficients where
  // the basis has a generated expansion and the blocks reproduce from them
  if (gaunt_coefficient_count(h) > 0) {
    double resid = 0.0, vmax = 0.0;
    if ((rc = dev_gaunt_coeffs(h, &resid, &vmax))) return bail(rc);
    h->gaunt_residual = resid;
    if (resid <= 1e-10 * vmax) {
      h->vformat = BSL_VFMT_GAUNT;
    } else {
      cudaFree(d.vc32);
      d.vc32 = nullptr;
    }
  }
  if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess) return bail(cuda_fail(e, "HvPrep"));
  // the potential grid is only needed to build the blocks; keep it for
  // inspection (bsl_copy_vgrid) when it is small
  if (ngrid > ((size_t)1 << 26) && !h->p.keep_potential_grid) {
    cudaFree(d.v1);
    cudaFree(d.v2);
    d.v1 = d.v2 = nullptr;
  }
  *out = h;
  return BSL_OK;
}

}  // namespace bsl

using namespace bsl;

extern "C" {

const char* bsl_last_error(void) { return g_last_error.c_str(); }

int bsl_parse_hv_input(const char* path, bsl_hv_params* out) {
  if (!path || !out) return fail(BSL_ERR_INPUT, "null argument");
  std::ifstream f(path);
  if (!f.is_open()) return fail(BSL_ERR_INPUT, std::string("Input file '") + path + "' could not be opened.");
  std::string line;
  std::getline(f, line);
  std::getline(f, line);
  std::vector<std::string> v;
  if (!read_token_pairs(f, &v, 22))
    return fail(BSL_ERR_INPUT, std::string("Input file '") + path + "' is truncated: expected 22 key/value pairs");
  bsl_hv_params p;
  std::memset(&p, 0, sizeof(p));
  bool ok = to_int(v[0], &p.nx) && to_double(v[1], &p.x_max) && to_int(v[2], &p.ny) && to_double(v[3], &p.y_max) &&
            to_int(v[4], &p.nz) && to_double(v[5], &p.z_max) && to_int(v[6], &p.l_max) &&
            to_int(v[7], &p.theta_points) && to_int(v[8], &p.phi_points) && to_int(v[9], &p.pnx) &&
            to_double(v[10], &p.px_max) && to_int(v[11], &p.pny) && to_double(v[12], &p.py_max) &&
            to_int(v[13], &p.pnz) && to_double(v[14], &p.pz_max) && to_double(v[15], &p.total_mass) &&
            to_double(v[16], &p.rotational_constant) && to_double(v[19], &p.ceiling_potential);
  if (!ok) return fail(BSL_ERR_INPUT, std::string("Input file '") + path + "': malformed number");
  std::snprintf(p.geometry_filename, sizeof(p.geometry_filename), "%s", v[17].c_str());
  std::snprintf(p.simulation_title, sizeof(p.simulation_title), "%s", v[18].c_str());
  p.quadrature_study = (v[20] == "TRUE");
  if (v[21] == "All") p.symmetry = BSL_SYM_ALL;
  else if (v[21] == "Even") p.symmetry = BSL_SYM_EVEN;
  else if (v[21] == "Odd") p.symmetry = BSL_SYM_ODD;
  else return fail(BSL_ERR_INPUT, "ERROR: Symmeterizer Flag not recognized.");
  p.potential = BSL_POT_ALAVI_SPCE;
  p.precision = BSL_PREC_FP64;
  p.device = 0;
  // the reference checks the geometry file before any computation (:330-337)
  if (std::string(p.geometry_filename) != "NULL") {
    std::ifstream g(p.geometry_filename);
    if (!g.is_open())
      return fail(BSL_ERR_INPUT, std::string("Atom geometry file '") + p.geometry_filename + "' could not be opened.");
  }
  int rc = validate(p);
  if (rc) return rc;
  *out = p;
  return BSL_OK;
}

int bsl_parse_isoharmosc_input(const char* path, bsl_hv_params* inout) {
  if (!path || !inout) return fail(BSL_ERR_INPUT, "null argument");
  std::ifstream f(path);
  if (!f.is_open())
    return fail(BSL_ERR_INPUT,
                std::string("Isotropic Harmonic Oscillator Potential input file '") + path + "' could not be opened.");
  std::string line;
  std::getline(f, line);
  std::getline(f, line);
  std::vector<std::string> v;
  if (!read_token_pairs(f, &v, 3)) return fail(BSL_ERR_INPUT, "IsoHarmOsc input file is truncated");
  if (!(to_double(v[0], &inout->iso_mass) && to_double(v[1], &inout->iso_frequency) &&
        to_double(v[2], &inout->iso_ceiling)))
    return fail(BSL_ERR_INPUT, "IsoHarmOsc input file: malformed number");
  inout->potential = BSL_POT_ISOHARMOSC;
  return BSL_OK;
}

int bsl_parse_coulomb_input(const char* path, bsl_hv_params* inout) {
  if (!path || !inout) return fail(BSL_ERR_INPUT, "null argument");
  std::ifstream f(path);
  if (!f.is_open())
    return fail(BSL_ERR_INPUT, std::string("Coulomb Potential input file '") + path + "' could not be opened.");
  std::string line;
  std::getline(f, line);
  std::getline(f, line);
  std::vector<std::string> v;
  if (!read_token_pairs(f, &v, 3)) return fail(BSL_ERR_INPUT, "Coulomb input file is truncated");
  if (!(to_double(v[0], &inout->coulomb_centre_charge) && to_double(v[1], &inout->coulomb_mol_charge) &&
        to_double(v[2], &inout->coulomb_ceiling)))
    return fail(BSL_ERR_INPUT, "Coulomb input file: malformed number");
  inout->potential = BSL_POT_COULOMB;
  return BSL_OK;
}

int bsl_calculator_potential(const char* calculator, int* potential) {
  if (!calculator || !potential) return fail(BSL_ERR_INPUT, "null argument");
  std::string c(calculator);
  static const struct {
    const char* name;
    int potential;
  } kPointGrid[] = {{"linRotCartSph_NoQuad_Alavi_SPCE", BSL_POT_POINT_ALAVI_SPCE},
                    {"linRotCartSph_NoQuad_Alavi_TIP4P", BSL_POT_POINT_ALAVI_TIP4P},
                    {"linRotCartSph_NoQuad_Coulomb", BSL_POT_COULOMB}};
  for (const auto& e : kPointGrid)
    if (c == e.name || c == std::string(e.name) + "_GB300") {
      *potential = e.potential;
      return BSL_OK;
    }
  if (c == "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE" || c == "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE_GB300") {
    *potential = BSL_POT_ALAVI_SPCE;
    return BSL_OK;
  }
  if (c == "linRotCartSph_NoQuad_ContGrid_Alavi_TIP4P" || c == "linRotCartSph_NoQuad_ContGrid_Alavi_TIP4P_GB300") {
    *potential = BSL_POT_ALAVI_TIP4P;
    return BSL_OK;
  }
  if (c == "linRotCartSph_NoQuad_IsoHarmOsc" || c == "linRotCartSph_NoQuad_IsoHarmOsc_GB300") {
    *potential = BSL_POT_ISOHARMOSC;
    return BSL_OK;
  }
  return fail(BSL_ERR_INPUT, "HvCalculator '" + c + "' not recognized.");
}

int bsl_hv_prep(const bsl_hv_params* params, bsl_handle** out) { return hv_prep(params, nullptr, out); }

int bsl_cage_sites(int potential, int nmol, const double* cm_ang, const double* euler, const double* q_site,
                   double* xyz, double* q) {
  if (nmol < 1 || !cm_ang || !euler || !xyz || !q) return fail(BSL_ERR_INPUT, "bad arguments");
  Cage c;
  build_cage(potential, nmol, cm_ang, euler, q_site, &c);
  std::copy(c.xyz.begin(), c.xyz.end(), xyz);
  std::copy(c.q.begin(), c.q.end(), q);
  return BSL_OK;
}

int bsl_rigid_body_gradient(int potential, int nmol, const double* cm_ang, const double* euler, int nlev,
                            const double* dr_site, double* d_cm, double* d_euler) {
  if (nmol < 1 || nlev < 1 || !cm_ang || !euler || !dr_site || !d_cm || !d_euler)
    return fail(BSL_ERR_INPUT, "bad arguments");
  Cage c;
  build_cage(potential, nmol, cm_ang, euler, nullptr, &c);
  const int S = c.sites;
  for (int n = 0; n < nlev; ++n)
    for (int m = 0; m < nmol; ++m) {
      double gc[3] = {0, 0, 0}, ge[3] = {0, 0, 0};
      for (int a = 0; a < S; ++a) {
        const double* g = dr_site + ((size_t)n * S * nmol + S * m + a) * 3;
        for (int k = 0; k < 3; ++k) gc[k] += kNmPerAngstrom * g[k];  // site = R body + 0.1 cm
        for (int k = 0; k < 3; ++k) {
          double dsite[3];
          site_angle_derivative(c, m, a, k, dsite);
          ge[k] += g[0] * dsite[0] + g[1] * dsite[1] + g[2] * dsite[2];
        }
      }
      for (int k = 0; k < 3; ++k) {
        d_cm[((size_t)n * nmol + m) * 3 + k] = gc[k];
        d_euler[((size_t)n * nmol + m) * 3 + k] = ge[k];
      }
    }
  return BSL_OK;
}

int bsl_hv_prep_cage(const bsl_hv_params* params, int nmol, const double* cm_ang, const double* euler,
                     const double* q_site, const double* q_alavi, bsl_handle** out) {
  if (!params || !out || nmol < 1 || !cm_ang || !euler) return fail(BSL_ERR_INPUT, "bad arguments");
  if (!has_cage(params->potential)) return fail(BSL_ERR_INPUT, "a cage needs an Alavi potential");
  Cage c;
  build_cage(params->potential, nmol, cm_ang, euler, q_site, &c);
  if (q_alavi) {
    c.q_h2_h = q_alavi[0];
    c.q_h2_cm = q_alavi[1];
  }
  return hv_prep(params, &c, out);
}

void bsl_destroy(bsl_handle* h) {
  if (!h) return;
  cudaSetDevice(h->p.device);
  free_device(h->d);
  delete h;
}

long long bsl_basis_size(const bsl_handle* h) { return h ? h->t.npts * h->t.nn_full : -1; }
long long bsl_packed_size(const bsl_handle* h) { return h ? h->t.npts * h->t.nn : -1; }
int bsl_packed_nn(const bsl_handle* h) { return h ? h->t.nn : -1; }
void* bsl_stream(const bsl_handle* h) { return h ? (void*)h->d.stream : nullptr; }

int bsl_set_precision(bsl_handle* h, int precision) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (precision != BSL_PREC_FP64 && precision != BSL_PREC_MIXED) return fail(BSL_ERR_INPUT, "unknown precision");
  h->precision = precision;
  return BSL_OK;
}

int bsl_set_kinetic_engine(bsl_handle* h, int engine) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (engine != BSL_KIN_SIMT && engine != BSL_KIN_TENSOR) return fail(BSL_ERR_INPUT, "unknown kinetic engine");
  if (engine == BSL_KIN_TENSOR && !h->d.kxy_slices)
    return fail(BSL_ERR_UNSUPPORTED, "tensor-core kinetic needs at most 64 points per axis and equal x and y axes");
  if (engine != h->kinetic_engine) h->state_pairs = -1;  // the FP32 copy of v is kept for the CUDA-core engine only
  h->kinetic_engine = engine;
  return BSL_OK;
}

int bsl_kinetic_engine(const bsl_handle* h) { return h ? h->kinetic_engine : -1; }

int bsl_potential_format(const bsl_handle* h) { return h ? h->vformat : -1; }

double bsl_gaunt_residual(const bsl_handle* h) { return h ? h->gaunt_residual : -1.0; }

int bsl_set_kinetic_slices(bsl_handle* h, int slices) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (slices < 1 || slices > 4) return fail(BSL_ERR_INPUT, "kinetic slices must be 1..4");
  h->kin_slices = slices;
  return BSL_OK;
}

int bsl_set_potential_format(bsl_handle* h, int format) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (format != BSL_VFMT_FP32 && format != BSL_VFMT_BF16 && format != BSL_VFMT_GAUNT)
    return fail(BSL_ERR_INPUT, "unknown block format");
  if (format == BSL_VFMT_GAUNT && !h->d.vc32)
    return fail(BSL_ERR_UNSUPPORTED, "no spherical-harmonic expansion of the blocks for this basis");
  if (format == BSL_VFMT_BF16 && h->t.nn != 15 && h->t.nn != 21)
    return fail(BSL_ERR_UNSUPPORTED, "BF16 potential blocks are built for blocks of 15 and 21 functions");
  cudaSetDevice(h->p.device);
  if (format == BSL_VFMT_BF16 && !h->d.vb16) {
    int rc = dev_vblocks_bf16(h);
    if (rc) return rc;
  }
  h->vformat = format;
  return BSL_OK;
}

int bsl_hv_apply_device(bsl_handle* h, const double* d_v, double* d_u, void* stream) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (!d_v || !d_u) return fail(BSL_ERR_INPUT, "null argument");
  cudaSetDevice(h->p.device);
  return dev_hv(h, d_v, d_u, (cudaStream_t)stream);
}

int bsl_hv_apply(bsl_handle* h, const double* vec, double* uec) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (!vec || !uec) return fail(BSL_ERR_INPUT, "null argument");
  cudaSetDevice(h->p.device);
  DeviceState& d = h->d;
  const size_t Df = (size_t)bsl_basis_size(h);
  int rc;
  if (!d.ref_vec && ((rc = dalloc(&d.ref_vec, Df, "staging")) || (rc = dalloc(&d.ref_out, Df, "staging")))) return rc;
  cudaStream_t s = d.stream;
  // the device Lanczos vectors serve as packed scratch here
  h->state_pairs = -1;
  BSL_CUDA(cudaMemcpyAsync(d.ref_vec, vec, Df * sizeof(double), cudaMemcpyHostToDevice, s));
  BSL_CUDA(cudaMemcpyAsync(d.ref_out, uec, Df * sizeof(double), cudaMemcpyHostToDevice, s));
  if ((rc = dev_gather_packed(h, d.ref_vec, d.vec, s))) return rc;
  if ((rc = dev_hv(h, d.vec, d.rvec, s))) return rc;
  // uec += H vec on the symmetry block; the reference adds S_n (...) = 0 elsewhere
  if ((rc = dev_scatter_full(h, d.rvec, d.ref_out, s))) return rc;
  BSL_CUDA(cudaMemcpyAsync(uec, d.ref_out, Df * sizeof(double), cudaMemcpyDeviceToHost, s));
  BSL_CUDA(cudaStreamSynchronize(s));
  int st[4] = {0, 0, 0, 0};
  BSL_CUDA(cudaMemcpy(st, d.status, sizeof(st), cudaMemcpyDeviceToHost));
  if (st[2] || st[3])
    return fail(BSL_ERR_CUDA, st[2] ? "potential-block stream: a bulk copy did not complete within its time limit"
                                    : "tensor-core kinetic: an MMA did not complete within its time limit");
  return BSL_OK;
}

long long bsl_vgrid_size(const bsl_handle* h) { return h ? h->t.npts * h->t.na * h->t.nb : -1; }

// potential grid in the reference order ((i*ny+j)*nz+k)*na*nb + a*nb + b
int bsl_copy_vgrid(const bsl_handle* h, double* v1, double* v2) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (!v1 || !v2) return fail(BSL_ERR_INPUT, "null argument");
  if (!h->d.v1) return fail(BSL_ERR_STATE, "the potential grid of a large problem is released after HvPrep");
  cudaSetDevice(h->p.device);
  const Tables& t = h->t;
  const size_t per = (size_t)t.na * t.nb, n = (size_t)t.npts * per;
  std::vector<double> a(n), b(n);
  BSL_CUDA(cudaMemcpy(a.data(), h->d.v1, n * sizeof(double), cudaMemcpyDeviceToHost));
  BSL_CUDA(cudaMemcpy(b.data(), h->d.v2, n * sizeof(double), cudaMemcpyDeviceToHost));
  for (int i = 0; i < t.nx; ++i)
    for (int j = 0; j < t.ny; ++j)
      for (int k = 0; k < t.nz; ++k) {
        const size_t pr = ((size_t)i * t.ny + j) * t.nz + k, pv = ((size_t)k * t.ny + j) * t.nx + i;
        std::memcpy(v1 + pr * per, a.data() + pv * per, per * sizeof(double));
        std::memcpy(v2 + pr * per, b.data() + pv * per, per * sizeof(double));
      }
  return BSL_OK;
}

long long bsl_vblock_size(const bsl_handle* h) { return h ? h->t.npts * h->t.nn * h->t.nn : -1; }

// potential blocks as full squares over the packed basis, reference point order
// [(i*ny+j)*nz+k][s][s']
int bsl_copy_vblocks(const bsl_handle* h, double* out) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (!out) return fail(BSL_ERR_INPUT, "null argument");
  cudaSetDevice(h->p.device);
  const Tables& t = h->t;
  const size_t N = (size_t)t.npts, nn = t.nn, ntri = nn * (nn + 1) / 2;
  std::vector<double> tri(ntri * N);
  BSL_CUDA(cudaMemcpy(tri.data(), h->d.vb64, tri.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int i = 0; i < t.nx; ++i)
    for (int j = 0; j < t.ny; ++j)
      for (int k = 0; k < t.nz; ++k) {
        const size_t pr = ((size_t)i * t.ny + j) * t.nz + k, pv = ((size_t)k * t.ny + j) * t.nx + i;
        size_t tt = 0;
        for (size_t s = 0; s < nn; ++s)
          for (size_t q = s; q < nn; ++q, ++tt) {
            const double x = tri[tt * N + pv];
            out[(pr * nn + s) * nn + q] = x;
            out[(pr * nn + q) * nn + s] = x;
          }
      }
  return BSL_OK;
}

int bsl_good_eigenvalues(int niter, const double* alpha, const double* beta, const double* beta2, double emin,
                         double emax, double* eval, double* err, int* ngood) {
  if (niter < 1 || !alpha || !beta || !beta2 || !eval || !err || !ngood) return fail(BSL_ERR_INPUT, "bad arguments");
  return cw_good_eigenvalues(niter, alpha, beta, beta2, emin, emax, eval, err, ngood);
}

int bsl_good_eigenvalues_unit(int niter, const double* alpha, const double* beta, const double* beta2, double emin,
                              double emax, double unit_roundoff, double* eval, double* err, int* ngood) {
  if (niter < 1 || !alpha || !beta || !beta2 || !eval || !err || !ngood || !(unit_roundoff > 0.0))
    return fail(BSL_ERR_INPUT, "bad arguments");
  return cw_good_eigenvalues(niter, alpha, beta, beta2, emin, emax, eval, err, ngood, unit_roundoff);
}

int bsl_good_eigenvalues_noise(int niter, const double* alpha, const double* beta, const double* beta2,
                               double emin, double emax, double unit_roundoff, double rel_noise, double* eval,
                               double* err, int* ngood) {
  if (niter < 1 || !alpha || !beta || !beta2 || !eval || !err || !ngood || !(unit_roundoff > 0.0) ||
      !(rel_noise >= 0.0))
    return fail(BSL_ERR_INPUT, "bad arguments");
  return cw_good_eigenvalues(niter, alpha, beta, beta2, emin, emax, eval, err, ngood, unit_roundoff, rel_noise);
}

int bsl_tm_eigenvectors(int niter, const double* alpha, const double* beta, const double* beta2,
                        const double* eval, int ngood, double* evtr) {
  if (niter < 1 || ngood < 0 || !alpha || !beta || !beta2 || !eval || !evtr)
    return fail(BSL_ERR_INPUT, "bad arguments");
  return cw_tm_eigenvectors(niter, alpha, beta, beta2, eval, ngood, evtr);
}

int bsl_last_run_ms_per_iter(const bsl_handle* h, double* ms) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (!ms) return fail(BSL_ERR_INPUT, "null argument");
  *ms = h->last_ms_per_iter;
  return BSL_OK;
}

}  // extern "C"
