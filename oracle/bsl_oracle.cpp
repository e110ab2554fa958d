// ORACLE — test infrastructure only.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg may load this library, and only as the checker
// or the timed CPU baseline.  It is never part of the product path.
//
// CPU restatement (C++, FP64, OpenMP where the reference uses OpenMP) of the
// reference's linRotCartSph_NoQuad Hv path, written from its behaviour:
//
//   inputs     HvInputFile tokens       HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:246-348
//              cage .xyz                potentialCalc/Alavi/SPCE/SPCE_AH2_EngRoutines.cpp:5-108
//              IsoHarmOsc input          potentialCalc/IsotropicHarmonicOscillatorPotential/IsoHarmOsc_Routines.cpp:34-79
//   tables     genIndices_lm             HvCalc/linRotCartSphHvRoutines.cpp:24-68
//              gauleg                    HvCalc/linRotCartSphHvRoutines.cpp:219-255
//              normAssocLegendrePoly     HvCalc/linRotCartSphHvRoutines.cpp:293-403
//              tesseralTrigTerm          HvCalc/linRotCartSphHvRoutines.cpp:405-434
//              gaussChebyshev            HvCalc/linRotCartSphHvRoutines.cpp:450-463
//              cartKinGrid               HvCalc/linRotCartSphHvRoutines.cpp:484-517
//              rotKinEng                 HvCalc/linRotCartSphHvRoutines.cpp:522-538
//              QuadraturePrep            HvCalc/linRotCartSphHvRoutines.cpp:1480-1532
//              TesseralPrep              HvCalc/linRotCartSphHvRoutines.cpp:1534-1735
//   potential  Alavi_SiteSite_Eng_contGrid potentialCalc/Alavi/AlaviGeneric/Alavi_ContGrid_H2_Routines.cpp:6-147
//              Q_SPCE_Eng / LJ_SPCE_Eng_Fast potentialCalc/Alavi/SPCE/SPCE_AH2_EngRoutines.cpp:110-178
//              CoulombEng / LJEngFast    potentialCalc/CommonRoutines/energyRoutines.cpp:5-54
//              rotMat3D                  librarySources/matVecClasses/rotmat.cpp:6-32
//              IsoHarmOscEng             potentialCalc/IsotropicHarmonicOscillatorPotential/IsoHarmOsc_Routines.cpp:6-31
//   V blocks   calc_Vlmlpmp_NoQuad_ContGrid HvCalc/NoQuadOnTheFly/ContinuousAngularGrid/linRotCartSphHvContGridRoutines.cpp:7-152
//              calc_Vlmlpmp_NoQuad       HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:7-227
//              calcSym                   HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:530-573
//   Hv         Tv_5D_oneCompositeIndex   HvCalc/linRotCartSphHvRoutines.cpp:1807-1969
//              Vv_5D_oneCompositeIndex_NoQuad HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:675-734
//              Hv_5D_oneCompositeIndex_NoQuad / Hv_linRotCartSph_NoQuad  same file :736-822
//   Lanczos    loop 1                    headLoop/LanczosCode/lanczosEigenValuesVectors.cpp:170-242
//              lancbis                   headLoop/LanczosCode/supportingRoutines/lancbis.cpp:5-105 (tail in cw_tail.cpp)
//              lanczosvectors + loop 2   headLoop/LanczosCode/lanczosEigenValuesVectors.cpp:329-469, 509-561
//
// Arithmetic is evaluated in the same order as the reference so that, with
// the same inputs, results agree to the last bit or nearly so (the reference
// is compiled with -O3 and OpenMP; this file with -ffp-contract=off).
// Reference paths here are relative to Hv-calculators/linRotor/cartSphBasis/
// unless they start with headLoop/.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <cfloat>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include <chrono>
#include <omp.h>

extern "C" {
void bisec_(double*, double*, double*, int*, double*, int*, double*, int*, double*, double*, int*);
void isoev_(double*, int*, int*);
void inverr_(double*, double*, double*, double*, double*, int*, double*, int*, double*, int*);
void trivec_(double*, double*, double*, double*, double*, int*, double*, int*, double*, double*);
}

namespace {

// headLoop/InterfaceCode/lanczosUnits.h:5-14
const double kPI = 3.141592653589793;
const double kK = 138.9354846111096;
const double kHBAR = 0.0635077857002;
const double kNmPerAng = 0.1;
// potentialCalc/Alavi/AlaviGeneric/Alavi_Parameters.h:5-10
const double kQ_H2_H = 0.4932, kQ_H2_CM = -0.9864, kH2_H1_Z = 0.03707;
// potentialCalc/Alavi/SPCE/SPCE_AH2_EngRoutines.h:17-38
const double kQ_H_SPCE = 0.4238, kQ_O_SPCE = -0.8476;
const double kO_SPCE[3] = {0.0, 0.0, 0.006461408220};
const double kH1_SPCE[3] = {-8.164965810E-2, 0.0, -0.05127361870};
const double kH2_SPCE[3] = {8.164965810E-2, 0.0, -0.05127361870};
const double kA_LJ = 1.364e-06, kB_LJ = 1.533e-3;

std::string g_err;

struct HvInput {
  int nx, ny, nz, l_max, theta_points, phi_points, pnx, pny, pnz;
  double x_max, y_max, z_max, px_max, py_max, pz_max;
  double total_mass, rot_const, ceiling;
  std::string geometry, title, quad_study, sym;
};

bool read_hv_input(const char* path, HvInput* h) {
  std::ifstream f(path);
  if (!f.is_open()) { g_err = std::string("cannot open HvInputFile ") + path; return false; }
  std::string line, junk;
  std::getline(f, line);
  std::getline(f, line);
  f >> junk >> h->nx >> junk >> h->x_max >> junk >> h->ny >> junk >> h->y_max >> junk >> h->nz >> junk >>
      h->z_max >> junk >> h->l_max >> junk >> h->theta_points >> junk >> h->phi_points >> junk >> h->pnx >>
      junk >> h->px_max >> junk >> h->pny >> junk >> h->py_max >> junk >> h->pnz >> junk >> h->pz_max >>
      junk >> h->total_mass >> junk >> h->rot_const >> junk >> h->geometry >> junk >> h->title >> junk >>
      h->ceiling >> junk >> h->quad_study >> junk >> h->sym;
  if (!f) { g_err = "truncated HvInputFile"; return false; }
  return true;
}

struct Cage {
  std::vector<double> pos;   // [atom][3] nm
  std::vector<double> q;     // charge
  std::vector<int> is_o;     // LJ site
  std::vector<double> cm, ea;  // per molecule: centre of mass (Angstrom), ZY'Z'' Euler angles (rad)
  double q_h2_h = kQ_H2_H, q_h2_cm = kQ_H2_CM;  // Alavi H2 charges (each H, centre of mass)
};

// getSPCEatoms: rotate the SPC/E body frame with the ZY'Z'' Euler angles and
// translate by the centre of mass (Angstrom -> nm).
bool read_cage(const std::string& path, Cage* c) {
  std::ifstream f(path);
  if (!f.is_open()) { g_err = "cannot open geometry " + path; return false; }
  int nmol;
  std::string line;
  f >> nmol;
  std::getline(f, line);
  std::getline(f, line);
  for (int i = 0; i < nmol; ++i) {
    std::string name;
    double cm[3], ea[3];
    f >> name >> cm[0] >> ea[0] >> cm[1] >> ea[1] >> cm[2] >> ea[2];
    if (!f) { g_err = "truncated geometry file"; return false; }
    for (int r = 0; r < 3; ++r) { c->cm.push_back(cm[r]); c->ea.push_back(ea[r]); }
    double cp = cos(ea[0]), sp = sin(ea[0]), ct = cos(ea[1]), st = sin(ea[1]), cx = cos(ea[2]), sx = sin(ea[2]);
    double R[3][3] = {{(cp * ct * cx) - (sp * sx), (-1 * cp * ct * sx) - (sp * cx), cp * st},
                      {(sp * ct * cx) + (cp * sx), (-1 * sp * ct * sx) + (cp * cx), sp * st},
                      {-1 * st * cx, st * sx, ct}};
    const double* local[3] = {kO_SPCE, kH1_SPCE, kH2_SPCE};
    const double qs[3] = {kQ_O_SPCE, kQ_H_SPCE, kQ_H_SPCE};
    for (int a = 0; a < 3; ++a) {
      for (int r = 0; r < 3; ++r) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += R[r][k] * local[a][k];
        c->pos.push_back(s + kNmPerAng * cm[r]);
      }
      c->q.push_back(qs[a]);
      c->is_o.push_back(a == 0);
    }
  }
  return true;
}

inline double coulomb_sum(const double* p, double qsite, const Cage& c) {
  double e = 0;
  size_t na = c.q.size();
  for (size_t i = 0; i < na; ++i) {
    double d0 = c.pos[3 * i] - p[0], d1 = c.pos[3 * i + 1] - p[1], d2 = c.pos[3 * i + 2] - p[2];
    double s = 0.;
    s += d0 * d0;
    s += d1 * d1;
    s += d2 * d2;
    e += kK * qsite * c.q[i] / sqrt(s);
  }
  return e;
}

inline double lj_sum(const double* p, const Cage& c) {
  double e = 0;
  size_t na = c.q.size();
  for (size_t i = 0; i < na; ++i) {
    if (!c.is_o[i]) continue;
    double d0 = c.pos[3 * i] - p[0], d1 = c.pos[3 * i + 1] - p[1], d2 = c.pos[3 * i + 2] - p[2];
    double s = 0.;
    s += d0 * d0;
    s += d1 * d1;
    s += d2 * d2;
    double r = sqrt(s);
    e += (kA_LJ / pow(r, 12)) - (kB_LJ / pow(r, 6));
  }
  return e;
}

double factorial(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f *= double(i);
  return f;
}

struct Model {
  HvInput in;
  int potential_kind = 0;  // 0 Alavi SPC/E continuous grid, 1 IsoHarmOsc, 2 synthetic blocks,
                           // 3 Alavi SPC/E point grid, 4 Coulomb
  double iso_factor = 0, iso_ceil = 0;
  int nn = 0;              // (l_max+1)^2
  std::vector<int> ql, qm; // n -> l, m
  std::vector<double> xgrid, ygrid, zgrid, Tx, Ty, Tz, rot, sym;
  std::vector<double> gl_x, gl_w, gc_x, gc_w, theta, phi, phi2;
  // tesseral factors: L[n][a], S1[m+lmax][b] (phi), S2 (2pi - phi)
  std::vector<double> L, S1, S2;
  std::vector<double> V1, V2;  // [(i*ny+j)*nz+k][a][b]
  std::vector<double> Vb;      // [(i*ny+j)*nz+k][n][n']
  Cage cage;
};

void cart_kin_grid(double xmax, int n, double mass, std::vector<double>* T, std::vector<double>* g) {
  double dx = xmax / double(n - 1);
  T->assign((size_t)n * n, 0.0);
  g->assign(n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double t = (kHBAR * kHBAR) / (2.0 * mass * dx * dx) * pow(-1.0, (i + 1) - (j + 1));
      if (i == j) t *= (kPI * kPI) / 3.0;
      else t *= 2.0 / double(((i + 1) - (j + 1)) * ((i + 1) - (j + 1)));
      (*T)[(size_t)i * n + j] = t;
    }
  for (int i = 0; i < n; ++i) (*g)[i] = double(i) * dx - xmax / 2.0;
}

void gauleg(double x1, double x2, double* x, double* w, int n) {
  int m = (n + 1) / 2;
  double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
  for (int i = 1; i <= m; i++) {
    double z = cos(M_PI * ((double)i - 0.25) / ((double)n + 0.5)), z1, pp, p1, p2, p3;
    do {
      p1 = 1.0;
      p2 = 0.0;
      for (int j = 1; j <= n; j++) {
        p3 = p2;
        p2 = p1;
        p1 = ((2.0 * (double)j - 1.0) * z * p2 - ((double)j - 1.0) * p3) / (double)j;
      }
      pp = (double)n * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    } while (fabs(z - z1) > DBL_EPSILON);
    x[i - 1] = xm - xl * z;
    x[n - i] = xm + xl * z;
    w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp);
    w[n - i] = w[i - 1];
  }
}

// normalised associated Legendre values for every n at cos(theta) = x
void norm_assoc_legendre(const Model& M, double x, double* out) {
  int lmax = M.in.l_max;
  std::vector<double> P((size_t)(lmax + 1) * (lmax + 1), 0.0);
  auto at = [&](int l, int m) -> double& { return P[(size_t)l * (lmax + 1) + m]; };
  double rf = sqrt(1.0 - x * x);
  at(0, 0) = 1.0;
  for (int l = 1; l <= lmax; l++) at(l, l) = (2.0 * double(l) - 1.0) * at(l - 1, l - 1) * rf;
  for (int m = 0; m <= lmax - 1; m++)
    for (int l = m; l <= lmax - 1; l++) {
      double ld = l, md = m;
      double prev = ((l - 1) < m) ? 0.0 : at(l - 1, m);
      at(l + 1, m) = (((2.0 * ld + 1.0) * x * at(l, m)) - ((ld + md) * prev)) / (ld - md + 1.0);
    }
  for (int l = 0; l <= lmax; l++) {
    double phase = 1.0;
    for (int m = 0; m <= l; m++) {
      double nf = factorial(l - m) * (2.0 * double(l) + 1.0) / (2.0 * factorial(l + m));
      at(l, m) *= phase * sqrt(nf);
      phase *= -1.0;
    }
  }
  for (int n = 0; n < M.nn; ++n) out[n] = at(M.ql[n], std::abs(M.qm[n]));
}

double trig_term(int m, double phi) {
  double s = 1.0 / sqrt(kPI);
  if (m == 0) return s / sqrt(2.0);
  if (m > 0) return s * cos(double(m) * phi);
  return s * sin(double(-m) * phi);
}

void build_tables(Model& M) {
  HvInput& in = M.in;
  cart_kin_grid(in.x_max, in.nx, in.total_mass, &M.Tx, &M.xgrid);
  cart_kin_grid(in.y_max, in.ny, in.total_mass, &M.Ty, &M.ygrid);
  cart_kin_grid(in.z_max, in.nz, in.total_mass, &M.Tz, &M.zgrid);
  int lmax = in.l_max;
  M.nn = (lmax + 1) * (lmax + 1);
  for (int m = -lmax; m <= lmax; m++)
    for (int l = std::abs(m); l <= lmax; l++) { M.ql.push_back(l); M.qm.push_back(m); }
  M.rot.resize(M.nn);
  for (int n = 0; n < M.nn; ++n) { double l = M.ql[n]; M.rot[n] = in.rot_const * l * (l + 1.0); }
  M.sym.resize(M.nn);
  for (int n = 0; n < M.nn; ++n) {
    int l = M.ql[n];
    if (in.sym == "All") M.sym[n] = 1.0;
    else if (in.sym == "Even") M.sym[n] = (l % 2 == 0) ? 1.0 : 0.0;
    else M.sym[n] = (l % 2 == 1) ? 1.0 : 0.0;
  }
  int na = in.theta_points, nb = in.phi_points;
  M.gl_x.resize(na); M.gl_w.resize(na);
  gauleg(-1.0, 1.0, M.gl_x.data(), M.gl_w.data(), na);
  M.gc_x.resize(nb); M.gc_w.resize(nb);
  for (int i = 0; i < nb; i++) {
    M.gc_x[i] = cos(kPI * (2.0 * double(i + 1) - 1.0) / (2.0 * double(nb)));
    M.gc_w[i] = kPI / double(nb);
  }
  M.theta.resize(na); M.phi.resize(nb); M.phi2.resize(nb);
  for (int a = 0; a < na; a++) M.theta[a] = acos(M.gl_x[a]);
  for (int b = 0; b < nb; b++) { M.phi[b] = acos(M.gc_x[b]); M.phi2[b] = 2 * kPI - acos(M.gc_x[b]); }
  M.L.assign((size_t)M.nn * na, 0.0);
  std::vector<double> tmp(M.nn);
  for (int a = 0; a < na; a++) {
    norm_assoc_legendre(M, M.gl_x[a], tmp.data());
    for (int n = 0; n < M.nn; ++n) M.L[(size_t)n * na + a] = tmp[n];
  }
  int nm = 2 * lmax + 1;
  M.S1.assign((size_t)nm * nb, 0.0);
  M.S2.assign((size_t)nm * nb, 0.0);
  for (int b = 0; b < nb; b++)
    for (int m = -lmax; m <= lmax; m++) {
      M.S1[(size_t)(m + lmax) * nb + b] = trig_term(m, acos(M.gc_x[b]));
      M.S2[(size_t)(m + lmax) * nb + b] = trig_term(m, 2.0 * kPI - acos(M.gc_x[b]));
    }
}

void build_potential_alavi(Model& M, int nthreads) {
  HvInput& in = M.in;
  int ni = in.nx, nj = in.ny, nk = in.nz, na = in.theta_points, nb = in.phi_points;
  size_t np = (size_t)ni * nj * nk;
  M.V1.assign(np * na * nb, 0.0);
  M.V2.assign(np * na * nb, 0.0);
  std::vector<double> cmpot(np);
  std::vector<double> h1((size_t)na * nb * 3), h2((size_t)na * nb * 3);
  for (int a = 0; a < na; a++)
    for (int b = 0; b < nb; b++) {
      size_t o = ((size_t)a * nb + b) * 3;
      h1[o] = kH2_H1_Z * sin(M.theta[a]) * M.gc_x[b];
      h1[o + 1] = kH2_H1_Z * sin(M.theta[a]) * sin(M.phi[b]);
      h1[o + 2] = kH2_H1_Z * M.gl_x[a];
      h2[o] = h1[o];
      h2[o + 1] = -1.0 * h1[o + 1];
      h2[o + 2] = h1[o + 2];
    }
  double ceil_v = in.ceiling;
#pragma omp parallel for schedule(guided) num_threads(nthreads)
  for (long p = 0; p < (long)np; ++p) {
    int i = p / ((size_t)nj * nk), j = (p / nk) % nj, k = p % nk;
    double g[3] = {M.xgrid[i], M.ygrid[j], M.zgrid[k]};
    double c = coulomb_sum(g, M.cage.q_h2_cm, M.cage);
    c += lj_sum(g, M.cage);
    cmpot[p] = c;
  }
#pragma omp parallel for schedule(guided) collapse(3) num_threads(nthreads)
  for (long p = 0; p < (long)np; ++p)
    for (int a = 0; a < na; a++)
      for (int b = 0; b < nb; b++) {
        int i = p / ((size_t)nj * nk), j = (p / nk) % nj, k = p % nk;
        double g[3] = {M.xgrid[i], M.ygrid[j], M.zgrid[k]};
        for (int half = 0; half < 2; ++half) {
          const double* h = (half ? h2.data() : h1.data()) + ((size_t)a * nb + b) * 3;
          double p1[3] = {g[0] + h[0], g[1] + h[1], g[2] + h[2]};
          double p2[3] = {g[0] - h[0], g[1] - h[1], g[2] - h[2]};
          double v = coulomb_sum(p1, M.cage.q_h2_h, M.cage);
          v += coulomb_sum(p2, M.cage.q_h2_h, M.cage);
          v += cmpot[p];
          if (v >= ceil_v) v = ceil_v;
          (half ? M.V2 : M.V1)[((size_t)p * na + a) * nb + b] = v;
        }
      }
}

// calc_Vlmlpmp_NoQuad (HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:126-177)
// with Alavi_H2_Eng_Point (potentialCalc/Alavi/AlaviGeneric/Alavi_H2_Routines.cpp:136-195):
// the centre-of-mass and H-atom site energies are tabulated on the potential
// universe (preCalcPotential_Alavi / Alavi_SiteSite_Eng, :197-310; generateGrid,
// CommonRoutines/gridFcns.cpp:6-56) and read at the universe point nearest to
// each site (AlaviMapH2GridToHGrid, :5-52: round half away from zero, clamped).
void build_potential_point_alavi(Model& M, int nthreads) {
  HvInput& in = M.in;
  int ni = in.nx, nj = in.ny, nk = in.nz, na = in.theta_points, nb = in.phi_points;
  size_t np = (size_t)ni * nj * nk;
  const int un[3] = {in.pnx, in.pny, in.pnz};
  const double gm[3] = {in.px_max, in.py_max, in.pz_max};
  double du[3];
  for (int q = 0; q < 3; ++q) du[q] = gm[q] / (double(un[q] - 1));
  size_t usize = (size_t)un[0] * un[1] * un[2];
  std::vector<double> cmpot(usize), hpot(usize);
#pragma omp parallel for schedule(guided) num_threads(nthreads)
  for (long u = 0; u < (long)usize; ++u) {
    const int ix = u % un[0], iy = (u / un[0]) % un[1], iz = u / ((size_t)un[0] * un[1]);
    double g[3] = {(double(ix) * du[0]) - (gm[0] / 2.0), (double(iy) * du[1]) - (gm[1] / 2.0),
                   (double(iz) * du[2]) - (gm[2] / 2.0)};
    double c = 0.0;
    c += coulomb_sum(g, kQ_H2_CM, M.cage);
    c += lj_sum(g, M.cage);
    cmpot[u] = c;
    double h = 0.0;
    h += coulomb_sum(g, kQ_H2_H, M.cage);
    hpot[u] = h;
  }
  auto nearest = [&](double numerator, int q) {
    int i = (int)round(numerator / du[q]);
    if (i <= 0) i = 0;
    else if (i >= un[q]) i = un[q] - 1;
    return i;
  };
  auto at = [&](const int* idx) { return (size_t)idx[0] + (size_t)un[0] * (idx[1] + (size_t)un[1] * idx[2]); };
  M.V1.assign(np * na * nb, 0.0);
  M.V2.assign(np * na * nb, 0.0);
  double ceil_v = in.ceiling;
#pragma omp parallel for schedule(guided) num_threads(nthreads)
  for (long p = 0; p < (long)np; ++p) {
    int i = p / ((size_t)nj * nk), j = (p / nk) % nj, k = p % nk;
    const double c[3] = {M.xgrid[i], M.ygrid[j], M.zgrid[k]};
    for (int a = 0; a < na; a++)
      for (int b = 0; b < nb; b++)
        for (int half = 0; half < 2; ++half) {
          const double th = M.theta[a], ph = half ? M.phi2[b] : M.phi[b];
          const double e[3] = {sin(th) * cos(ph), sin(th) * sin(ph), cos(th)};
          int icm[3], ih1[3], ih2[3];
          for (int q = 0; q < 3; ++q) {
            const double grid_min = (-0.5) * gm[q];
            icm[q] = nearest(c[q] - grid_min, q);
            ih1[q] = nearest(c[q] + e[q] * kH2_H1_Z - grid_min, q);
            ih2[q] = nearest(c[q] + e[q] * (-kH2_H1_Z) - grid_min, q);
          }
          double v = 0.0;
          v += cmpot[at(icm)];
          v += hpot[at(ih1)];
          v += hpot[at(ih2)];
          if (v >= ceil_v) v = ceil_v;
          (half ? M.V2 : M.V1)[((size_t)p * na + a) * nb + b] = v;
        }
  }
}

// calc_Vlmlpmp_NoQuad with CoulombPotential
// (potentialCalc/CoulombPotential/Coulomb_Routines.cpp:6-33, CoulombEng,
// CommonRoutines/energyRoutines.cpp:5-26): V = K q_c q_m / |r| for a charge at
// the origin, |V| > |c| -> c, then the HvInputFile ceiling.
void build_potential_coulomb(Model& M, double qc, double qm, double c_ceil) {
  HvInput& in = M.in;
  int ni = in.nx, nj = in.ny, nk = in.nz, na = in.theta_points, nb = in.phi_points;
  size_t np = (size_t)ni * nj * nk;
  M.V1.assign(np * na * nb, 0.0);
  M.V2.assign(np * na * nb, 0.0);
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < nj; ++j)
      for (int k = 0; k < nk; ++k) {
        double x = M.xgrid[i], y = M.ygrid[j], z = M.zgrid[k];
        double d2 = 0.;
        d2 += x * x;
        d2 += y * y;
        d2 += z * z;
        double v = kK * qc * qm / sqrt(d2);
        if (fabs(v) > fabs(c_ceil)) v = c_ceil;
        if (v >= in.ceiling) v = in.ceiling;
        size_t p = ((size_t)i * nj + j) * nk + k;
        for (int a = 0; a < na; ++a)
          for (int b = 0; b < nb; ++b) {
            M.V1[(p * na + a) * nb + b] = v;
            M.V2[(p * na + a) * nb + b] = v;
          }
      }
}

// calc_Vlmlpmp_NoQuad with IsoHarmOscEng: V = 0.5 m w^2 |r|^2, clipped first by
// the oscillator's own ceiling (|V| > |c| -> c) and then by the HvInputFile
// ceiling (V >= c -> c).
void build_potential_iso(Model& M) {
  HvInput& in = M.in;
  int ni = in.nx, nj = in.ny, nk = in.nz, na = in.theta_points, nb = in.phi_points;
  size_t np = (size_t)ni * nj * nk;
  M.V1.assign(np * na * nb, 0.0);
  M.V2.assign(np * na * nb, 0.0);
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < nj; ++j)
      for (int k = 0; k < nk; ++k) {
        double x = M.xgrid[i], y = M.ygrid[j], z = M.zgrid[k];
        double d2 = 0.;
        d2 += x * x;
        d2 += y * y;
        d2 += z * z;
        double v = M.iso_factor * d2;
        if (fabs(v) > fabs(M.iso_ceil)) v = M.iso_ceil;
        if (v >= in.ceiling) v = in.ceiling;
        size_t p = ((size_t)i * nj + j) * nk + k;
        for (int a = 0; a < na; ++a)
          for (int b = 0; b < nb; ++b) {
            M.V1[(p * na + a) * nb + b] = v;
            M.V2[(p * na + a) * nb + b] = v;
          }
      }
}

void build_vblocks(Model& M, int nthreads) {
  HvInput& in = M.in;
  int ni = in.nx, nj = in.ny, nk = in.nz, na = in.theta_points, nb = in.phi_points, nn = M.nn;
  int lmax = in.l_max;
  size_t np = (size_t)ni * nj * nk;
  std::vector<double> hf((size_t)nn * nn * na * nb), hf2((size_t)nn * nn * na * nb);
  for (int n = 0; n < nn; n++)
    for (int q = 0; q < nn; q++)
      for (int a = 0; a < na; a++)
        for (int b = 0; b < nb; b++) {
          size_t o = (((size_t)n * nn + q) * na + a) * nb + b;
          int m = M.qm[n], mp = M.qm[q];
          hf[o] = M.gl_w[a] * M.gc_w[b] * M.L[(size_t)n * na + a] * M.S1[(size_t)(m + lmax) * nb + b] *
                  M.L[(size_t)q * na + a] * M.S1[(size_t)(mp + lmax) * nb + b];
          hf2[o] = M.gl_w[a] * M.gc_w[b] * M.L[(size_t)n * na + a] * M.S2[(size_t)(m + lmax) * nb + b] *
                   M.L[(size_t)q * na + a] * M.S2[(size_t)(mp + lmax) * nb + b];
        }
  M.Vb.assign(np * nn * nn, 0.0);
#pragma omp parallel for schedule(guided) collapse(3) num_threads(nthreads)
  for (long p = 0; p < (long)np; ++p)
    for (int n = 0; n < nn; n++)
      for (int q = 0; q < nn; q++) {
        double s = 0.0;
        const double* h1 = &hf[((size_t)n * nn + q) * na * nb];
        const double* h2 = &hf2[((size_t)n * nn + q) * na * nb];
        const double* v1 = &M.V1[(size_t)p * na * nb];
        const double* v2 = &M.V2[(size_t)p * na * nb];
        for (int ab = 0; ab < na * nb; ++ab) s += h1[ab] * v1[ab] + h2[ab] * v2[ab];
        M.Vb[((size_t)p * nn + n) * nn + q] = s;
      }
}

// uec += S (T + V) vec in the reference layout ((n*nz+k)*ny+j)*nx+i.
void hv(const Model& M, const double* v, double* uec, int nthreads) {
  const HvInput& in = M.in;
  const int ni = in.nx, nj = in.ny, nk = in.nz, nn = M.nn;
  const size_t N = (size_t)ni * nj * nk, D = N * nn;
  std::vector<double> t(D);
  // Kinetic: each axis is a serial dense line contraction (Mv_5D, reference
  // loops with the OpenMP pragmas commented out), summed as
  // rot + (Tz + (Ty + Tx)).
  for (int n = 0; n < nn; n++)
    for (int k = 0; k < nk; k++)
      for (int j = 0; j < nj; j++)
        for (int i = 0; i < ni; i++) {
          const size_t base = ((size_t)n * nk + k) * nj;
          double tx = 0.0, ty = 0.0, tz = 0.0;
          for (int q = 0; q < ni; q++) tx += M.Tx[(size_t)i * ni + q] * v[(base + j) * ni + q];
          for (int q = 0; q < nj; q++) ty += M.Ty[(size_t)j * nj + q] * v[(base + q) * ni + i];
          for (int q = 0; q < nk; q++) tz += M.Tz[(size_t)k * nk + q] * v[((((size_t)n * nk + q) * nj) + j) * ni + i];
          const size_t p = (base + j) * ni + i;
          t[p] = M.rot[n] * v[p] + (tz + (ty + tx));
        }
  // Potential: per grid point an nn x nn block times the local coefficients.
#pragma omp parallel for schedule(guided) collapse(3) num_threads(nthreads)
  for (int i = 0; i < ni; i++)
    for (int j = 0; j < nj; j++)
      for (int k = 0; k < nk; k++) {
        const size_t pb = ((size_t)i * nj + j) * nk + k;
        const size_t pv = ((size_t)k * nj + j) * ni + i;
        for (int n = 0; n < nn; n++) {
          double s = 0.0;
          const double* blk = &M.Vb[(pb * nn + n) * nn];
          for (int q = 0; q < nn; q++) s += blk[q] * v[(size_t)q * N + pv];
          const size_t o = (size_t)n * N + pv;
          double h = t[o] + s;
          h *= M.sym[n];
          uec[o] += h;
        }
      }
}

// ---------------------------------------------------------------------------
// Hellmann-Feynman derivatives, FP64 (no counterpart in the reference: the
// derivative of the restated potential above).  The continuous-grid blocks are
// the quadrature of build_vblocks,
//   <s|V|s'>(p) = sum_{a,b} w_a w_b [Y_s Y_s' V1 + Y2_s Y2_s' V2](p, a, b),
// so for any fixed psi (a unit-independent Rayleigh quotient, H(theta) in a
// basis that does not depend on theta)
//   d<psi|H|psi>/dtheta / <psi|psi> = sum_p sum_{a,b,half} w_a w_b f_half(p,a,b)^2 dV_half/dtheta / <psi|psi>,
//   f_half(p, a, b) = sum_s psi_s(p) L_s(a) S^half_{m_s}(b),
// over the functions of the symmetry block, and zero where the ceiling clips V
// (V >= ceiling stored as the ceiling).  V (Alavi_ContGrid_H2_Routines.cpp:6-147,
// SPCE_AH2_EngRoutines.cpp:110-178, energyRoutines.cpp:5-54) is
//   K [q_cm sum_w q_w / |g - r_w| + q_h sum_w q_w (1/|g + h - r_w| + 1/|g - h - r_w|)]
//   + sum_O (A / |g - r_O|^12 - B / |g - r_O|^6),
// h = d u(theta_a, phi_b) (y component negated on the 2 pi - phi half).
// Outputs per level n: dq[n][w], dr[n][w][3] (per nm), da[n][{q_h, q_cm}].
void hf_gradient(const Model& M, int nlev, const double* psi, double* dq, double* dr, double* da, int nthreads) {
  const HvInput& in = M.in;
  const int ni = in.nx, nj = in.ny, nk = in.nz, na = in.theta_points, nb = in.phi_points, nn = M.nn;
  const int lmax = in.l_max;
  const size_t N = (size_t)ni * nj * nk, D = N * nn;
  const Cage& c = M.cage;
  const int nat = (int)c.q.size();
  std::vector<int> block;
  for (int s = 0; s < nn; ++s)
    if (M.sym[s] != 0.0) block.push_back(s);
  const int nbk = (int)block.size();
  // Y[(a nb + b) 2 + half][k] for the block's functions k, with sqrt(w_a w_b)
  std::vector<double> Y((size_t)na * nb * 2 * nbk), hoff((size_t)na * nb * 3);
  for (int a = 0; a < na; ++a)
    for (int b = 0; b < nb; ++b) {
      const double w = sqrt(M.gl_w[a] * M.gc_w[b]);
      for (int half = 0; half < 2; ++half)
        for (int k = 0; k < nbk; ++k) {
          const int sfun = block[k];
          const std::vector<double>& S = half ? M.S2 : M.S1;
          Y[(((size_t)a * nb + b) * 2 + half) * nbk + k] =
              w * M.L[(size_t)sfun * na + a] * S[(size_t)(M.qm[sfun] + lmax) * nb + b];
        }
      hoff[((size_t)a * nb + b) * 3] = kH2_H1_Z * sin(M.theta[a]) * M.gc_x[b];
      hoff[((size_t)a * nb + b) * 3 + 1] = kH2_H1_Z * sin(M.theta[a]) * sin(M.phi[b]);
      hoff[((size_t)a * nb + b) * 3 + 2] = kH2_H1_Z * M.gl_x[a];
    }
  std::vector<double> norm(nlev, 0.0);
  for (int n = 0; n < nlev; ++n)
    for (int k = 0; k < nbk; ++k)
      for (size_t p = 0; p < N; ++p) {
        const double x = psi[(size_t)n * D + (size_t)block[k] * N + p];
        norm[n] += x * x;
      }
  const size_t nsite = (size_t)nlev * nat * 4, nacc = nsite + (size_t)nlev * 2;
  std::vector<double> total(nacc, 0.0);
  const double ceil_v = in.ceiling;
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<double> acc(nacc, 0.0), ps(nbk * (size_t)nlev), rho(nlev), sv(nat * 4);
#pragma omp for schedule(dynamic, 16)
    for (long p = 0; p < (long)N; ++p) {
      // vector index p = ((k nj) + j) ni + i; potential index (i nj + j) nk + k
      const int i = (int)(p % ni), j = (int)((p / ni) % nj), kz = (int)(p / ((long)ni * nj));
      const size_t pb = ((size_t)i * nj + j) * nk + kz;
      const double g[3] = {M.xgrid[i], M.ygrid[j], M.zgrid[kz]};
      for (int n = 0; n < nlev; ++n)
        for (int k = 0; k < nbk; ++k) ps[(size_t)n * nbk + k] = psi[(size_t)n * D + (size_t)block[k] * N + p];
      // centre-of-mass terms do not depend on the node: per site 1/rc, dc/rc^3 and the LJ force
      std::vector<double> cm_inv(nat), cm_f(nat * 3);
      for (int w = 0; w < nat; ++w) {
        const double d0 = g[0] - c.pos[3 * w], d1 = g[1] - c.pos[3 * w + 1], d2 = g[2] - c.pos[3 * w + 2];
        const double r2 = d0 * d0 + d1 * d1 + d2 * d2, r = sqrt(r2), inv = 1.0 / r, inv3 = inv * inv * inv;
        cm_inv[w] = inv;
        double f = kK * c.q[w] * c.q_h2_cm * inv3;
        if (c.is_o[w]) f += 12.0 * kA_LJ / pow(r, 14) - 6.0 * kB_LJ / pow(r, 8);
        cm_f[3 * w] = f * d0;
        cm_f[3 * w + 1] = f * d1;
        cm_f[3 * w + 2] = f * d2;
      }
      for (int a = 0; a < na; ++a)
        for (int b = 0; b < nb; ++b)
          for (int half = 0; half < 2; ++half) {
            const double v = (half ? M.V2 : M.V1)[(pb * na + a) * nb + b];
            if (!(v < ceil_v)) continue;
            const double* y = &Y[(((size_t)a * nb + b) * 2 + half) * nbk];
            double rsum = 0.0;
            for (int n = 0; n < nlev; ++n) {
              double f = 0.0;
              for (int k = 0; k < nbk; ++k) f += ps[(size_t)n * nbk + k] * y[k];
              rho[n] = f * f;
              rsum += rho[n];
            }
            if (rsum == 0.0) continue;
            const double* h = &hoff[((size_t)a * nb + b) * 3];
            const double hx = h[0], hy = half ? -h[1] : h[1], hz = h[2];
            double sh = 0.0, sc = 0.0;  // d V / d q_h, d V / d q_cm
            for (int w = 0; w < nat; ++w) {
              const double bx = g[0] - c.pos[3 * w], by = g[1] - c.pos[3 * w + 1], bz = g[2] - c.pos[3 * w + 2];
              const double px = bx + hx, py = by + hy, pz = bz + hz, mx = bx - hx, my = by - hy, mz = bz - hz;
              const double ip = 1.0 / sqrt(px * px + py * py + pz * pz), im = 1.0 / sqrt(mx * mx + my * my + mz * mz);
              const double ip3 = ip * ip * ip, im3 = im * im * im;
              const double kq = kK * c.q[w] * c.q_h2_h;
              sv[4 * w] = kK * (c.q_h2_h * (ip + im) + c.q_h2_cm * cm_inv[w]);
              sv[4 * w + 1] = kq * (px * ip3 + mx * im3) + cm_f[3 * w];
              sv[4 * w + 2] = kq * (py * ip3 + my * im3) + cm_f[3 * w + 1];
              sv[4 * w + 3] = kq * (pz * ip3 + mz * im3) + cm_f[3 * w + 2];
              sh += kK * c.q[w] * (ip + im);
              sc += kK * c.q[w] * cm_inv[w];
            }
            for (int n = 0; n < nlev; ++n) {
              const double rn = rho[n];
              double* o = &acc[(size_t)n * nat * 4];
              for (int e = 0; e < nat * 4; ++e) o[e] += rn * sv[e];
              acc[nsite + 2 * n] += rn * sh;
              acc[nsite + 2 * n + 1] += rn * sc;
            }
          }
    }
#pragma omp critical
    for (size_t e = 0; e < nacc; ++e) total[e] += acc[e];
  }
  for (int n = 0; n < nlev; ++n) {
    for (int w = 0; w < nat; ++w) {
      const double* t = &total[((size_t)n * nat + w) * 4];
      dq[(size_t)n * nat + w] = t[0] / norm[n];
      for (int k = 0; k < 3; ++k) dr[((size_t)n * nat + w) * 3 + k] = t[1 + k] / norm[n];
    }
    da[2 * n] = total[nsite + 2 * n] / norm[n];
    da[2 * n + 1] = total[nsite + 2 * n + 1] / norm[n];
  }
}

// SPC/E site s of a molecule with Euler angles e (getSPCEatoms' rotation,
// SPCE_AH2_EngRoutines.cpp:5-108, rotmat.cpp:6-32), relative to the centre of
// mass, for a real or complex angle type.
template <typename T>
void spce_site_rel(const T e[3], int s, T out[3]) {
  using std::cos;
  using std::sin;
  const T cp = cos(e[0]), sp = sin(e[0]), ct = cos(e[1]), st = sin(e[1]), cx = cos(e[2]), sx = sin(e[2]);
  const T R[3][3] = {{(cp * ct * cx) - (sp * sx), (-1.0 * cp * ct * sx) - (sp * cx), cp * st},
                     {(sp * ct * cx) + (cp * sx), (-1.0 * sp * ct * sx) + (cp * cx), sp * st},
                     {-1.0 * st * cx, st * sx, ct}};
  const double* local[3] = {kO_SPCE, kH1_SPCE, kH2_SPCE};
  for (int r = 0; r < 3; ++r) out[r] = R[r][0] * local[s][0] + R[r][1] * local[s][1] + R[r][2] * local[s][2];
}

// chain rule from site positions to (centre of mass in Angstrom, Euler angles):
// d site / d cm_k = 0.1 e_k; d site / d e_k by complex-step differentiation of
// the rotation (exact to rounding: Im f(x + i h) / h with h = 1e-30)
void rigid_body_chain(const Cage& c, int nlev, const double* dr, double* dcm, double* dea) {
  const int nmol = (int)c.cm.size() / 3, nat = (int)c.q.size();
  for (int n = 0; n < nlev; ++n)
    for (int m = 0; m < nmol; ++m) {
      for (int k = 0; k < 3; ++k) {
        double gc = 0.0;
        for (int s = 0; s < 3; ++s) gc += kNmPerAng * dr[((size_t)n * nat + 3 * m + s) * 3 + k];
        dcm[((size_t)n * nmol + m) * 3 + k] = gc;
        double ge = 0.0;
        for (int s = 0; s < 3; ++s) {
          std::complex<double> e[3] = {c.ea[3 * m], c.ea[3 * m + 1], c.ea[3 * m + 2]}, x[3];
          e[k] += std::complex<double>(0.0, 1e-30);
          spce_site_rel(e, s, x);
          for (int r = 0; r < 3; ++r) ge += dr[((size_t)n * nat + 3 * m + s) * 3 + r] * (x[r].imag() / 1e-30);
        }
        dea[((size_t)n * nmol + m) * 3 + k] = ge;
      }
    }
}

}  // namespace

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

// calculator: "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE",
// "linRotCartSph_NoQuad_Alavi_SPCE", "linRotCartSph_NoQuad_Coulomb" or
// "linRotCartSph_NoQuad_IsoHarmOsc".  extra_input: the IsoHarmOsc or Coulomb
// parameter file (argv[3]).
void* orc_create(const char* calculator, const char* hv_input, const char* extra_input, int nthreads) {
  Model* M = new Model();
  if (!read_hv_input(hv_input, &M->in)) { delete M; return nullptr; }
  std::string calc(calculator);
  build_tables(*M);
  if (calc == "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE") {
    if (!read_cage(M->in.geometry, &M->cage)) { delete M; return nullptr; }
    M->potential_kind = 0;
    build_potential_alavi(*M, nthreads);
  } else if (calc == "linRotCartSph_NoQuad_Alavi_SPCE") {
    if (!read_cage(M->in.geometry, &M->cage)) { delete M; return nullptr; }
    M->potential_kind = 3;
    build_potential_point_alavi(*M, nthreads);
  } else if (calc == "linRotCartSph_NoQuad_Coulomb") {
    std::ifstream f(extra_input ? extra_input : "");
    if (!f.is_open()) { g_err = "cannot open Coulomb input"; delete M; return nullptr; }
    std::string line, junk;
    double qc, qm, c_ceil;
    std::getline(f, line);
    std::getline(f, line);
    f >> junk >> qc >> junk >> qm >> junk >> c_ceil;
    M->potential_kind = 4;
    build_potential_coulomb(*M, qc, qm, c_ceil);
  } else if (calc == "linRotCartSph_NoQuad_IsoHarmOsc") {
    std::ifstream f(extra_input ? extra_input : "");
    if (!f.is_open()) { g_err = "cannot open IsoHarmOsc input"; delete M; return nullptr; }
    std::string line, junk;
    double mass, freq, ceil_v;
    std::getline(f, line);
    std::getline(f, line);
    f >> junk >> mass >> junk >> freq >> junk >> ceil_v;
    M->iso_factor = 0.5 * mass * freq * freq;
    M->iso_ceil = ceil_v;
    M->potential_kind = 1;
    build_potential_iso(*M);
  } else {
    g_err = "unknown calculator " + calc;
    delete M;
    return nullptr;
  }
  build_vblocks(*M, nthreads);
  return M;
}

// Timing-only model at production sizes: the Hv cost does not depend on the
// potential values, so the blocks are filled with a cheap deterministic
// symmetric pattern instead of running the potential and block assembly.
void* orc_create_synthetic(int nx, int ny, int nz, int l_max, double x_max, double mass, double rot_const,
                           const char* sym) {
  Model* M = new Model();
  HvInput& in = M->in;
  in.nx = nx; in.ny = ny; in.nz = nz; in.l_max = l_max;
  in.x_max = in.y_max = in.z_max = x_max;
  in.theta_points = 2; in.phi_points = 2;
  in.total_mass = mass; in.rot_const = rot_const; in.sym = sym; in.ceiling = 18.0;
  build_tables(*M);
  M->potential_kind = 2;
  size_t np = (size_t)nx * ny * nz, nn = M->nn;
  M->Vb.assign(np * nn * nn, 0.0);
#pragma omp parallel for
  for (long p = 0; p < (long)np; ++p)
    for (size_t n = 0; n < nn; ++n)
      for (size_t q = 0; q < nn; ++q)
        M->Vb[((size_t)p * nn + n) * nn + q] = 1e-3 * double((p + n + q) % 17) - 8e-3;
  return M;
}

void orc_destroy(void* h) { delete static_cast<Model*>(h); }

long orc_basis_size(void* h) {
  Model* M = static_cast<Model*>(h);
  return (long)M->in.nx * M->in.ny * M->in.nz * M->nn;
}
int orc_nn(void* h) { return static_cast<Model*>(h)->nn; }

void orc_hv(void* h, const double* vec, double* uec, int nthreads) {
  hv(*static_cast<Model*>(h), vec, uec, nthreads);
}

// Potential grid halves V(x,y,z,theta_a,phi_b) and V(..,2pi-phi_b), point index
// (i*ny+j)*nz+k slowest.
long orc_vgrid_size(void* h) { Model* M = static_cast<Model*>(h); return (long)M->V1.size(); }
void orc_vgrid(void* h, double* v1, double* v2) {
  Model* M = static_cast<Model*>(h);
  std::memcpy(v1, M->V1.data(), M->V1.size() * sizeof(double));
  std::memcpy(v2, M->V2.data(), M->V2.size() * sizeof(double));
}
long orc_vblock_size(void* h) { return (long)static_cast<Model*>(h)->Vb.size(); }
void orc_vblocks(void* h, double* out) {
  Model* M = static_cast<Model*>(h);
  std::memcpy(out, M->Vb.data(), M->Vb.size() * sizeof(double));
}
// Tables for unit tests: kinetic matrix of one axis, GL/GC nodes, tesseral L.
void orc_tables(void* h, double* Tx, double* gl_x, double* gl_w, double* gc_x, double* L, double* S1, double* S2) {
  Model* M = static_cast<Model*>(h);
  std::memcpy(Tx, M->Tx.data(), M->Tx.size() * sizeof(double));
  std::memcpy(gl_x, M->gl_x.data(), M->gl_x.size() * sizeof(double));
  std::memcpy(gl_w, M->gl_w.data(), M->gl_w.size() * sizeof(double));
  std::memcpy(gc_x, M->gc_x.data(), M->gc_x.size() * sizeof(double));
  std::memcpy(L, M->L.data(), M->L.size() * sizeof(double));
  std::memcpy(S1, M->S1.data(), M->S1.size() * sizeof(double));
  std::memcpy(S2, M->S2.data(), M->S2.size() * sizeof(double));
}

// Lanczos loop 1 of the reference driver.  v0 == NULL selects the uniform
// start vector 1/sqrt(D).  alpha[niter], beta[niter+1], beta2[niter+1] (index
// 0 unused, zero).  Returns seconds spent.
double orc_lanczos(void* h, int niter, const double* v0, double* alpha, double* beta, double* beta2, int nthreads) {
  Model* M = static_cast<Model*>(h);
  const long D = orc_basis_size(h);
  std::vector<double> r(D, 0.0), v(D), u(D, 0.0);
  for (long i = 0; i < D; ++i) v[i] = v0 ? v0[i] : 1. / sqrt((double)D);
  beta[0] = 0.0;
  beta2[0] = 0.0;
  auto t0 = std::chrono::steady_clock::now();
  for (int j = 1; j <= niter; ++j) {
    for (long i = 0; i < D; ++i) u[i] = 0.;
    hv(*M, v.data(), u.data(), nthreads);
    for (long i = 0; i < D; ++i) r[i] += u[i];
    double a = 0.;
    for (long i = 0; i < D; ++i) a += v[i] * r[i];
    alpha[j - 1] = a;
    for (long i = 0; i < D; ++i) r[i] -= (a * v[i]);
    double b2 = 0.;
    for (long i = 0; i < D; ++i) b2 += r[i] * r[i];
    beta2[j] = b2;
    double b = sqrt(b2);
    beta[j] = b;
    for (long i = 0; i < D; ++i) r[i] = (1. / b) * r[i];
    for (long i = 0; i < D; ++i) v[i] = (-b) * v[i];
    for (long i = 0; i < D; ++i) { u[i] = v[i]; v[i] = r[i]; r[i] = u[i]; }
  }
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// lancbis (lancbis.cpp:5-105): good eigenvalues in (emin, emax] with
// inverse-iteration error estimates; returns ngood.  eval/err need niter slots.
int orc_lancbis(int niter, const double* alpha, const double* beta, const double* beta2, double emin, double emax,
                double* eval, double* err) {
  std::vector<double> la(alpha, alpha + niter), lb(beta, beta + niter + 1), lb2(beta2, beta2 + niter + 1);
  std::vector<double> ql(niter, 0.0), wrk2(2 * niter, 0.0);
  std::vector<int> mp2(niter, 0);
  int ndis = 0, nit = niter;
  bisec_(la.data(), lb.data(), lb2.data(), &nit, ql.data(), mp2.data(), wrk2.data(), &nit, &emin, &emax, &ndis);
  std::vector<double> vs(ql.begin(), ql.begin() + ndis);
  std::vector<int> mp(mp2.begin(), mp2.begin() + ndis);
  if (ndis > 1) isoev_(vs.data(), mp.data(), &ndis);
  std::vector<double> w1(niter, 0.0), w2(niter + 1, 0.0), w3(niter, 0.0), e(niter > ndis ? niter : ndis, 0.0);
  if (ndis > 0) inverr_(la.data(), lb.data(), w1.data(), w2.data(), w3.data(), &nit, vs.data(), mp.data(), e.data(), &ndis);
  int ii = 0;
  for (int i = 0; i < ndis; ++i)
    if (mp[i] != 0) { eval[ii] = vs[i]; err[ii] = e[i]; ++ii; }
  return ii;
}

// lanczosvectors (lanczosEigenValuesVectors.cpp:509-561): Tm eigenvectors,
// column-major evtr[niter x ngood].
void orc_trivec(int niter, const double* alpha, const double* beta, const double* beta2, const double* eval, int ngood,
                double* evtr) {
  std::vector<double> la(alpha, alpha + niter), lb(niter + 1), lb2(niter + 1), le(eval, eval + ngood);
  lb[0] = 0.;
  lb2[0] = 0.;
  for (int j = 1; j <= niter; ++j) { lb[j] = beta[j]; lb2[j] = beta2[j]; }
  std::vector<double> w1(niter, 0.0), w2(niter, 0.0), mamin(ngood, 0.0);
  std::vector<double> ev((size_t)niter * ngood, 0.0);
  int nit = niter, ng = ngood;
  trivec_(la.data(), lb.data(), lb2.data(), w1.data(), w2.data(), &nit, le.data(), &ng, ev.data(), mamin.data());
  std::memcpy(evtr, ev.data(), ev.size() * sizeof(double));
}

// Lanczos loop 2 with Ritz accumulation (lanczosEigenValuesVectors.cpp:371-469):
// ritz[n*D + row] = sum_j evtr[j,n] v_j[row], skipping terms once the
// cumulative squared coefficient reaches 1 - 1e-16.
void orc_ritz(void* h, int niter, const double* evtr, int ngood, double* ritz, int nthreads) {
  Model* M = static_cast<Model*>(h);
  const long D = orc_basis_size(h);
  std::vector<double> r(D, 0.0), v(D), u(D, 0.0), cum(ngood, 0.0);
  for (long i = 0; i < D; ++i) v[i] = 1. / sqrt((double)D);
  for (long i = 0; i < D * (long)ngood; ++i) ritz[i] = 0.;
  for (int j = 1; j <= niter; ++j) {
    for (int n = 0; n < ngood; ++n) {
      double c = evtr[(size_t)n * niter + (j - 1)];
      cum[n] += pow(c, 2.);
      for (long row = 0; row < D; ++row) {
        double coeff = c * v[row];
        if (cum[n] < (1. - 1.e-16)) ritz[row + D * n] += coeff;
      }
    }
    for (long i = 0; i < D; ++i) u[i] = 0.;
    hv(*M, v.data(), u.data(), nthreads);
    for (long i = 0; i < D; ++i) r[i] += u[i];
    double a = 0.;
    for (long i = 0; i < D; ++i) a += v[i] * r[i];
    for (long i = 0; i < D; ++i) r[i] -= (a * v[i]);
    double b2 = 0.;
    for (long i = 0; i < D; ++i) b2 += r[i] * r[i];
    double b = sqrt(b2);
    for (long i = 0; i < D; ++i) r[i] = (1. / b) * r[i];
    for (long i = 0; i < D; ++i) v[i] = (-b) * v[i];
    for (long i = 0; i < D; ++i) { u[i] = v[i]; v[i] = r[i]; r[i] = u[i]; }
  }
}


// Hellmann-Feynman derivatives of the levels of eigenvectors psi[n][D]
// (reference layout, any normalisation) for the continuous-grid Alavi SPC/E
// model: dq_site[n][w], dr_site[n][w][3] (per nm), dq_alavi[n][{H, centre}].
int orc_hf_gradient(void* h, int nlev, const double* psi, double* dq_site, double* dr_site, double* dq_alavi,
                    int nthreads) {
  Model* M = static_cast<Model*>(h);
  if (M->potential_kind != 0) { g_err = "derivatives need the continuous-grid Alavi SPC/E potential"; return 1; }
  hf_gradient(*M, nlev, psi, dq_site, dr_site, dq_alavi, nthreads);
  return 0;
}

// dr_site[n][w][3] -> d_cm[n][m][3] (per Angstrom), d_euler[n][m][3] (per rad)
int orc_rigid_body_gradient(void* h, int nlev, const double* dr_site, double* d_cm, double* d_euler) {
  Model* M = static_cast<Model*>(h);
  if (M->cage.cm.empty()) { g_err = "no cage"; return 1; }
  rigid_body_chain(M->cage, nlev, dr_site, d_cm, d_euler);
  return 0;
}

// Replace the site charges (q_site[w], NULL: unchanged) and the Alavi H2
// charges (q_alavi[2], NULL: unchanged), then rebuild the potential and the
// blocks (continuous-grid Alavi SPC/E only).
int orc_set_charges(void* h, const double* q_site, const double* q_alavi, int nthreads) {
  Model* M = static_cast<Model*>(h);
  if (M->potential_kind != 0) { g_err = "charges need the continuous-grid Alavi SPC/E potential"; return 1; }
  if (q_site)
    for (size_t w = 0; w < M->cage.q.size(); ++w) M->cage.q[w] = q_site[w];
  if (q_alavi) {
    M->cage.q_h2_h = q_alavi[0];
    M->cage.q_h2_cm = q_alavi[1];
  }
  build_potential_alavi(*M, nthreads);
  build_vblocks(*M, nthreads);
  return 0;
}

}  // extern "C"
