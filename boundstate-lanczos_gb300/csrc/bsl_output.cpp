// Result files in the reference's formats.
//
// Reference: headLoop/LanczosCode/lanczosEigenValuesVectors.cpp
//   boundstates.txt and states_zpe.txt   :263-290
//   lv (squared Tm eigenvector coefficients and cumulative norms)   :339-364
//   eigVecFile.txt (Ritz vectors in the reference layout)   :470-492
// Numbers are written as the reference's streams write them (scientific with
// 15 digits after the point, which is printf's %.15e); every file starts with
// the empty line the reference's "<< scientific << setprecision(15) << endl"
// produces.
#include <cstdio>
#include <string>

#include "bsl_internal.h"

namespace bsl {
namespace {

std::string join(const char* dir, const char* name) {
  std::string d = dir ? dir : ".";
  if (d.empty()) d = ".";
  if (d.back() != '/') d += '/';
  return d + name;
}

struct File {
  FILE* f = nullptr;
  explicit File(const std::string& path) : f(std::fopen(path.c_str(), "w")) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

int open_fail(const std::string& path) { return fail(BSL_ERR_INPUT, "cannot write " + path); }

}  // namespace
}  // namespace bsl

using namespace bsl;

extern "C" {

int bsl_write_boundstates(const char* dir, const char* sim_descr, int ngood, const double* eval, const double* err) {
  if (ngood < 0 || (ngood > 0 && (!eval || !err))) return fail(BSL_ERR_INPUT, "bad arguments");
  const char* descr = sim_descr ? sim_descr : "";
  const std::string p1 = join(dir, "boundstates.txt"), p2 = join(dir, "states_zpe.txt");
  File a(p1), b(p2);
  if (!a.f) return open_fail(p1);
  if (!b.f) return open_fail(p2);
  std::fprintf(a.f, "\nThe following are the eigenvalues and errors for the simulation %s\n", descr);
  std::fprintf(a.f, "Number of Eigenvalues: %d\n", ngood);
  std::fprintf(a.f, "State | Eigenvalue (kJ/mol) | Error (kJ/mol?)\n");
  std::fprintf(b.f, "\nThe following are the relative energies for the simulation %s\n", descr);
  std::fprintf(b.f, "Number of Eigenvalues: %d\n", ngood);
  std::fprintf(b.f, "Zero Point Energy = %.15e kJ/mol\n", ngood > 0 ? eval[0] : 0.0);
  std::fprintf(b.f, "State | Relative Energy (kJ/mol)\n");
  for (int i = 0; i < ngood; ++i) {
    std::fprintf(a.f, "%d %.15e %.15e\n", i, eval[i], err[i]);
    std::fprintf(b.f, "%d %.15e\n", i, eval[i] - eval[0]);
  }
  return (std::ferror(a.f) || std::ferror(b.f)) ? fail(BSL_ERR_INPUT, "write error in " + p1) : BSL_OK;
}

int bsl_write_tm_vectors(const char* dir, const char* sim_descr, int niter, int ngood, const double* evtr) {
  if (niter < 1 || ngood < 0 || (ngood > 0 && !evtr)) return fail(BSL_ERR_INPUT, "bad arguments");
  const std::string path = join(dir, "lv");
  File a(path);
  if (!a.f) return open_fail(path);
  std::fprintf(a.f, "\nThe following are the Coefficients squared of the Eigenvectors of Tm for the simulation %s\n",
               sim_descr ? sim_descr : "");
  std::fprintf(a.f, "Number of Eigenvectors: %d\n", ngood);
  std::fprintf(a.f, "Iteration | Coefficient Squared | Cumulative Norm \n");
  std::vector<double> cum(ngood, 0.0);
  for (int j = 1; j <= niter; ++j) {
    std::fprintf(a.f, "%d ", j);
    for (int n = 0; n < ngood; ++n) {
      const double c = evtr[(size_t)n * niter + (j - 1)];  // column-major [niter x ngood]
      const double c2 = c * c;
      cum[n] += c2;
      std::fprintf(a.f, "%.15e %.15e ", c2, cum[n]);
    }
    std::fprintf(a.f, "\n");
  }
  return std::ferror(a.f) ? fail(BSL_ERR_INPUT, "write error in " + path) : BSL_OK;
}

int bsl_write_ritz_vectors(const char* dir, const char* sim_descr, long long basis_size, int ngood,
                           const double* ritz) {
  if (basis_size < 1 || ngood < 0 || (ngood > 0 && !ritz)) return fail(BSL_ERR_INPUT, "bad arguments");
  const std::string path = join(dir, "eigVecFile.txt");
  File a(path);
  if (!a.f) return open_fail(path);
  std::fprintf(a.f, "\nThe following are the Ritz vectors of H for the simulation %s\n", sim_descr ? sim_descr : "");
  std::fprintf(a.f, "Number of Ritz vectors: %d\n", ngood);
  std::fprintf(a.f, "Basis Index | Vector 1 | Vector 2 ... \n");
  for (long long row = 0; row < basis_size; ++row) {
    std::fprintf(a.f, "%lld ", row);
    for (int n = 0; n < ngood; ++n) std::fprintf(a.f, "%.15e ", ritz[(size_t)n * basis_size + row]);
    std::fprintf(a.f, "\n");
  }
  return std::ferror(a.f) ? fail(BSL_ERR_INPUT, "write error in " + path) : BSL_OK;
}

}  // extern "C"
