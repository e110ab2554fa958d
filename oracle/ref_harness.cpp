// ORACLE — test infrastructure only.
// extern "C" harness around the UNMODIFIED reference Hv plugin, compiled
// together with the reference sources by oracle/Makefile into
// oracle/_ref/libref_hv.so.  It goes through the reference's own registry
// (HvInterfaceSetup, headLoop/InterfaceCode/interface.cpp:3-250) and calls
// the function pointers exactly as the reference driver does
// (headLoop/LanczosCode/lanczosEigenValuesVectors.cpp:100-103, :191-195).
#include <chrono>
#include <string>
#include <cstring>
#include "interface.h"

namespace {
generalStor* g_general = nullptr;
lanczosStor* g_lanczos = nullptr;
void (*g_prep)(int, char**, generalStor*, lanczosStor*) = nullptr;
void (*g_hv)(int, char**, generalStor*, lanczosStor*, double*, double*) = nullptr;
std::string g_args[4];
char* g_argv[5];
}

extern "C" {

// argv layout of the reference: argv[1] LanczosInputFile (unused by HvPrep),
// argv[2] HvInputFile, argv[3] potential input file (IsoHarmOsc/Coulomb only).
long ref_hv_setup(const char* calculator, const char* hv_input, const char* extra_input) {
  g_args[0] = "Lanczos";
  g_args[1] = "unused";
  g_args[2] = hv_input;
  g_args[3] = extra_input ? extra_input : "";
  for (int i = 0; i < 4; ++i) g_argv[i] = const_cast<char*>(g_args[i].c_str());
  g_argv[4] = nullptr;
  g_lanczos = new lanczosStor();
  HvInterfaceSetup(std::string(calculator), &g_general, &g_prep, &g_hv);
  (*g_prep)(4, g_argv, g_general, g_lanczos);
  return g_lanczos->total_basis_size;
}

long ref_basis_size() { return g_lanczos ? g_lanczos->total_basis_size : -1; }

// uec += H vec, reference layout ((n*nz+k)*ny+j)*nx+i
void ref_hv(const double* vec, double* uec) {
  (*g_hv)(4, g_argv, g_general, g_lanczos, const_cast<double*>(vec), uec);
}

// <n|V|n'>(x,y,z) blocks as stored by the reference: [(i*ny+j)*nz+k][n][n']
long ref_vblock_count() {
  interfaceStor* s = reinterpret_cast<interfaceStor*>(g_general);
  long nn = s->lmBasis->length;
  return (long)s->grids->nx * s->grids->ny * s->grids->nz * nn * nn;
}
void ref_vblocks(double* out) {
  interfaceStor* s = reinterpret_cast<interfaceStor*>(g_general);
  long cnt = ref_vblock_count();
  std::memcpy(out, s->potential->fullPotential, sizeof(double) * cnt);
}

// Seconds per Hv call over `reps` calls (uec zeroed before each call, as the
// reference driver does at lanczosEigenValuesVectors.cpp:191-192).
double ref_time_hv(int reps, const double* vec, double* uec) {
  long n = g_lanczos->total_basis_size;
  auto t0 = std::chrono::steady_clock::now();
  for (int r = 0; r < reps; ++r) {
    for (long i = 0; i < n; ++i) uec[i] = 0.0;
    (*g_hv)(4, g_argv, g_general, g_lanczos, const_cast<double*>(vec), uec);
  }
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count() / reps;
}

}  // extern "C"
