// Test driver for the reference-signature shim (include/bsl_reference_shim.h).
// It makes the calls the reference's Lanczos driver makes
// (headLoop/LanczosCode/lanczosEigenValuesVectors.cpp:97-103: the registry
// lookup, HvPrep once; :191-195: uec zeroed, then Hv) and writes uec += H vec
// for a vector read from a file.
//
//   shim_driver CALCULATOR HV_INPUT EXTRA_INPUT|- VEC_IN UEC_OUT
//
// VEC_IN and UEC_OUT hold total_basis_size doubles in the reference layout.
// Prints "total_basis_size|sim_descr_short|sim_descr".
#include <cstdio>
#include <string>
#include <vector>

#include "bsl_reference_shim.h"

int main(int argc, char** argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: shim_driver CALCULATOR HV_INPUT EXTRA_INPUT|- VEC_IN UEC_OUT\n");
    return 2;
  }
  generalStor* general = bsl_reference_storage(argv[1]);
  if (!general) {
    std::fprintf(stderr, "HvCalculator %s not recognized\n", argv[1]);
    return 3;
  }
  // the reference's argv: [1] LanczosInputFile (unused by HvPrep), [2] HvInputFile, [3] potential file
  std::string args[4] = {"Lanczos", "unused", argv[2], std::string(argv[3]) == "-" ? "" : argv[3]};
  char* av[5] = {&args[0][0], &args[1][0], &args[2][0], &args[3][0], nullptr};
  lanczosStor lanczos;
  Hv_Prep_linRotCartSph_NoQuad_GB300(4, av, general, &lanczos);
  const size_t n = (size_t)lanczos.total_basis_size;
  std::vector<double> vec(n), uec(n, 0.0);
  FILE* f = std::fopen(argv[4], "rb");
  if (!f || std::fread(vec.data(), sizeof(double), n, f) != n) {
    std::fprintf(stderr, "cannot read %zu doubles from %s\n", n, argv[4]);
    return 4;
  }
  std::fclose(f);
  Hv_linRotCartSph_NoQuad_GB300(4, av, general, &lanczos, vec.data(), uec.data());
  f = std::fopen(argv[5], "wb");
  if (!f || std::fwrite(uec.data(), sizeof(double), n, f) != n) {
    std::fprintf(stderr, "cannot write %s\n", argv[5]);
    return 5;
  }
  std::fclose(f);
  std::printf("%d|%s|%s\n", lanczos.total_basis_size, lanczos.sim_descr_short.c_str(), lanczos.sim_descr.c_str());
  return 0;
}
