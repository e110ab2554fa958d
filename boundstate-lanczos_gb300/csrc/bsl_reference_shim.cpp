// Reference-signature shim over the C ABI (see include/bsl_reference_shim.h).
#include "bsl_reference_shim.h"

#include <cstdlib>
#include <cstring>
#include <iostream>

#include "bsl.h"

namespace {

struct GB300Storage {
  generalStor base;  // keeps the reference's opaque-pointer contract
  int potential;
  bsl_handle* handle;
};

[[noreturn]] void die(const char* what) {
  std::cerr << what << ": " << bsl_last_error() << std::endl;
  std::exit(1);
}

}  // namespace

generalStor* bsl_reference_storage(const std::string& calculator) {
  int pot = 0;
  const std::string suffix = "_GB300";
  if (calculator.size() <= suffix.size() ||
      calculator.compare(calculator.size() - suffix.size(), suffix.size(), suffix) != 0)
    return nullptr;
  if (bsl_calculator_potential(calculator.c_str(), &pot) != BSL_OK) return nullptr;
  GB300Storage* s = new GB300Storage();
  s->potential = pot;
  s->handle = nullptr;
  return reinterpret_cast<generalStor*>(s);
}

void Hv_Prep_linRotCartSph_NoQuad_GB300(int argc, char** argv, generalStor* general_data, lanczosStor* lanczos_data) {
  GB300Storage* s = reinterpret_cast<GB300Storage*>(general_data);
  if (argc < 3) die("HvPrep needs argv[2] (HvInputFile)");
  bsl_hv_params p;
  if (bsl_parse_hv_input(argv[2], &p) != BSL_OK) die("HvInputFile");
  p.potential = s->potential;
  if (p.potential == BSL_POT_ISOHARMOSC) {
    if (argc < 4) die("the oscillator needs argv[3]");
    if (bsl_parse_isoharmosc_input(argv[3], &p) != BSL_OK) die("IsoHarmOsc input");
  }
  if (p.potential == BSL_POT_COULOMB) {
    if (argc < 4) die("the Coulomb potential needs argv[3]");
    if (bsl_parse_coulomb_input(argv[3], &p) != BSL_OK) die("Coulomb input");
  }
  const char* prec = std::getenv("BSL_PRECISION");
  p.precision = (prec && std::strcmp(prec, "mixed") == 0) ? BSL_PREC_MIXED : BSL_PREC_FP64;
  const char* dev = std::getenv("BSL_DEVICE");
  p.device = dev ? std::atoi(dev) : 0;
  if (bsl_hv_prep(&p, &s->handle) != BSL_OK) die("HvPrep");
  lanczos_data->total_basis_size = (int)bsl_basis_size(s->handle);
  lanczos_data->sim_descr = p.simulation_title;
  lanczos_data->sim_descr_short = p.simulation_title;
}

void Hv_linRotCartSph_NoQuad_GB300(int argc, char** argv, generalStor* general_data, lanczosStor* lanczos_data,
                                   double* vec, double* uec) {
  (void)argc;
  (void)argv;
  (void)lanczos_data;
  GB300Storage* s = reinterpret_cast<GB300Storage*>(general_data);
  if (!s->handle) die("Hv called before HvPrep");
  if (bsl_hv_apply(s->handle, vec, uec) != BSL_OK) die("Hv");
}
