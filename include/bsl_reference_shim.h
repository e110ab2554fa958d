/*
 * Reference-signature shim: the HvPrep/Hv function-pointer pair that the
 * reference registry hands to its Lanczos driver
 * (headLoop/InterfaceCode/interface.cpp:3-250, interface.h:40), implemented
 * on top of the C ABI in bsl.h.  Registering these under new HvCalculator
 * names lets the unmodified reference driver run the GB300 Hv path.
 *
 * This header must see the reference's lanczosStor/generalStor
 * (headLoop/InterfaceCode/interfaceContainers.h:6-14); it declares identical
 * structs under the same include guard when that header was not included.
 */
#ifndef BSL_REFERENCE_SHIM_H
#define BSL_REFERENCE_SHIM_H

#include <string>

#ifndef INTERFACECONTAINERS_H
#define INTERFACECONTAINERS_H
struct lanczosStor {
  int total_basis_size;
  std::string sim_descr;
  std::string sim_descr_short;
};
struct generalStor {
  double dummy;
};
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* Storage for one of the GB300 HvCalculators, the reference's NoQuad names
   with the suffix "_GB300":
     "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE_GB300"
     "linRotCartSph_NoQuad_ContGrid_Alavi_TIP4P_GB300"
     "linRotCartSph_NoQuad_Alavi_SPCE_GB300"
     "linRotCartSph_NoQuad_Alavi_TIP4P_GB300"
     "linRotCartSph_NoQuad_Coulomb_GB300"
     "linRotCartSph_NoQuad_IsoHarmOsc_GB300"
   Returns NULL for any other name.  The arithmetic is chosen by the
   environment variable BSL_PRECISION ("fp64", the default, or "mixed") and
   the device by BSL_DEVICE (default 0). */
generalStor* bsl_reference_storage(const std::string& calculator);

/* Replaces Hv_Prep_linRotCartSph_NoQuad
   (Hv-calculators/linRotor/cartSphBasis/HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:798-805):
   reads argv[2] (HvInputFile) and, for the oscillator and the Coulomb
   potential, argv[3]; sets
   total_basis_size, sim_descr and sim_descr_short.  Errors print to cerr and
   exit(1), as the reference does. */
void Hv_Prep_linRotCartSph_NoQuad_GB300(int argc, char** argv, generalStor* general_data, lanczosStor* lanczos_data);

/* Replaces Hv_linRotCartSph_NoQuad (same file :807-822): uec += H vec on host
   buffers of total_basis_size doubles in the reference layout. */
void Hv_linRotCartSph_NoQuad_GB300(int argc, char** argv, generalStor* general_data, lanczosStor* lanczos_data,
                                   double* vec, double* uec);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#endif
