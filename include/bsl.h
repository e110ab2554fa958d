/*
 * boundstate-lanczos GB300 — C ABI of the NoQuad Hv path.
 *
 * One process drives one GPU.  Every entry point returns a status code
 * (BSL_OK on success) and never exits the process; the text of the last error
 * of the calling thread is available from bsl_last_error().  No entry point
 * takes or returns a C++ or torch type: plain pointers, sizes and a CUDA
 * stream handle passed as void*.
 *
 * Layouts
 *   reference layout  double[nx*ny*nz*(l_max+1)^2], index ((n*nz+k)*ny+j)*nx+i,
 *                     n = composite (l,m) index with m outer (-l_max..l_max) and
 *                     l inner (|m|..l_max); the layout of the reference's vec/uec
 *                     (Hv-calculators/linRotor/cartSphBasis/HvCalc/NoQuadOnTheFly/
 *                     linRotCartSphHvFullVPrepRoutines.cpp:807-822).
 *   packed layout     double[nx*ny*nz*nn_sym] on the device, index (s*nz+k)*ny+j)*nx+i
 *                     where s runs over the (l,m) pairs kept by the rotational
 *                     symmetry (All: all, Even: even l, Odd: odd l) in reference
 *                     order.  The reference multiplies every other component by
 *                     zero (calcSym, same file :530-573), so the packed operator is
 *                     the reference operator restricted to its non-zero block.
 */
#ifndef BSL_H
#define BSL_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The library is built with hidden symbol visibility; the entry points
   declared here are its exported interface. */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* status codes */
#define BSL_OK 0
#define BSL_ERR_INPUT 1       /* bad or missing input file / parameter */
#define BSL_ERR_CUDA 2        /* CUDA runtime error (message has the CUDA text) */
#define BSL_ERR_STATE 3       /* call out of order, null handle */
#define BSL_ERR_BREAKDOWN 4   /* Lanczos breakdown: beta == 0 or non-finite alpha/beta */
#define BSL_ERR_UNSUPPORTED 5 /* option not available in this build */
#define BSL_ERR_NOMEM 6       /* device or host allocation failed */

/* rotationalSymmetry(All/Even/Odd) */
#define BSL_SYM_ALL 0
#define BSL_SYM_EVEN 1
#define BSL_SYM_ODD 2

/* potential selected by the HvCalculator string */
#define BSL_POT_ALAVI_SPCE 0  /* linRotCartSph_NoQuad_ContGrid_Alavi_SPCE */
#define BSL_POT_ISOHARMOSC 1  /* linRotCartSph_NoQuad_IsoHarmOsc */
#define BSL_POT_ALAVI_TIP4P 2 /* linRotCartSph_NoQuad_ContGrid_Alavi_TIP4P */
/* point-grid calculators: the H2 site energies are tabulated on the potential
   universe grid (pointPotential_* fields) and read at the grid point nearest
   to each site (Alavi_H2_Routines.cpp:136-195) */
#define BSL_POT_POINT_ALAVI_SPCE 3  /* linRotCartSph_NoQuad_Alavi_SPCE */
#define BSL_POT_POINT_ALAVI_TIP4P 4 /* linRotCartSph_NoQuad_Alavi_TIP4P */
#define BSL_POT_COULOMB 5           /* linRotCartSph_NoQuad_Coulomb: a point charge at the
                                       origin and one on the H2 centre of mass */

/* arithmetic of the Hv application */
#define BSL_PREC_FP64 0  /* every step in FP64 */
#define BSL_PREC_MIXED 1 /* FP32 potential values, an FP32 / tensor-core kinetic
                            exact to ~2^-36 (or FP32 head and tail coefficients
                            on the CUDA cores), double-float rotor diagonal and
                            double-float (~48-bit) Lanczos recurrence; grids of
                            at most 64 points per axis (the kinetic engines) */

/* engine of the FP32 kinetic contractions in BSL_PREC_MIXED */
#define BSL_KIN_SIMT 0   /* FP32 head/tail coefficients on the CUDA cores; grids of
                            at most 64 points per axis: one thread owns a 4 x 4
                            tile of a plane's output and a CTA of at most 256
                            threads a whole plane, with the next plane held in
                            16 registers per thread */
#define BSL_KIN_TENSOR 1 /* fixed-point FP16 slices on the tensor cores
                            (tcgen05.mma), exact FP32 accumulation in tensor
                            memory; grids of at most 64 points per axis with
                            equal x and y axes */

/* Lanczos start vector */
#define BSL_START_UNIFORM 0 /* 1/sqrt(D) over the reference layout, as the
                               reference driver (lanczosEigenValuesVectors.cpp:177-181) */
#define BSL_START_NORMAL 1  /* N(0,1) from a seeded generator, normalised */

typedef struct bsl_hv_params {
  /* HvInputFile, in file order (linRotCartSphHvFullVPrepRoutines.cpp:256-320) */
  int nx;
  double x_max; /* full box width in nm; grid spans [-x_max/2, x_max/2] */
  int ny;
  double y_max;
  int nz;
  double z_max;
  int l_max;
  int theta_points; /* Gauss-Legendre nodes in cos(theta) */
  int phi_points;   /* half of the uniform phi nodes: 2*phi_points in total */
  int pnx;
  double px_max;
  int pny;
  double py_max;
  int pnz;
  double pz_max;
  double total_mass;          /* amu */
  double rotational_constant; /* kJ/mol */
  char geometry_filename[1024];
  char simulation_title[256];
  double ceiling_potential; /* kJ/mol */
  int quadrature_study;     /* parsed, not used (the reference ignores it for NoQuad) */
  int symmetry;             /* BSL_SYM_* */
  /* potential */
  int potential;       /* BSL_POT_* */
  double iso_mass;     /* IsoHarmOsc input file (argv[3]) */
  double iso_frequency;
  double iso_ceiling;
  /* execution */
  int precision; /* BSL_PREC_* */
  int device;    /* CUDA device ordinal */
  int keep_potential_grid; /* keep V(x,y,z,theta,phi) on the device after HvPrep
                              (needed by bsl_hf_gradient; otherwise released when
                              larger than 2^26 values) */
  double coulomb_centre_charge; /* Coulomb input file (argv[3]), e */
  double coulomb_mol_charge;
  double coulomb_ceiling;       /* |V| > |ceiling| -> ceiling, kJ/mol */
} bsl_hv_params;

typedef struct bsl_handle bsl_handle;

/* Text of the last error on the calling thread ("" if none). */
const char* bsl_last_error(void);

/* Parse an HvInputFile (two comment lines, then 22 "key= value" pairs whose keys
   are ignored; replaces HvPrep_Internal_NoQuad's reader, linRotCartSphHvFullVPrepRoutines.cpp:246-348,
   including its size checks).  Leaves potential/precision/device at defaults
   (Alavi SPC/E, FP64, device 0). */
int bsl_parse_hv_input(const char* path, bsl_hv_params* out);

/* Parse the IsoHarmOsc potential file (IsoHarmOsc_Routines.cpp:41-58). */
int bsl_parse_isoharmosc_input(const char* path, bsl_hv_params* inout);

/* Parse the Coulomb potential file read as argv[3]: two comment lines, then
   centreCharge, molCharge and the potential ceiling as key/value pairs
   (potentialCalc/CoulombPotential/Coulomb_Routines.cpp:36-85). */
int bsl_parse_coulomb_input(const char* path, bsl_hv_params* inout);

/* Map an HvCalculator string (headLoop/InterfaceCode/interface.cpp:3-250) to
   BSL_POT_*; unknown names give BSL_ERR_INPUT. */
int bsl_calculator_potential(const char* calculator, int* potential);

/* HvPrep: build grids, tables and the potential on the device.  Replaces
   Hv_Prep_linRotCartSph_NoQuad (linRotCartSphHvFullVPrepRoutines.cpp:798-805). */
int bsl_hv_prep(const bsl_hv_params* params, bsl_handle** out);

/* HvPrep with the cage given as arrays instead of the geometry file (for
   parameter derivatives): nmol rigid SPC/E waters, centres of mass in
   Angstrom cm_ang[3 nmol] and ZYZ Euler angles euler[3 nmol] in the file's
   order (SPCE_AH2_EngRoutines.cpp:5-108); q_site[3 nmol] (O, H1, H2 per
   molecule) replaces the SPC/E charges when not NULL, q_alavi[2] (each H,
   centre of mass) the Alavi H2 charges when not NULL.  Alavi SPC/E or TIP4P
   (params->potential; TIP4P: q_site[4 nmol], O, H1, H2, M per molecule). */
int bsl_hv_prep_cage(const bsl_hv_params* params, int nmol, const double* cm_ang, const double* euler,
                     const double* q_site, const double* q_alavi, bsl_handle** out);

void bsl_destroy(bsl_handle* h);

/* Sizes: reference layout (the reference's total_basis_size) and packed layout. */
long long bsl_basis_size(const bsl_handle* h);
long long bsl_packed_size(const bsl_handle* h);
int bsl_packed_nn(const bsl_handle* h);

/* Switch the arithmetic of later Hv applications (BSL_PREC_*). */
int bsl_set_precision(bsl_handle* h, int precision);

/* Select the kinetic engine of BSL_PREC_MIXED (BSL_KIN_*).  bsl_hv_prep selects
   BSL_KIN_TENSOR where the grid allows it (at most 64 points per axis, equal x
   and y axes), else BSL_KIN_SIMT; BSL_ERR_UNSUPPORTED when the grid does not
   allow BSL_KIN_TENSOR.  The tensor engine slices the double-float Lanczos
   vector exactly into FP16 fixed-point parts and accumulates exactly: its H v
   deviates from the FP64 path by ~3e-9 relative, the CUDA-core engine's by
   ~2e-7. */
int bsl_set_kinetic_engine(bsl_handle* h, int engine);
int bsl_kinetic_engine(const bsl_handle* h);

/* Precision variants of BSL_PREC_MIXED, for precision studies; no counterpart
   in the reference (FP64 throughout).  The defaults are the exact tensor-core
   kinetic (4 slices) and FP32 blocks.

   Slices of v and of T kept by the tensor-core kinetic (1..4): v and T are cut
   into 9-bit fixed-point slices and the slice products of classes k + l <
   slices are accumulated; 4 (the default) is exact to ~2^-36 of each plane's
   largest value, 2 keeps 3 products of 18-bit halves (a split 3-term product),
   1 is a plain 9-bit product.  T loses its slices beyond `slices` too, a fixed
   perturbation of the operator that shifts the levels. */
int bsl_set_kinetic_slices(bsl_handle* h, int slices);

/* Storage of the potential blocks streamed by BSL_PREC_MIXED. */
#define BSL_VFMT_FP32 0  /* FP32 upper triangles, nn (nn + 1) / 2 values per point */
#define BSL_VFMT_BF16 1  /* BF16 scaled per grid point by max |block element| (FP32
                            scale): half the bytes, unit roundoff 2^-9; blocks of
                            15 and 21 functions */
#define BSL_VFMT_GAUNT 2 /* FP32 coefficients c_k(p) of real spherical harmonics of
                            degree <= 2 l_max: every product of two basis functions
                            is a finite sum of them, so the quadrature blocks are
                            exactly <s|V|s'>(p) = sum_k G[s s'][k] c_k(p) and the
                            stream rebuilds them per point (66 values instead of 231
                            for odd l <= 5, 45 instead of 120 for even l <= 4, 28
                            instead of 55 for odd l <= 3).  bsl_hv_prep selects it
                            for those bases when the FP64 blocks reproduce from the
                            coefficients to 1e-10 of their largest element. */
int bsl_set_potential_format(bsl_handle* h, int format);
int bsl_potential_format(const bsl_handle* h);

/* Largest |block element - its spherical-harmonic expansion| of the prepared
   FP64 blocks (kJ/mol), or -1 when the basis has no generated expansion. */
double bsl_gaunt_residual(const bsl_handle* h);

/* uec += H vec with host buffers in the reference layout.  Replaces
   Hv_linRotCartSph_NoQuad (linRotCartSphHvFullVPrepRoutines.cpp:807-822):
   same accumulation contract, same masking of the components outside the
   symmetry block. */
int bsl_hv_apply(bsl_handle* h, const double* vec, double* uec);

/* u = H v on device buffers in the packed layout, on `stream` (cudaStream_t,
   NULL = the legacy default stream). */
int bsl_hv_apply_device(bsl_handle* h, const double* d_v, double* d_u, void* stream);

/* Lanczos loop 1 on the device (lanczosEigenValuesVectors.cpp:170-242): niter
   iterations from the given start vector; alpha[niter], beta[niter+1] and
   beta2[niter+1] are written on the host (index 0 of beta/beta2 is zero).
   Returns BSL_ERR_BREAKDOWN (with the iteration in the message) if beta
   vanishes or alpha/beta stop being finite. */
int bsl_lanczos_run(bsl_handle* h, int niter, int start, unsigned long long seed, double* alpha, double* beta,
                    double* beta2);

/* bsl_lanczos_run for n independent problems (different cages, symmetry
   blocks or grids, each prepared by its own bsl_hv_prep) in one call, as one
   batch on the first problem's device; alpha[b], beta[b], beta2[b] as in
   bsl_lanczos_run for problem b.  No counterpart in the reference (one problem
   per process there).
   When every problem runs BSL_PREC_MIXED with the tensor-core kinetic, FP32
   blocks and blocks of 15 or 21 functions, the iteration of all the problems
   is four grouped launches (kinetic x/y, kinetic z, potential stream, update),
   each CTA working on one problem in proportion to its size, replayed from a
   CUDA graph: alpha and beta are reduced over each problem's own CTAs, so they
   agree with separate runs to rounding, not bit for bit.  Otherwise it runs
   as bsl_lanczos_run_batch_streams.  bsl_last_run_ms_per_iter reports the
   device time of one iteration of all the problems. */
int bsl_lanczos_run_batch(bsl_handle** hs, int n, int niter, int start, unsigned long long seed, double** alpha,
                          double** beta, double** beta2);

/* The same with each problem on its own stream and blocks of iterations
   interleaved across the streams (iteration j of every problem is queued
   before iteration j + 1 of any), so the kernels of small problems overlap;
   the results are bit-identical to separate bsl_lanczos_run calls. */
int bsl_lanczos_run_batch_streams(bsl_handle** hs, int n, int niter, int start, unsigned long long seed,
                                  double** alpha, double** beta, double** beta2);

/* One iteration of the reference loop body (lanczosEigenValuesVectors.cpp:191-238)
   with the Lanczos state on the host in the reference layout: on return vec
   holds v_{j+1} and rvec holds -beta_j v_j, alpha_j/beta_j/beta2_j are written.
   Components outside the symmetry block follow the reference arithmetic
   (they receive no H contribution). */
int bsl_lanczos_step_host(bsl_handle* h, double* vec, double* rvec, double* alpha_j, double* beta_j,
                          double* beta2_j);

/* The rest of one Lanczos iteration after r += H v, on device buffers the
   caller owns, without allocating any device memory.  No counterpart in the
   reference.  It is for callers that cannot call cudaMalloc at the point where
   they run the recurrence: applications that reserve all GPU memory up front
   in their own pool (an allocation would fail or break their accounting), and
   loops that cannot afford the device-wide synchronisation an allocation or a
   free may imply.

   d_vec holds v_j, d_rvec holds r_j + H v_j (n doubles each, any layout, FP64;
   the two ranges and d_abb must not overlap: BSL_ERR_INPUT).  On return, as in
   the reference loop body (lanczosEigenValuesVectors.cpp:202-238):
   alpha = v.r, r -= alpha v, beta = |r|, d_vec = r / beta, d_rvec = -beta v_j,
   and d_abb[0..2] = {alpha, beta, beta^2} (device memory).  Work is queued on
   `stream` (cudaStream_t as void*, NULL = legacy default stream) and runs in
   the calling thread's current CUDA context; nothing is synchronised, so a
   breakdown cannot be returned as a status: when beta is zero or not finite
   (or alpha not finite) d_abb holds those values and d_vec, d_rvec are left as
   v_j and r_j - alpha v_j, unscaled.  Check d_abb[1] > 0 and finite before the
   next iteration.

   The reduction scratch is one static device array of 4112 doubles (32.9 KB)
   that every GPU loading the library holds until the process exits; it limits
   n to 1..8,388,608 (BSL_ERR_INPUT beyond).  All calls in a context share it
   and it keeps the last call's contents: calls that overlap on the GPU
   (different streams without ordering) race and give wrong results.  The
   array's device address is looked up once per CUDA context
   (cudaGetSymbolAddress) by the first call made in that context, and again
   after a cudaDeviceReset (a new context); make that first call before any
   stream capture begins. */
int bsl_lanczos_orthonormalize_static(double* d_vec, double* d_rvec, long long n, double* d_abb, void* stream);

/* Cullum-Willoughby good eigenvalues in (emin, emax] with inverse-iteration
   error estimates (lancbis.cpp:5-105 with BISEC/ISOEV/INVERR).  eval and err
   need niter entries; *ngood receives the count. */
int bsl_good_eigenvalues(int niter, const double* alpha, const double* beta, const double* beta2, double emin,
                         double emax, double* eval, double* err, int* ngood);

/* The same with the multiplicity tolerances of the bisection built on
   `unit_roundoff` instead of the FP64 unit roundoff 2^-52: eigenvalues of T_m
   closer than (niter + 1000) * unit_roundoff * max|T| count as one multiple
   eigenvalue.  No counterpart in the reference.  For recurrences driven by an
   inexact H v (BSL_PREC_MIXED): the converged copies of a level then scatter by
   the H v noise instead of coinciding to FP64 rounding, and with the FP64
   tolerance each copy is tested as a simple eigenvalue and can be discarded as
   spurious.  BSL_MIXED_UNIT_ROUNDOFF is the value measured for BSL_PREC_MIXED
   with the tensor-core kinetic. */
#define BSL_MIXED_UNIT_ROUNDOFF 4.0e-15
int bsl_good_eigenvalues_unit(int niter, const double* alpha, const double* beta, const double* beta2, double emin,
                              double emax, double unit_roundoff, double* eval, double* err, int* ngood);

/* The same with a floor under the multiplicity window: eigenvalues of T_m
   closer than max((niter + 1000) * unit_roundoff, rel_noise) * max|T| count as
   one multiple (good) eigenvalue; an eigenvalue alone in that window is tested
   against T without its first row in the window built on unit_roundoff, as in
   bsl_good_eigenvalues_unit.  The copies of a converged level that an inexact
   H v produces scatter by about the relative error of H v times max|T|
   however long the run, while the window built on a unit roundoff grows with
   niter; in short runs it can be narrower than the scatter, every copy then
   looks simple and each sits next to a copy in T without its first row, so
   the level is lost as spurious.  BSL_MIXED_REL_NOISE is the floor for
   BSL_PREC_MIXED (rel_noise = 0: bsl_good_eigenvalues_unit). */
#define BSL_MIXED_REL_NOISE 1.0e-9
int bsl_good_eigenvalues_noise(int niter, const double* alpha, const double* beta, const double* beta2,
                               double emin, double emax, double unit_roundoff, double rel_noise, double* eval,
                               double* err, int* ngood);

/* Tm eigenvectors for the first ngood good eigenvalues (lanczosvectors +
   TRIVEC, lanczosEigenValuesVectors.cpp:509-561): evtr is column-major
   [niter x ngood]. */
int bsl_tm_eigenvectors(int niter, const double* alpha, const double* beta, const double* beta2,
                        const double* eval, int ngood, double* evtr);

/* Lanczos loop 2 with Ritz accumulation on the device
   (lanczosEigenValuesVectors.cpp:371-469): ritz[n*D + row] in the reference
   layout, D = bsl_basis_size(h). */
int bsl_ritz_vectors(bsl_handle* h, int niter, const double* evtr, int ngood, double* ritz);

/* Result files in the reference's formats (lanczosEigenValuesVectors.cpp):
   boundstates.txt + states_zpe.txt (:263-290), lv (:339-364, evtr column-major
   [niter x ngood]) and eigVecFile.txt (:470-492, ritz[n * basis_size + row]),
   written into `dir` with the simulation description sim_descr. */
int bsl_write_boundstates(const char* dir, const char* sim_descr, int ngood, const double* eval, const double* err);
int bsl_write_tm_vectors(const char* dir, const char* sim_descr, int niter, int ngood, const double* evtr);
int bsl_write_ritz_vectors(const char* dir, const char* sim_descr, long long basis_size, int ngood,
                           const double* ritz);

/* Hellmann-Feynman derivatives dE_n/dtheta = <psi_n| dV/dtheta |psi_n> of nlev
   levels with respect to the cage (Alavi SPC/E potential, the grid kept with
   keep_potential_grid): psi[n * basis_size + row] eigenvectors in the reference
   layout (any normalisation; e.g. from bsl_ritz_vectors); outputs
   dq_site[n * natoms + w] (kJ/mol per e), dr_site[(n * natoms + w) * 3 + k]
   (kJ/mol per nm), dq_alavi[2 n + {0, 1}] (the H and centre-of-mass charges of
   H2).  Sites are O, H1, H2 (SPC/E) or O, H1, H2, M (TIP4P) per molecule in file
   order.  No counterpart in the reference. */
int bsl_hf_gradient(bsl_handle* h, int nlev, const double* psi, double* dq_site, double* dr_site,
                    double* dq_alavi);

/* Chain rule from site positions to the rigid-body coordinates of the cage
   (centre of mass in Angstrom, ZYZ Euler angles in rad; SPCE_AH2_EngRoutines.cpp:5-108,
   TIP4P_AH2_EngRoutines.cpp): potential = BSL_POT_ALAVI_SPCE (3 sites per
   molecule) or BSL_POT_ALAVI_TIP4P (4); dr_site[(n * S nmol + site) * 3 + k] ->
   d_cm[(n * nmol + m) * 3 + k], d_euler[(n * nmol + m) * 3 + k].  Host only. */
int bsl_rigid_body_gradient(int potential, int nmol, const double* cm_ang, const double* euler, int nlev,
                            const double* dr_site, double* d_cm, double* d_euler);

/* Site positions (nm) and charges of a cage of rigid waters of the given model:
   xyz[3 * S nmol], q[S nmol] (q_site NULL: the model's charges).  Host only. */
int bsl_cage_sites(int potential, int nmol, const double* cm_ang, const double* euler, const double* q_site,
                   double* xyz, double* q);

/* bsl_ritz_vectors from the start vector of a bsl_lanczos_run(start, seed)
   (bsl_ritz_vectors itself restarts from BSL_START_UNIFORM, as the reference). */
int bsl_ritz_vectors_start(bsl_handle* h, int niter, int start, unsigned long long seed, const double* evtr, int ngood,
                           double* ritz);

/* Timing of the last bsl_lanczos_run: average device milliseconds per
   iteration, measured with CUDA events on the library's stream.  After
   bsl_lanczos_run_batch every handle of the batch reports the batch's device
   time (first problem's start to last problem's end) divided by niter: the
   time of one iteration of all the problems. */
int bsl_last_run_ms_per_iter(const bsl_handle* h, double* ms);

/* Diagnostic: one 128 x 64 x 64 TF32 product through the tensor cores
   (tcgen05.mma from swizzled shared memory into tensor memory) on the current
   device, compared with its exact value; *max_abs_err receives the largest
   deviation (0 when the tensor-core path is sound). */
int bsl_selftest_tensor_core(double* max_abs_err);

/* Per-kernel device time of the Lanczos iteration: runs `iters` iterations
   (continuing the current device state) with CUDA events around every
   kernel on the library's stream and writes the average milliseconds per
   launch of the stages {kinetic x/y, kinetic z, potential apply + alpha,
   update + beta, normalise + swap} into ms[0..4]; names[i] (optional) receives
   the kernel name of stage i (static strings). */
int bsl_stage_times(bsl_handle* h, int iters, double* ms, const char** names);

/* Launch-shape autotuner, with no counterpart in the reference: times
   `iters` Lanczos iterations of the problem (n = 1, bsl_lanczos_run) or of the
   batch (n > 1, bsl_lanczos_run_batch) for each launch shape that the
   problem's size does not fix -- resident CTAs per SM of the potential stream
   or the fused update (1-3, capped by its occupancy) and, where a problem runs
   the streamed update, of that update (1-3; else it stays 2) -- and keeps the
   fastest in the handles for later runs.  The choice is cached per problem
   set (block sizes, grids, precision, kinetic engine, block format, slices),
   so a later call with the same sizes reuses it without timing.  Outputs (any
   may be NULL): the chosen shapes and the best device ms per iteration (of the
   whole batch for n > 1).  Overwrites the handles' Lanczos state. */
int bsl_autotune(bsl_handle** hs, int n, int iters, int* vs_per_sm, int* upd_per_sm, double* ms_per_iter);

/* Test hook for the failure paths, with no counterpart in the reference.
   Every bounded wait of the potential-block stream and of the tensor-core
   kinetic records a time-out in a device status word, and the next
   bsl_lanczos_run / bsl_lanczos_step_host returns BSL_ERR_CUDA with the
   stage named.  kernel_mask bit 0 (potential stream) and bit 1 (tensor-core
   kinetic) make every later run or step start with that stage's time-out
   already recorded: the kernels then skip their copies, MMAs and waits, the
   results are meaningless and the call returns the error.  0 clears the
   injection; the handle is usable again at once.  Nothing on the GPU is made
   to wait or fault. */
int bsl_debug_inject_timeout(bsl_handle* h, int kernel_mask);

/* Kernel launches per Lanczos iteration of the current configuration. */
int bsl_launches_per_iteration(const bsl_handle* h);

/* The stream the library launches on (cudaStream_t as void*). */
void* bsl_stream(const bsl_handle* h);

/* Diagnostics for tests: copy the potential grid (packed halves, see
   bsl_vgrid_size) or the potential blocks to the host, FP64. */
long long bsl_vgrid_size(const bsl_handle* h);
int bsl_copy_vgrid(const bsl_handle* h, double* v1, double* v2);
long long bsl_vblock_size(const bsl_handle* h);
int bsl_copy_vblocks(const bsl_handle* h, double* out);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* BSL_H */
