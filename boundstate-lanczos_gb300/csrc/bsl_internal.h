// Internal declarations shared by the host translation units and the CUDA
// kernels of the boundstate-lanczos GB300 library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "bsl.h"

namespace bsl {

// Physical constants in the reference's unit system (nm, ps, amu, kJ/mol),
// headLoop/InterfaceCode/lanczosUnits.h:5-14.
constexpr double kPi = 3.141592653589793;
constexpr double kCoulombK = 138.9354846111096;
constexpr double kHbar = 0.0635077857002;
constexpr double kNmPerAngstrom = 0.1;

// Largest packed (l,m) block with a register-resident potential kernel.
constexpr int kMaxNN = 36;

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);

#define BSL_CUDA(call)                                        \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return ::bsl::cuda_fail(_e, #call); \
  } while (0)

// Host-side basis and quadrature tables (all FP64).
struct Tables {
  int nx = 0, ny = 0, nz = 0;
  long long npts = 0;          // nx*ny*nz
  int lmax = 0, nn_full = 0;   // (lmax+1)^2
  int nn = 0;                  // functions kept by the symmetry block
  int na = 0, nb = 0;          // theta nodes, phi nodes per half
  std::vector<int> l_of, m_of; // full composite index -> l, m
  std::vector<int> full_of;    // packed index -> full index
  std::vector<double> xg, yg, zg;       // grids
  std::vector<double> tx, ty, tz;       // kinetic matrices, row-major [i*n + i']
  std::vector<double> rot;              // rotor energies B l(l+1), packed
  std::vector<double> gl_x, gl_w;       // Gauss-Legendre nodes in cos(theta), weights
  std::vector<double> gc_x, gc_w;       // cos(phi_b), weights pi/nb
  std::vector<double> theta, phi, phi2; // acos values, 2pi - phi
  std::vector<double> leg;              // [s][a] normalised associated Legendre, packed
  std::vector<double> trig1, trig2;     // [m+lmax][b] trig factor at phi_b and 2pi-phi_b
};

// Water cage: atom positions (nm), charges, LJ flag (oxygen).
struct Cage {
  std::vector<double> xyz;  // [atom][3], nm
  std::vector<double> q;
  std::vector<int> is_o;
  // rigid-body description: per molecule the centre of mass (Angstrom) and the
  // ZYZ Euler angles (rad); `sites` sites per molecule (SPC/E: O, H1, H2;
  // TIP4P: O, H1, H2, M)
  std::vector<double> cm_ang, euler;
  int model = BSL_POT_ALAVI_SPCE, sites = 3;
  // Lennard-Jones A / r^12 - B / r^6 between the H2 centre of mass and each O
  double lj_a = 1.364e-06, lj_b = 1.533e-3;
  // Alavi H2 charges on each H and on the centre of mass (Alavi_Parameters.h:5-6)
  double q_h2_h = 0.4932, q_h2_cm = -0.9864;
};

// water model of the cage a potential reads (BSL_POT_ALAVI_SPCE or BSL_POT_ALAVI_TIP4P)
inline int cage_model(int potential) {
  return (potential == BSL_POT_ALAVI_TIP4P || potential == BSL_POT_POINT_ALAVI_TIP4P) ? BSL_POT_ALAVI_TIP4P
                                                                                      : BSL_POT_ALAVI_SPCE;
}
inline bool has_cage(int potential) { return potential != BSL_POT_ISOHARMOSC && potential != BSL_POT_COULOMB; }
inline bool point_grid_alavi(int potential) {
  return potential == BSL_POT_POINT_ALAVI_SPCE || potential == BSL_POT_POINT_ALAVI_TIP4P;
}

// Sites of a cage of rigid waters (SPC/E: SPCE_AH2_EngRoutines.cpp:5-108; TIP4P:
// TIP4P_AH2_EngRoutines.cpp getTIP4Patoms; rotmat.cpp:6-32); q_site (one per
// site) may be null for the model's charges.
void build_cage(int model, int nmol, const double* cm_ang, const double* euler, const double* q_site, Cage* c);
// d site / d (Euler angle k) for molecule m, site a of the model: out[3]
void site_angle_derivative(const Cage& c, int m, int a, int k, double* out);

int build_tables(const bsl_hv_params& p, Tables* t);
int read_cage(const std::string& path, int model, Cage* c);

// Device-resident state of one prepared Hamiltonian.
struct DeviceState {
  cudaStream_t stream = nullptr;
  // kinetic matrices: FP64 and the FP32 hi/lo split (T = hi + lo + O(2^-48))
  double *tx = nullptr, *ty = nullptr, *tz = nullptr;
  // FP32 heads fl32(T) and tails fl32(T - head), both stored transposed, for the mixed kernels
  float *kx_head = nullptr, *ky_head = nullptr, *kz_head = nullptr;
  float *kx_band = nullptr, *ky_band = nullptr, *kz_band = nullptr;
  // fixed-point FP16 slices of T (5 zero-padded 64 x 64 tiles) and their scale
  // exponents, for the tensor-core kinetic
  uint16_t *kxy_slices = nullptr, *kz_slices = nullptr;
  int e_txy = 0, e_tz = 0;
  int kin_grid_xy = 0, kin_grid_z = 0;  // persistent grid sizes
  double* rot = nullptr;  // [nn]
  // potential grid V(p, a, b) for phi_b and 2pi - phi_b, p in vector order
  double *v1 = nullptr, *v2 = nullptr;
  // potential blocks, packed upper triangle t = (s, s') with s <= s', [t][p]
  double* vb64 = nullptr;
  float* vb32 = nullptr;
  // Lanczos work vectors (packed layout) and reduction scratch
  double *vec = nullptr, *rvec = nullptr, *ukin = nullptr;  // ukin: FP64, or (hi, lo) FP32 pairs (mixed)
  float* v32 = nullptr;                       // FP32 copy of the current Lanczos v (mixed)
  float2* vpair = nullptr;                    // double-float copy of an FP64 input v (tensor-core kinetic)
  float *rot_hi = nullptr, *rot_lo = nullptr; // rotor energies as FP32 head + tail
  double* partials = nullptr;  // one double per reduction block
  unsigned int* counter = nullptr;
  // [0] alpha_j, [1] beta_j, [2] beta2_j, [3] 1/beta_j, [4] sv, [5] sr, [6] sv/sr, [7] sv*sr;
  // pair state: [8] sv/sr and [9] -alpha sv/sr as double-float pairs, [10] (int) exponent of
  // the update's power-of-two factor
  double* scalars = nullptr;
  // [0] breakdown, [1] its iteration, [2] potential-block stream timeout, [3] tensor-core kinetic timeout
  int* status = nullptr;
  double* hist = nullptr;      // alpha/beta/beta2 history [3][niter+1]
  int hist_cap = 0;
  // host-layout staging
  double *ref_vec = nullptr, *ref_out = nullptr;  // full reference layout
  int* full_of = nullptr;                          // packed -> full index
  int* packed_of = nullptr;                        // full (l, m) index -> packed, -1 outside the block
  cudaStream_t copy_stream = nullptr;              // host-state step: second copy-in stream
  cudaEvent_t copy_done = nullptr;
  cudaEvent_t vec_in = nullptr;                    // host-state step: vec is on the device
  double* ritz = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int red_blocks = 0;
  int* jdev = nullptr;  // iteration counter of graph-replayed Lanczos loops
  int pair_blocks = 0;  // grid of the double-float update: a few resident blocks per SM
  // captured block of device-counted Lanczos iterations, kept across runs until
  // something its launches depend on changes (graph_key)
  cudaGraph_t iter_graph = nullptr;
  cudaGraphExec_t iter_exec = nullptr;
  // precision, kinetic engine, buffer roles, hist, hist_cap, kinetic slices, block format, launch shapes
  long long graph_key[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  // BF16 potential blocks (tile-major like vb32) and their per-point FP32 scales
  uint16_t* vb16 = nullptr;
  float* vscale = nullptr;
  // the blocks as spherical-harmonic coefficients, FP32 tile-major [tile][k][128]
  float* vc32 = nullptr;
  // graph-replayed iterations with the fused update: the potential block
  // product of the next v, FP32 [s][p] (allocated by prepare_iterations)
  float* vprod = nullptr;
  // test hook: status words set again after every reset of the status (host-side
  // injection of a kernel time-out; bit 2: potential stream, bit 3: kinetic)
  int inject_status = 0;
};

}  // namespace bsl

struct bsl_handle {
  bsl_hv_params p;
  bsl::Tables t;
  bsl::Cage cage;
  bsl::DeviceState d;
  int precision = BSL_PREC_FP64;
  int kinetic_engine = BSL_KIN_SIMT;  // engine of the mixed-precision kinetic (BSL_KIN_*)
  int kin_slices = 4;                 // 9-bit slices of the tensor-core kinetic (4: exact)
  int vformat = BSL_VFMT_FP32;        // storage of the mixed path's potential blocks (BSL_VFMT_*)
  double gaunt_residual = -1.0;       // largest |block - expansion| at prep (FP64), -1: no expansion
  // launch shapes picked by bsl_autotune (0: the defaults): resident CTAs per SM
  // of the potential stream (capped by its occupancy) and of the update
  int tune_vs = 0, tune_upd = 0;
  // the iteration being launched defers its reductions (graph-replayed iterations)
  int defer_reductions = 0;
  double last_ms_per_iter = 0.0;
  int lanczos_flip = 0;           // 0: vec holds v_j and rvec r_j; 1: roles swapped
  int state_pairs = -1;           // Lanczos buffers: 0 FP64, 1 double-float pairs (mixed), -1 not set up
  double init_scalars[8] = {0, 0, 0, 0, 1, 1, 1, 1};  // alpha, beta, beta2, 1/beta, sv, sr, sv/sr, sv*sr
};

namespace bsl {

// ---- kernel launchers (bsl_kernels.cu) -----------------------------------
int dev_potential_alavi(bsl_handle* h);
int dev_potential_iso(bsl_handle* h);
int dev_set_iteration(bsl_handle* h, int j, cudaStream_t s);
bool device_counted_iterations(const bsl_handle* h);
// after the last device-counted iteration of a run: its deferred beta
int dev_finish_iterations(bsl_handle* h, cudaStream_t s);
// device-counted iterations that use the fused update (and its product buffer)
bool fused_iterations(const bsl_handle* h);
// before the first device-counted iteration of a run: the product buffer and,
// for the fused update, the block product of the current v
int dev_begin_iterations(bsl_handle* h, cudaStream_t s);
// the product buffer alone (before an iteration graph is captured)
int ensure_product_buffer(bsl_handle* h);
// the block totals of the beta an iteration of h leaves pending
int deferred_beta_count(bsl_handle* h);
int dev_potential_point_alavi(bsl_handle* h);
int dev_potential_coulomb(bsl_handle* h);
int dev_vblocks(bsl_handle* h);
int dev_hv(bsl_handle* h, const double* v, double* u, cudaStream_t s);
// One Lanczos iteration on the packed state (vec, rvec) with the device
// iteration index j (1-based) used to store alpha/beta history.
int dev_lanczos_iteration(bsl_handle* h, int j, cudaStream_t s);
int dev_lanczos_iteration_timed(bsl_handle* h, int j, cudaStream_t s, cudaEvent_t* ev);
const char* dev_stage_name(bsl_handle* h, int i);
int dev_fill_start(bsl_handle* h, int start, unsigned long long seed, cudaStream_t s);
int dev_gather_packed(bsl_handle* h, const double* full, double* packed, cudaStream_t s);
int dev_hv_full(bsl_handle* h, const double* full, double* out, cudaStream_t s);
int dev_full_step_fused(bsl_handle* h, double* v, double* r, long long L, const double* hv, int j, cudaStream_t s,
                        double* v_out = nullptr, double* r_out = nullptr);
int dev_scatter_full(bsl_handle* h, const double* packed, double* full_accum, cudaStream_t s);
// previous: the v of the iteration just launched (the buffer roles have flipped)
int dev_ritz_accumulate(bsl_handle* h, const double* coef, const int* active, int ngood, double* ritz,
                        cudaStream_t s, bool previous);

// mixed-precision kinetic (bsl_kinetic.cu)
void kinetic_split_tables(const std::vector<double>& T, int n, bool transpose, std::vector<float>* head,
                          std::vector<float>* band);
// mixed kinetic: FP32 input v, output u_kin as (hi, lo) FP32 pairs in d.ukin
int launch_kin_xy_mixed(bsl_handle* h, const float* v, cudaStream_t s);
int launch_kin_z_mixed(bsl_handle* h, const float* v, cudaStream_t s);

// tensor-core kinetic (bsl_kinetic_tc.cu): the same output as the mixed
// kernels, from the double-float Lanczos vector, for grids of at most 64 points
// per axis with Tx = Ty
void kinetic_smem_image(const std::vector<double>& T, int n, bool with_zero_tiles, std::vector<uint16_t>* image,
                        int* e_t);
bool kinetic_tc_supported(const Tables& t);
int launch_kin_xy_tc(bsl_handle* h, const float2* v, cudaStream_t s);
int launch_kin_z_tc(bsl_handle* h, const float2* v, cudaStream_t s);
// grouped tensor-core kinetic over several problems: per-problem argument
// records (kin_group_arg_size() bytes each, filled by kin_tc_group_args for the
// vectors v[b]) and per-CTA work (problem, first pair, end pair, 0)
size_t kin_group_arg_size();
long long kin_tc_pairs(const bsl_handle* h, bool xy);
// fin_counts (x/y, or null): per problem, the block totals of the deferred beta
// its first CTA finishes
void kin_tc_group_args(bsl_handle** hs, int n, const float2* const* v, bool xy, const int* fin_counts, void* args);
int launch_kin_tc_group(bool xy, const void* d_args, const int4* d_work, int nctas, cudaStream_t s);

// potential-block apply (bsl_vapply_f32.cu / bsl_vapply_f64.cu)
// FP32 blocks in the tile-major layout of bsl_vstream.cu (vstream_tile_points() points per tile)
struct StreamArgs {
  const float* vb;      // tile-major FP32 blocks
  const float* v32;     // FP32 copy of v
  const double* vec;    // FP64 v (alpha dot product, extra coordinate)
  const float2* ukin;   // kinetic (hi, lo) pairs
  const float* rot_hi;  // rotor energies, head and tail
  const float* rot_lo;
  double* out;          // mode 0: u = H v; mode 1: the Lanczos r buffer (r += c H v)
  const uint16_t* vb16; // BSL_VFMT_BF16: tile-major BF16 blocks, V = vscale[p] * block
  const float* vscale;
  const float* vc;      // BSL_VFMT_GAUNT: tile-major spherical-harmonic coefficients
  float* vprod;         // fused update: the block product of the next v (FP32 [s][p])
  int vformat;
  int nn, red_count;    // grouped launch: block size, blocks that reduce this problem's alpha
  int defer;            // mode 2: store the block totals of alpha only (the update forms alpha)
  int ctas_per_sm;      // 0: as many as fit
  long long npts, dpk;
  long long tiles_per_cta;  // set by the launcher
  int mode, j;          // j > 0: the iteration; j == 0: read it from *jdev
  const int* jdev;
  double *partials, *scalars, *hist;
  unsigned int* counter;
  int* status;
};
int launch_vapply_f32(const StreamArgs& a, int nn, cudaStream_t s);
// Graph-replayed iterations with the fused update: the light H v apply
// (R += c H v with the block product from a.vprod; alpha's block totals) and
// the update fused with the next block product (role 1), or that product
// alone (role 2, before the first iteration).
bool fused_update_supported(int vformat, int nn);
int fused_update_ctas(const StreamArgs& a, int nn);
int launch_update_fused(const StreamArgs& a, int nn, int role, cudaStream_t s);
int launch_vapply_light(const StreamArgs& a, int nn, cudaStream_t s);
long long vstream_tile_points();
// double-float update R = g (R - alpha c V), beta and the next scales, streamed
// with bulk copies (V, R 16-byte aligned; partials sized for 2 CTAs per SM)
// j == 0: the iteration is read from *jdev, which the last block then advances
// defer: alpha from the stream's block totals, beta's block totals left for
// the next x/y kinetic or launch_finish_beta (graph-replayed iterations)
int launch_update_stream(const float2* V, float2* R, long long L, double* partials, unsigned int* counter,
                         double* scalars, double* hist, int hist_stride, int j, int* jdev, int* status,
                         cudaStream_t s, int ctas_per_sm = 0, int defer = 0);
int update_stream_ctas(int ctas_per_sm);
// index of the first of the deferred beta's block totals in the partials
// buffer (alpha's block totals start at 0)
constexpr int kBetaPartials = 2048;
// the deferred beta after the last iteration of a run (`count` block totals)
int launch_finish_beta(double* partials, int count, double* scalars, double* hist, int hist_stride, int* jdev,
                       int* status, cudaStream_t s);
// grouped launches of the fused iteration over several problems: per-problem
// argument records (StreamArgs) and per-CTA work (problem, first unit, end
// unit, block index in the problem's reduction); the light apply in blocks of
// light_points_per_cta() points (one block per CTA), the fused update in tiles
// of vstream_tile_points() points
size_t vstream_group_arg_size();
long long light_points_per_cta();
bool vstream_group_supported(int nn);
int vstream_group_ctas_per_sm();
int launch_light_group(const void* d_args, const int4* d_work, int nctas, cudaStream_t s);
int launch_vstream_group(const void* d_args, const int4* d_work, int nctas, cudaStream_t s);
// the potential stream's arguments for one problem (mode 2, j from the device counter)
StreamArgs vstream_args(bsl_handle* h, const double* v, double* out);
int launch_vapply_f64(const double* vb, dim3 g, cudaStream_t s, int nn, const double* v, const double* uk,
                      const double* rot, double* out, long long N, int mode, double* partials, unsigned int* counter,
                      double* scalars, double* hist, int j, long long dpk);

// BF16 copy of the potential blocks with per-point scales (bsl_vstream.cu)
int dev_vblocks_bf16(bsl_handle* h);
// spherical-harmonic coefficients of the potential blocks (bsl_gaunt.cu): the
// count for the handle's basis (0: no generated expansion), and the prep that
// recovers them from the FP64 blocks (largest reconstruction residual and
// largest |block element| returned)
int gaunt_coefficient_count(const bsl_handle* h);
int dev_gaunt_coeffs(bsl_handle* h, double* residual, double* vmax);

// the cached iteration graph (bsl_lanczos.cpp)
void release_iteration_graph(DeviceState& d);

// ---- Cullum-Willoughby tail (bsl_tail.cpp) --------------------------------
// unit <= 0: the reference's 2^-52; noise > 0: floor of the multiplicity
// window relative to max|T|
int cw_good_eigenvalues(int niter, const double* alpha, const double* beta, const double* beta2, double emin,
                        double emax, double* eval, double* err, int* ngood, double unit = 0.0, double noise = 0.0);
int cw_tm_eigenvectors(int niter, const double* alpha, const double* beta, const double* beta2,
                       const double* eval, int ngood, double* evtr);

}  // namespace bsl
