// Lanczos drivers of the C ABI: the device-resident loop, the host-state
// single step, and the Ritz-vector pass.
//
// Reference driver: headLoop/LanczosCode/lanczosEigenValuesVectors.cpp
//   start vector 1/sqrt(D)                       :177-181
//   loop 1 (alpha, beta, scale, swap)            :187-242
//   loop 2 with Ritz accumulation and cut-off    :371-469
//
// The device loop runs on the packed symmetry block plus one extra
// coordinate.  The reference keeps all (l_max+1)^2 functions and multiplies H
// by the 0/1 symmetry mask, so the components outside the block never receive
// an H contribution: starting from the uniform vector they stay proportional to
// one fixed unit vector.  That direction is carried as the single extra
// coordinate (H acts on it as 0), which reproduces the reference's recurrence
// -- including its spurious eigenvalue at 0 -- with D_packed + 1 unknowns.
#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "bsl_internal.h"

namespace bsl {
int dev_fill(double* x, long long L, double val, cudaStream_t s);
int dev_to_f32(const double* x, float* y, long long n, cudaStream_t s);
int dev_to_pair(double* x, long long n, cudaStream_t s);

namespace {

// The history buffer grows in steps of kHistStep iterations, so runs of
// similar length reuse it (and the captured iteration graph, whose launches
// name it).
constexpr int kHistStep = 1024;

int ensure_hist(bsl_handle* h, int niter) {
  DeviceState& d = h->d;
  if (d.hist && d.hist_cap >= niter + 1) return BSL_OK;
  release_iteration_graph(d);
  if (d.hist) cudaFree(d.hist);
  d.hist = nullptr;
  d.hist_cap = (niter + 1 + kHistStep - 1) / kHistStep * kHistStep;
  BSL_CUDA(cudaMalloc(&d.hist, 3 * (size_t)d.hist_cap * sizeof(double)));
  BSL_CUDA(cudaMemset(d.hist, 0, 3 * (size_t)d.hist_cap * sizeof(double)));
  return BSL_OK;
}

// status words cleared at the start of a run or step, then the injected
// time-out flags of the test hook (bsl_debug_inject_timeout)
int reset_status(bsl_handle* h, cudaStream_t s) {
  DeviceState& d = h->d;
  BSL_CUDA(cudaMemsetAsync(d.status, 0, 4 * sizeof(int), s));
  for (int w = 2; w <= 3; ++w)
    if (d.inject_status & (1 << w)) BSL_CUDA(cudaMemsetAsync(d.status + w, 0x01, 1, s));
  return BSL_OK;
}

// device address of a page-locked (pinned or registered) host buffer, or null
double* mapped_host(double* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? static_cast<double*>(a.devicePointer) : nullptr;
}

int ensure_staging(bsl_handle* h) {
  DeviceState& d = h->d;
  if (!d.copy_stream) {
    BSL_CUDA(cudaStreamCreateWithFlags(&d.copy_stream, cudaStreamNonBlocking));
    BSL_CUDA(cudaEventCreateWithFlags(&d.copy_done, cudaEventDisableTiming));
    BSL_CUDA(cudaEventCreateWithFlags(&d.vec_in, cudaEventDisableTiming));
  }
  if (d.ref_vec) return BSL_OK;
  const size_t Df = (size_t)bsl_basis_size(h);
  BSL_CUDA(cudaMalloc(&d.ref_vec, Df * sizeof(double) + 16));
  BSL_CUDA(cudaMalloc(&d.ref_out, Df * sizeof(double) + 16));
  return BSL_OK;
}

uint64_t splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// N(0,1) by Box-Muller on splitmix64 uniforms (53-bit), normalised to 1.
void normal_vector(uint64_t seed, size_t n, std::vector<double>* v) {
  v->resize(n);
  uint64_t s = seed;
  const double two_pi = 6.283185307179586;
  for (size_t i = 0; i < n; i += 2) {
    const double u1 = ((splitmix64(&s) >> 11) + 1.0) * (1.0 / 9007199254740993.0);
    const double u2 = (splitmix64(&s) >> 11) * (1.0 / 9007199254740992.0);
    const double r = std::sqrt(-2.0 * std::log(u1));
    (*v)[i] = r * std::cos(two_pi * u2);
    if (i + 1 < n) (*v)[i + 1] = r * std::sin(two_pi * u2);
  }
  double nrm = 0.0;
  for (size_t i = 0; i < n; ++i) nrm += (*v)[i] * (*v)[i];
  nrm = std::sqrt(nrm);
  for (size_t i = 0; i < n; ++i) (*v)[i] /= nrm;
}

int init_state(bsl_handle* h, int start, unsigned long long seed) {
  DeviceState& d = h->d;
  const long long D = bsl_packed_size(h), Df = bsl_basis_size(h);
  cudaStream_t s = d.stream;
  int rc;
  if (start == BSL_START_UNIFORM) {
    if ((rc = dev_fill(d.vec, D, 1. / std::sqrt((double)Df), s))) return rc;
    const double ghost = std::sqrt((double)(Df - D) / (double)Df);
    BSL_CUDA(cudaMemcpyAsync(d.vec + D, &ghost, sizeof(double), cudaMemcpyHostToDevice, s));
  } else if (start == BSL_START_NORMAL) {
    std::vector<double> v;
    normal_vector(seed, (size_t)D, &v);
    v.push_back(0.0);
    BSL_CUDA(cudaMemcpyAsync(d.vec, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    BSL_CUDA(cudaStreamSynchronize(s));
  } else {
    return fail(BSL_ERR_INPUT, "unknown start vector kind");
  }
  if ((rc = dev_fill(d.rvec, D + 1, 0.0, s))) return rc;
  if ((rc = reset_status(h, s))) return rc;
  BSL_CUDA(cudaMemsetAsync(d.scalars, 0, 16 * sizeof(double), s));
  BSL_CUDA(cudaMemcpyAsync(d.scalars, h->init_scalars, 8 * sizeof(double), cudaMemcpyHostToDevice, s));
  // pair-state constants: [8] c = 1 as a double-float pair, [10] the update's exponent 0
  static const float kOnePair[2] = {1.f, 0.f};
  BSL_CUDA(cudaMemcpyAsync(d.scalars + 8, kOnePair, sizeof(kOnePair), cudaMemcpyHostToDevice, s));
  if ((rc = dev_to_f32(d.vec, d.v32, D, s))) return rc;
  // mixed precision keeps the Lanczos buffers as double-float pairs (the zero
  // R buffer is the same bits either way)
  h->state_pairs = h->precision == BSL_PREC_MIXED ? 1 : 0;
  if (h->state_pairs && (rc = dev_to_pair(d.vec, D + 1, s))) return rc;
  h->lanczos_flip = 0;
  return BSL_OK;
}

int check_status(bsl_handle* h) {
  int st[4] = {0, 0, 0, 0};
  BSL_CUDA(cudaMemcpy(st, h->d.status, 4 * sizeof(int), cudaMemcpyDeviceToHost));
  if (st[2]) return fail(BSL_ERR_CUDA, "potential-block stream: a bulk copy did not complete within its time limit");
  if (st[3]) return fail(BSL_ERR_CUDA, "tensor-core kinetic: an MMA did not complete within its time limit");
  if (st[0]) return fail(BSL_ERR_BREAKDOWN, "Lanczos breakdown at iteration " + std::to_string(st[1]) +
                                                ": beta is zero or alpha/beta are not finite");
  return BSL_OK;
}

// niter Lanczos iterations of one problem on stream s.  Where the iteration's
// kernels can take j from the device counter, kGraphIters iterations are
// captured into a CUDA graph (programmatic launches become programmatic
// edges) and replayed; an even count leaves the buffer roles as they were.
// The graph is kept with the handle until the precision, the kinetic engine
// or the history buffer changes.  The remainder, and every other
// configuration, is launched directly.
constexpr int kGraphIters = 32;

// capture kGraphIters device-counted iterations of h on its stream (nothing
// runs) unless the cached graph already matches the current configuration
int ensure_iteration_graph(bsl_handle* h) {
  DeviceState& d = h->d;
  const long long key[9] = {h->precision, h->kinetic_engine, h->lanczos_flip, (long long)(uintptr_t)d.hist,
                            d.hist_cap, h->kin_slices, h->vformat, h->tune_vs, h->tune_upd};
  if (d.iter_exec && std::memcmp(key, d.graph_key, sizeof(key)) == 0) return BSL_OK;
  release_iteration_graph(d);
  cudaStream_t s = d.stream;
  BSL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  int rc = BSL_OK;
  for (int i = 0; i < kGraphIters && rc == BSL_OK; ++i) rc = dev_lanczos_iteration(h, 0, s);
  const cudaError_t e = cudaStreamEndCapture(s, &d.iter_graph);
  if (rc) {
    release_iteration_graph(d);
    return rc;
  }
  if (e != cudaSuccess) {
    release_iteration_graph(d);
    return cuda_fail(e, "cudaStreamEndCapture");
  }
  const cudaError_t ei = cudaGraphInstantiate(&d.iter_exec, d.iter_graph, 0);
  if (ei != cudaSuccess) {
    release_iteration_graph(d);
    return cuda_fail(ei, "cudaGraphInstantiate");
  }
  BSL_CUDA(cudaGraphUpload(d.iter_exec, s));
  std::memcpy(d.graph_key, key, sizeof(key));
  return BSL_OK;
}

// Everything a run of niter iterations needs before its first launch: the
// iteration graphs of the problems that replay one (captured and uploaded
// here, outside the timed region).
int prepare_iterations(bsl_handle** hs, int n, int niter) {
  int rc;
  for (int b = 0; b < n; ++b) {
    bsl_handle* h = hs[b];
    cudaSetDevice(h->p.device);
    if (device_counted_iterations(h) && ((rc = ensure_product_buffer(h)) ||
                                         (niter >= kGraphIters && (rc = ensure_iteration_graph(h)))))
      return rc;
  }
  return BSL_OK;
}

// the iterations of several problems, iteration blocks interleaved across
// their streams (prepare_iterations first)
int run_iterations(bsl_handle** hs, int n, int niter) {
  std::vector<char> counted(n, 0);
  int rc;
  for (int b = 0; b < n; ++b) {
    bsl_handle* h = hs[b];
    cudaSetDevice(h->p.device);
    counted[b] = device_counted_iterations(h) ? 1 : 0;
    if (counted[b] && ((rc = dev_set_iteration(h, 1, h->d.stream)) || (rc = dev_begin_iterations(h, h->d.stream))))
      return rc;
  }
  const int nblocks = niter / kGraphIters;
  for (int k = 0; k < nblocks; ++k)
    for (int b = 0; b < n; ++b) {
      bsl_handle* h = hs[b];
      cudaSetDevice(h->p.device);
      if (counted[b]) {
        BSL_CUDA(cudaGraphLaunch(h->d.iter_exec, h->d.stream));
      } else {
        for (int i = 0; i < kGraphIters; ++i)
          if ((rc = dev_lanczos_iteration(h, k * kGraphIters + i + 1, h->d.stream))) return rc;
      }
    }
  for (int j = nblocks * kGraphIters + 1; j <= niter; ++j)
    for (int b = 0; b < n; ++b) {
      cudaSetDevice(hs[b]->p.device);
      if ((rc = dev_lanczos_iteration(hs[b], counted[b] ? 0 : j, hs[b]->d.stream))) return rc;
    }
  for (int b = 0; b < n; ++b)
    if (counted[b]) {
      cudaSetDevice(hs[b]->p.device);
      if ((rc = dev_finish_iterations(hs[b], hs[b]->d.stream))) return rc;
    }
  return BSL_OK;
}

// ---------------------------------------------------------------------------
// Grouped batches: the iteration of every problem in one launch per stage.
// Each stage kernel takes a table of per-problem arguments and a table of
// per-CTA work (problem, first unit, end unit, block index within the
// problem); every CTA works on one problem only, so it uses that problem's
// grid, T image, vectors, scalars and reduction buffers, and each problem's
// alpha and beta are reduced over its own CTAs.  Four launches (the fused
// iteration: x/y and z kinetic, light apply, fused update) advance all the
// problems by one iteration; kGraphIters of them are captured into one graph.
// ---------------------------------------------------------------------------

// Split units[b] work units of each problem over about `slots` CTAs in
// proportion to the units (at least one CTA per problem), each CTA one
// contiguous range of one problem; ctas[b] receives problem b's CTA count.
std::vector<int4> split_work(const std::vector<long long>& units, long long slots, std::vector<int>* ctas) {
  long long total = 0;
  for (long long u : units) total += u;
  std::vector<int4> w;
  ctas->assign(units.size(), 0);
  for (size_t b = 0; b < units.size(); ++b) {
    const long long want = std::max(1LL, total > 0 ? slots * units[b] / total : 1LL);
    const long long per = std::max(1LL, (units[b] + want - 1) / want);
    int k = 0;
    for (long long u0 = 0; u0 < units[b]; u0 += per, ++k)
      w.push_back(make_int4((int)b, (int)u0, (int)std::min(u0 + per, units[b]), k));
    (*ctas)[b] = k;
  }
  return w;
}

bool groupable(bsl_handle** hs, int n) {
  if (n < 2) return false;
  for (int b = 0; b < n; ++b) {
    const bsl_handle* h = hs[b];
    if (h->p.device != hs[0]->p.device || h->precision != BSL_PREC_MIXED || h->kinetic_engine != BSL_KIN_TENSOR ||
        (h->vformat != BSL_VFMT_FP32 && h->vformat != BSL_VFMT_GAUNT) || !vstream_group_supported(h->t.nn))
      return false;
  }
  return true;
}

struct GroupedBatch {
  std::vector<bsl_handle*> hs;
  cudaStream_t s = nullptr;
  char* mem = nullptr;  // device: argument tables [stage][parity][problem], then the work tables
  const void* args[4][2] = {};
  const int4* work[4] = {};
  int nctas[4] = {0, 0, 0, 0};
  std::vector<int> upd_ctas;  // per problem: the update's CTAs (block totals of its deferred beta)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~GroupedBatch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (mem) cudaFree(mem);
  }
};

int build_grouped(bsl_handle** hs, int n, GroupedBatch* g) {
  g->hs.assign(hs, hs + n);
  g->s = hs[0]->d.stream;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, hs[0]->p.device);
  sms = std::max(1, sms);
  // stages of the fused iteration: 0 kinetic x/y, 1 kinetic z, 2 light apply
  // (one block of points per CTA), 3 fused update (tiles)
  std::vector<long long> units[4];
  long long light_blocks = 0;
  for (int b = 0; b < n; ++b) {
    int rc;
    if ((rc = ensure_product_buffer(hs[b]))) return rc;
    units[0].push_back(kin_tc_pairs(hs[b], true));
    units[1].push_back(kin_tc_pairs(hs[b], false));
    units[2].push_back((hs[b]->t.npts + light_points_per_cta() - 1) / light_points_per_cta());
    units[3].push_back((hs[b]->t.npts + vstream_tile_points() - 1) / vstream_tile_points());
    light_blocks += units[2].back();
  }
  const int vs = vstream_group_ctas_per_sm();
  const long long slots[4] = {sms, sms, light_blocks,
                              (long long)(hs[0]->tune_vs > 0 && hs[0]->tune_vs < vs ? hs[0]->tune_vs : vs) * sms};
  std::vector<int4> work[4];
  std::vector<int> ctas[4];
  for (int k = 0; k < 4; ++k) {
    work[k] = split_work(units[k], slots[k], &ctas[k]);
    g->nctas[k] = (int)work[k].size();
  }
  const size_t sz[4] = {kin_group_arg_size(), kin_group_arg_size(), vstream_group_arg_size(),
                        vstream_group_arg_size()};
  std::vector<char> host;
  size_t off_args[4][2], off_work[4];
  for (int k = 0; k < 4; ++k)
    for (int p = 0; p < 2; ++p) {
      off_args[k][p] = host.size();
      host.resize(host.size() + (sz[k] * n + 255) / 256 * 256);
    }
  for (int k = 0; k < 4; ++k) {
    off_work[k] = host.size();
    host.resize(host.size() + (work[k].size() * sizeof(int4) + 255) / 256 * 256);
    std::memcpy(host.data() + off_work[k], work[k].data(), work[k].size() * sizeof(int4));
  }
  for (int p = 0; p < 2; ++p) {
    std::vector<const float2*> V(n);
    for (int b = 0; b < n; ++b) V[b] = reinterpret_cast<const float2*>(p ? hs[b]->d.rvec : hs[b]->d.vec);
    kin_tc_group_args(hs, n, V.data(), true, ctas[3].data(), host.data() + off_args[0][p]);
    kin_tc_group_args(hs, n, V.data(), false, nullptr, host.data() + off_args[1][p]);
    for (int b = 0; b < n; ++b) {
      bsl_handle* h = hs[b];
      DeviceState& d = h->d;
      double* Vd = p ? d.rvec : d.vec;
      double* Rd = p ? d.vec : d.rvec;
      StreamArgs a = vstream_args(h, Vd, Rd);
      a.red_count = ctas[2][b];  // the light apply's blocks: alpha's block totals
      std::memcpy(host.data() + off_args[2][p] + sz[2] * b, &a, sizeof(a));
      a.red_count = ctas[3][b];  // the fused update's CTAs: beta's block totals
      std::memcpy(host.data() + off_args[3][p] + sz[3] * b, &a, sizeof(a));
    }
  }
  // every problem's reductions need partials for its CTAs
  for (int b = 0; b < n; ++b)
    if (std::max(ctas[2][b], ctas[3][b]) > hs[b]->d.red_blocks)
      return fail(BSL_ERR_UNSUPPORTED, "grouped batch: more CTAs per problem than reduction slots");
  g->upd_ctas = ctas[3];
  BSL_CUDA(cudaMalloc(&g->mem, host.size()));
  BSL_CUDA(cudaMemcpyAsync(g->mem, host.data(), host.size(), cudaMemcpyHostToDevice, g->s));
  BSL_CUDA(cudaStreamSynchronize(g->s));
  for (int k = 0; k < 4; ++k) {
    for (int p = 0; p < 2; ++p) g->args[k][p] = g->mem + off_args[k][p];
    g->work[k] = reinterpret_cast<const int4*>(g->mem + off_work[k]);
  }
  return BSL_OK;
}

// one iteration of every problem (buffer roles `parity`)
int grouped_iteration(GroupedBatch* g, int parity) {
  int rc;
  if ((rc = launch_kin_tc_group(true, g->args[0][parity], g->work[0], g->nctas[0], g->s)) ||
      (rc = launch_kin_tc_group(false, g->args[1][parity], g->work[1], g->nctas[1], g->s)) ||
      (rc = launch_light_group(g->args[2][parity], g->work[2], g->nctas[2], g->s)) ||
      (rc = launch_vstream_group(g->args[3][parity], g->work[3], g->nctas[3], g->s)))
    return rc;
  return BSL_OK;
}

// niter grouped iterations on the batch stream, timed with the first
// problem's events; problems' start states are set up on their own streams
int run_grouped(bsl_handle** hs, int n, int niter) {
  GroupedBatch g;
  int rc;
  if ((rc = build_grouped(hs, n, &g))) return rc;
  if (niter >= kGraphIters) {
    BSL_CUDA(cudaStreamBeginCapture(g.s, cudaStreamCaptureModeRelaxed));
    for (int i = 0; i < kGraphIters && rc == BSL_OK; ++i) rc = grouped_iteration(&g, i & 1);
    const cudaError_t e = cudaStreamEndCapture(g.s, &g.graph);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (grouped batch)");
    BSL_CUDA(cudaGraphInstantiate(&g.exec, g.graph, 0));
    BSL_CUDA(cudaGraphUpload(g.exec, g.s));
  }
  // the problems' start vectors and counters are ready before the first launch
  cudaEvent_t ready;
  BSL_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  for (int b = 0; b < n; ++b) {
    // the counter and the block product of the start vector
    if ((rc = dev_set_iteration(hs[b], 1, hs[b]->d.stream)) || (rc = dev_begin_iterations(hs[b], hs[b]->d.stream)))
      break;
    if (b > 0) {
      cudaEventRecord(ready, hs[b]->d.stream);
      cudaStreamWaitEvent(g.s, ready, 0);
    }
  }
  cudaEventDestroy(ready);
  if (rc) return rc;
  DeviceState& d0 = hs[0]->d;
  BSL_CUDA(cudaEventRecord(d0.ev0, g.s));
  const int nblocks = niter / kGraphIters;
  for (int k = 0; k < nblocks && rc == BSL_OK; ++k) {
    const cudaError_t e = cudaGraphLaunch(g.exec, g.s);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaGraphLaunch (grouped batch)");
  }
  for (int j = nblocks * kGraphIters; j < niter && rc == BSL_OK; ++j) rc = grouped_iteration(&g, j & 1);
  for (int b = 0; b < n && rc == BSL_OK; ++b) {  // the last iteration's deferred betas
    DeviceState& d = hs[b]->d;
    rc = launch_finish_beta(d.partials, g.upd_ctas[b], d.scalars, d.hist, d.hist_cap, d.jdev, d.status, g.s);
  }
  BSL_CUDA(cudaEventRecord(d0.ev1, g.s));
  const cudaError_t es = cudaStreamSynchronize(g.s);
  if (rc) return rc;
  if (es != cudaSuccess) return cuda_fail(es, "grouped batch");
  float ms = 0.f;
  BSL_CUDA(cudaEventElapsedTime(&ms, d0.ev0, d0.ev1));
  for (int b = 0; b < n; ++b) {
    hs[b]->last_ms_per_iter = ms / niter;
    hs[b]->lanczos_flip = niter & 1;
  }
  return BSL_OK;
}

}  // namespace

void release_iteration_graph(DeviceState& d) {
  if (d.iter_exec) cudaGraphExecDestroy(d.iter_exec);
  if (d.iter_graph) cudaGraphDestroy(d.iter_graph);
  d.iter_exec = nullptr;
  d.iter_graph = nullptr;
  std::memset(d.graph_key, 0, sizeof(d.graph_key));
}

}  // namespace bsl

using namespace bsl;

extern "C" {

int bsl_lanczos_run(bsl_handle* h, int niter, int start, unsigned long long seed, double* alpha, double* beta,
                    double* beta2) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (niter < 1 || !alpha || !beta || !beta2) return fail(BSL_ERR_INPUT, "bad arguments");
  cudaSetDevice(h->p.device);
  DeviceState& d = h->d;
  int rc;
  if ((rc = ensure_hist(h, niter)) || (rc = init_state(h, start, seed))) return rc;
  cudaStream_t s = d.stream;
  if ((rc = prepare_iterations(&h, 1, niter))) return rc;
  BSL_CUDA(cudaEventRecord(d.ev0, s));
  if ((rc = run_iterations(&h, 1, niter))) {
    cudaStreamSynchronize(s);
    return rc;
  }
  BSL_CUDA(cudaEventRecord(d.ev1, s));
  BSL_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  BSL_CUDA(cudaEventElapsedTime(&ms, d.ev0, d.ev1));
  h->last_ms_per_iter = ms / niter;
  std::vector<double> hist(3 * (size_t)d.hist_cap);
  BSL_CUDA(cudaMemcpy(hist.data(), d.hist, hist.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int j = 0; j < niter; ++j) alpha[j] = hist[j];
  beta[0] = 0.0;
  beta2[0] = 0.0;
  for (int j = 1; j <= niter; ++j) {
    beta[j] = hist[d.hist_cap + j];
    beta2[j] = hist[2 * (size_t)d.hist_cap + j];
  }
  return check_status(h);
}

}  // extern "C"

namespace bsl {
namespace {

// bsl_lanczos_run_batch(_streams): grouped launches when `grouped` and the
// problems allow them, else blocks of iterations interleaved across the
// problems' streams
int run_batch(bsl_handle** hs, int n, int niter, int start, unsigned long long seed, double** alpha, double** beta,
              double** beta2, bool grouped) {
  if (!hs || n < 1 || niter < 1 || !alpha || !beta || !beta2) return fail(BSL_ERR_INPUT, "bad arguments");
  for (int b = 0; b < n; ++b) {
    if (!hs[b]) return fail(BSL_ERR_STATE, "null handle in the batch");
    if (!alpha[b] || !beta[b] || !beta2[b]) return fail(BSL_ERR_INPUT, "null output in the batch");
    for (int c = 0; c < b; ++c)
      if (hs[c] == hs[b]) return fail(BSL_ERR_INPUT, "a handle appears twice in the batch");
  }
  int rc;
  for (int b = 0; b < n; ++b) {
    cudaSetDevice(hs[b]->p.device);
    if ((rc = ensure_hist(hs[b], niter)) || (rc = init_state(hs[b], start, seed))) return rc;
  }
  if (grouped && groupable(hs, n)) {
    cudaSetDevice(hs[0]->p.device);
    if ((rc = run_grouped(hs, n, niter))) {
      for (int b = 0; b < n; ++b) cudaStreamSynchronize(hs[b]->d.stream);
      return rc;
    }
  } else {
    // blocks of iterations interleaved across the problems' streams, so the
    // kernels of different problems overlap
    if ((rc = prepare_iterations(hs, n, niter))) return rc;
    for (int b = 0; b < n; ++b) {
      cudaSetDevice(hs[b]->p.device);
      BSL_CUDA(cudaEventRecord(hs[b]->d.ev0, hs[b]->d.stream));
    }
    if ((rc = run_iterations(hs, n, niter))) {
      for (int b = 0; b < n; ++b) cudaStreamSynchronize(hs[b]->d.stream);
      return rc;
    }
    for (int b = 0; b < n; ++b) {
      cudaSetDevice(hs[b]->p.device);
      BSL_CUDA(cudaEventRecord(hs[b]->d.ev1, hs[b]->d.stream));
    }
    // the batch's device time: from the first problem's start to the last end
    // (events of one device compare across streams)
    float batch_ms = 0.f;
    for (int b = 0; b < n; ++b) {
      cudaSetDevice(hs[b]->p.device);
      BSL_CUDA(cudaEventSynchronize(hs[b]->d.ev1));
      float ms = 0.f;
      if (hs[b]->p.device == hs[0]->p.device && cudaEventElapsedTime(&ms, hs[0]->d.ev0, hs[b]->d.ev1) == cudaSuccess)
        batch_ms = ms > batch_ms ? ms : batch_ms;
    }
    for (int b = 0; b < n; ++b) hs[b]->last_ms_per_iter = batch_ms / niter;
  }
  for (int b = 0; b < n; ++b) {
    bsl_handle* h = hs[b];
    cudaSetDevice(h->p.device);
    DeviceState& d = h->d;
    BSL_CUDA(cudaStreamSynchronize(d.stream));
    std::vector<double> hist(3 * (size_t)d.hist_cap);
    BSL_CUDA(cudaMemcpy(hist.data(), d.hist, hist.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int j = 0; j < niter; ++j) alpha[b][j] = hist[j];
    beta[b][0] = 0.0;
    beta2[b][0] = 0.0;
    for (int j = 1; j <= niter; ++j) {
      beta[b][j] = hist[d.hist_cap + j];
      beta2[b][j] = hist[2 * (size_t)d.hist_cap + j];
    }
    if ((rc = check_status(h))) return rc;
  }
  return BSL_OK;
}

}  // namespace
}  // namespace bsl

extern "C" {

int bsl_lanczos_run_batch(bsl_handle** hs, int n, int niter, int start, unsigned long long seed, double** alpha,
                          double** beta, double** beta2) {
  return run_batch(hs, n, niter, start, seed, alpha, beta, beta2, true);
}

int bsl_lanczos_run_batch_streams(bsl_handle** hs, int n, int niter, int start, unsigned long long seed,
                                  double** alpha, double** beta, double** beta2) {
  return run_batch(hs, n, niter, start, seed, alpha, beta, beta2, false);
}

int bsl_autotune(bsl_handle** hs, int n, int iters, int* vs_per_sm, int* upd_per_sm, double* ms_per_iter) {
  if (!hs || n < 1 || iters < 8) return fail(BSL_ERR_INPUT, "bad arguments");
  for (int b = 0; b < n; ++b)
    if (!hs[b]) return fail(BSL_ERR_STATE, "null handle");
  // the choice is cached for the same problem set (block sizes, grids, formats)
  std::string key = std::to_string(n);
  for (int b = 0; b < n; ++b) {
    const bsl_handle* h = hs[b];
    key += "|" + std::to_string(h->t.nn) + ":" + std::to_string(h->t.nx) + "x" + std::to_string(h->t.ny) + "x" +
           std::to_string(h->t.nz) + ":" + std::to_string(h->precision) + ":" + std::to_string(h->kinetic_engine) +
           ":" + std::to_string(h->vformat) + ":" + std::to_string(h->kin_slices);
  }
  static std::mutex mu;
  static std::map<std::string, std::array<double, 3>> cache;
  std::array<double, 3> best = {0, 0, 1e300};
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) best = it->second;
  }
  if (best[2] >= 1e300) {
    const int wv = iters + 1;
    std::vector<double> a((size_t)n * wv), bb((size_t)n * (wv + 1)), b2((size_t)n * (wv + 1));
    std::vector<double*> pa(n), pb(n), pb2(n);
    for (int b = 0; b < n; ++b) {
      pa[b] = a.data() + (size_t)b * wv;
      pb[b] = bb.data() + (size_t)b * (wv + 1);
      pb2[b] = b2.data() + (size_t)b * (wv + 1);
    }
    // the update's shape matters only where a problem runs the streamed update
    // (the fused iteration and the grouped batch do not use it): there it is
    // timed too, elsewhere it stays at the default 2
    bool upd_matters = false;
    if (!(n > 1 && groupable(hs, n)))
      for (int b = 0; b < n; ++b) {
        const bsl_handle* h = hs[b];
        if (!(h->precision == BSL_PREC_MIXED && h->kinetic_engine == BSL_KIN_TENSOR &&
              fused_update_supported(h->vformat, h->t.nn)))
          upd_matters = true;
      }
    const int up_lo = upd_matters ? 1 : 2, up_hi = upd_matters ? 3 : 2;
    for (int vs = 1; vs <= 3; ++vs)
      for (int up = up_lo; up <= up_hi; ++up) {
        for (int b = 0; b < n; ++b) {
          hs[b]->tune_vs = vs;
          hs[b]->tune_upd = up;
        }
        int rc = BSL_OK;
        for (int rep = 0; rep < 2 && rc == BSL_OK; ++rep)  // the first run captures the graphs
          rc = n == 1 ? bsl_lanczos_run(hs[0], iters, BSL_START_UNIFORM, 0, pa[0], pb[0], pb2[0])
                      : run_batch(hs, n, iters, BSL_START_UNIFORM, 0, pa.data(), pb.data(), pb2.data(), true);
        if (rc) return rc;
        const double ms = hs[0]->last_ms_per_iter;
        if (ms < best[2]) best = {(double)vs, (double)up, ms};
      }
    std::lock_guard<std::mutex> lock(mu);
    cache[key] = best;
  }
  for (int b = 0; b < n; ++b) {
    hs[b]->tune_vs = (int)best[0];
    hs[b]->tune_upd = (int)best[1];
  }
  if (vs_per_sm) *vs_per_sm = (int)best[0];
  if (upd_per_sm) *upd_per_sm = (int)best[1];
  if (ms_per_iter) *ms_per_iter = best[2];
  return BSL_OK;
}

int bsl_lanczos_step_host(bsl_handle* h, double* vec, double* rvec, double* alpha_j, double* beta_j,
                          double* beta2_j) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (!vec || !rvec) return fail(BSL_ERR_INPUT, "null argument");
  cudaSetDevice(h->p.device);
  DeviceState& d = h->d;
  int rc;
  if ((rc = ensure_hist(h, 1)) || (rc = ensure_staging(h))) return rc;
  const size_t Df = (size_t)bsl_basis_size(h);
  cudaStream_t s = d.stream;
  // vec feeds H v at once; rvec is copied in on a second stream while H v runs
  // and only waited for where r += H v needs it.  The rvec copy starts after
  // the vec copy has finished: both share the host link's bandwidth in one
  // direction, and running them side by side would delay H v until both had
  // arrived.
  BSL_CUDA(cudaMemcpyAsync(d.ref_vec, vec, Df * sizeof(double), cudaMemcpyHostToDevice, s));
  BSL_CUDA(cudaEventRecord(d.vec_in, s));
  BSL_CUDA(cudaStreamWaitEvent(d.copy_stream, d.vec_in, 0));
  BSL_CUDA(cudaMemcpyAsync(d.ref_out, rvec, Df * sizeof(double), cudaMemcpyHostToDevice, d.copy_stream));
  BSL_CUDA(cudaEventRecord(d.copy_done, d.copy_stream));
  if ((rc = reset_status(h, s))) return rc;
  // r += S H v: H on the packed block, nothing elsewhere (the device Lanczos
  // vectors serve as packed scratch)
  h->state_pairs = -1;
  if ((rc = dev_hv_full(h, d.ref_vec, d.rvec, s))) return rc;
  BSL_CUDA(cudaStreamWaitEvent(s, d.copy_done, 0));
  // page-locked caller buffers are written by the last pass itself; others by copies
  double* vec_d = mapped_host(vec);
  double* rvec_d = vec_d ? mapped_host(rvec) : nullptr;
  if (vec_d && rvec_d) {
    if ((rc = dev_full_step_fused(h, d.ref_vec, d.ref_out, (long long)Df, d.rvec, 1, s, vec_d, rvec_d))) return rc;
  } else {
    if ((rc = dev_full_step_fused(h, d.ref_vec, d.ref_out, (long long)Df, d.rvec, 1, s))) return rc;
    BSL_CUDA(cudaMemcpyAsync(vec, d.ref_vec, Df * sizeof(double), cudaMemcpyDeviceToHost, s));
    BSL_CUDA(cudaMemcpyAsync(rvec, d.ref_out, Df * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  double sc[3];
  BSL_CUDA(cudaMemcpyAsync(sc, d.scalars, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  BSL_CUDA(cudaStreamSynchronize(s));
  if (alpha_j) *alpha_j = sc[0];
  if (beta_j) *beta_j = sc[1];
  if (beta2_j) *beta2_j = sc[2];
  return check_status(h);
}

int bsl_ritz_vectors(bsl_handle* h, int niter, const double* evtr, int ngood, double* ritz) {
  return bsl_ritz_vectors_start(h, niter, BSL_START_UNIFORM, 0, evtr, ngood, ritz);
}

int bsl_ritz_vectors_start(bsl_handle* h, int niter, int start, unsigned long long seed, const double* evtr, int ngood,
                           double* ritz) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (niter < 1 || ngood < 1 || !evtr || !ritz) return fail(BSL_ERR_INPUT, "bad arguments");
  cudaSetDevice(h->p.device);
  DeviceState& d = h->d;
  const long long D = bsl_packed_size(h), Df = bsl_basis_size(h), L = D + 1;
  int rc;
  if ((rc = ensure_hist(h, niter)) || (rc = init_state(h, start, seed))) return rc;
  // coefficient schedule with the reference's cumulative-norm cut-off
  std::vector<double> coef((size_t)niter * ngood);
  std::vector<int> active((size_t)niter * ngood);
  std::vector<double> cum(ngood, 0.0);
  for (int j = 1; j <= niter; ++j)
    for (int n = 0; n < ngood; ++n) {
      const double c = evtr[(size_t)n * niter + (j - 1)];
      cum[n] += std::pow(c, 2.);
      coef[(size_t)(j - 1) * ngood + n] = c;
      active[(size_t)(j - 1) * ngood + n] = (cum[n] < (1. - 1.e-16)) ? 1 : 0;
    }
  double* dcoef = nullptr;
  int* dact = nullptr;
  double* dritz = nullptr;
  auto cleanup = [&]() {
    cudaFree(dcoef);
    cudaFree(dact);
    cudaFree(dritz);
  };
  cudaError_t e;
  if ((e = cudaMalloc(&dcoef, coef.size() * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&dact, active.size() * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&dritz, (size_t)ngood * L * sizeof(double))) != cudaSuccess) {
    cleanup();
    return fail(BSL_ERR_NOMEM, std::string("Ritz buffers: ") + cudaGetErrorString(e));
  }
  cudaStream_t s = d.stream;
  cudaMemcpyAsync(dcoef, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dact, active.data(), active.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(dritz, 0, (size_t)ngood * L * sizeof(double), s);
  // The iterations regenerate loop 1's vectors with loop 1's kernels: where
  // bsl_lanczos_run counts iterations on the device (deferred reductions, the
  // fused update), v_j and its scale are complete only once iteration j's x/y
  // kinetic has finished the previous beta, so v_j is taken after iteration j
  // (it is that iteration's V, unchanged by it).
  const bool counted = device_counted_iterations(h);
  if (counted && ((rc = ensure_product_buffer(h)) || (rc = dev_set_iteration(h, 1, s)) ||
                  (rc = dev_begin_iterations(h, s)))) {
    cleanup();
    return rc;
  }
  for (int j = 1; j <= niter; ++j) {
    const double* cj = dcoef + (size_t)(j - 1) * ngood;
    const int* aj = dact + (size_t)(j - 1) * ngood;
    if (counted) {
      rc = dev_lanczos_iteration(h, 0, s);
      if (!rc) rc = dev_ritz_accumulate(h, cj, aj, ngood, dritz, s, true);
    } else {
      rc = dev_ritz_accumulate(h, cj, aj, ngood, dritz, s, false);
      if (!rc) rc = dev_lanczos_iteration(h, j, s);
    }
    if (rc) {
      cleanup();
      return rc;
    }
  }
  if (counted && (rc = dev_finish_iterations(h, s))) {
    cleanup();
    return rc;
  }
  std::vector<double> host((size_t)ngood * L);
  e = cudaMemcpyAsync(host.data(), dritz, host.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "Ritz vectors");
  const Tables& t = h->t;
  const long long N = t.npts;
  const double off = (Df > D) ? 1.0 / std::sqrt((double)(Df - D)) : 0.0;
  for (int n = 0; n < ngood; ++n) {
    double* out = ritz + (size_t)n * Df;
    const double* in = host.data() + (size_t)n * L;
    const double masked = in[D] * off;
    for (long long i = 0; i < Df; ++i) out[i] = masked;
    for (int sidx = 0; sidx < t.nn; ++sidx)
      std::memcpy(out + (size_t)t.full_of[sidx] * N, in + (size_t)sidx * N, N * sizeof(double));
  }
  return check_status(h);
}

}  // extern "C"

extern "C" {

int bsl_stage_times(bsl_handle* h, int iters, double* ms, const char** names) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (iters < 1 || !ms) return fail(BSL_ERR_INPUT, "bad arguments");
  cudaSetDevice(h->p.device);
  DeviceState& d = h->d;
  int rc;
  if ((rc = ensure_hist(h, iters))) return rc;
  // the state must match the current precision's buffer format
  if (h->state_pairs != (h->precision == BSL_PREC_MIXED ? 1 : 0) && (rc = init_state(h, BSL_START_UNIFORM, 0)))
    return rc;
  cudaEvent_t ev[6];
  for (int i = 0; i < 6; ++i) BSL_CUDA(cudaEventCreate(&ev[i]));
  const int nst = 4;
  double acc[5] = {0, 0, 0, 0, 0};
  // device-counted iterations are timed as they run in a Lanczos run (reductions deferred)
  const bool counted = device_counted_iterations(h);
  if (counted && ((rc = dev_set_iteration(h, 1, d.stream)) || (rc = dev_begin_iterations(h, d.stream)))) return rc;
  for (int j = 1; j <= iters && !rc; ++j) {
    rc = dev_lanczos_iteration_timed(h, counted ? 0 : j, d.stream, ev);
    if (rc) break;
    cudaError_t e = cudaEventSynchronize(ev[nst]);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "stage timing");
      break;
    }
    for (int i = 0; i < nst; ++i) {
      float x = 0.f;
      cudaEventElapsedTime(&x, ev[i], ev[i + 1]);
      acc[i] += x;
    }
  }
  if (!rc && counted) rc = dev_finish_iterations(h, d.stream);
  for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
  if (rc) return rc;
  for (int i = 0; i < 5; ++i) {
    ms[i] = i < nst ? acc[i] / iters : 0.0;
    if (names) names[i] = i < nst ? dev_stage_name(h, i) : "";
  }
  return check_status(h);
}

int bsl_launches_per_iteration(const bsl_handle* h) { return h ? 4 : -1; }

int bsl_debug_inject_timeout(bsl_handle* h, int kernel_mask) {
  if (!h) return fail(BSL_ERR_STATE, "null handle");
  if (kernel_mask & ~3) return fail(BSL_ERR_INPUT, "kernel_mask has bits other than 0 and 1");
  h->d.inject_status = ((kernel_mask & 1) ? (1 << 2) : 0) | ((kernel_mask & 2) ? (1 << 3) : 0);
  return BSL_OK;
}

}  // extern "C"
