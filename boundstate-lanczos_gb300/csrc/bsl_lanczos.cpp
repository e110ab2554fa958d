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
constexpr int kGraphIters = 8;

// capture kGraphIters device-counted iterations of h on its stream (nothing
// runs) unless the cached graph already matches the current configuration
int ensure_iteration_graph(bsl_handle* h) {
  DeviceState& d = h->d;
  const long long key[7] = {h->precision, h->kinetic_engine, h->lanczos_flip, (long long)(uintptr_t)d.hist,
                            d.hist_cap, h->kin_slices, h->vformat};
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
    if (device_counted_iterations(h) && niter >= kGraphIters && (rc = ensure_iteration_graph(h))) return rc;
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
    if (counted[b] && (rc = dev_set_iteration(h, 1, h->d.stream))) return rc;
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

int bsl_lanczos_run_batch(bsl_handle** hs, int n, int niter, int start, unsigned long long seed, double** alpha,
                          double** beta, double** beta2) {
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
  for (int j = 1; j <= niter; ++j) {
    rc = dev_ritz_accumulate(h, dcoef + (size_t)(j - 1) * ngood, dact + (size_t)(j - 1) * ngood, ngood, dritz, s);
    if (!rc) rc = dev_lanczos_iteration(h, j, s);
    if (rc) {
      cleanup();
      return rc;
    }
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
  for (int j = 1; j <= iters && !rc; ++j) {
    rc = dev_lanczos_iteration_timed(h, j, d.stream, ev);
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
