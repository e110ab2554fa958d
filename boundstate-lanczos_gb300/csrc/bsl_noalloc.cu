// Lanczos orthonormalisation step that allocates nothing: the reduction
// scratch (per-block partial sums, the scalars and the completion counter)
// lives in one file-scope static device array instead of memory obtained from
// cudaMalloc, so callers that cannot allocate device memory can still run the
// recurrence on buffers they own.  See bsl_lanczos_orthonormalize_static in
// include/bsl.h for the contract.
#include <mutex>

#include "bsl_device.cuh"

namespace bsl {
namespace {

constexpr int kNaBlocks = 4096;     // partial sums held in the static scratch
constexpr int kNaPerThread = 8;     // elements per thread, no grid-stride loop
constexpr long long kNaTile = (long long)kThreads * kNaPerThread;  // 2048 elements per block
constexpr long long kNaMaxN = (long long)kNaBlocks * kNaTile;      // 8,388,608 elements
constexpr int kNaScalars = kNaBlocks;       // [alpha, beta, beta^2, 1/beta]
constexpr int kNaCounter = kNaBlocks + 8;   // completion counter (unsigned int bits)
constexpr int kNaDoubles = kNaBlocks + 16;  // 32.9 KB in total

// Shared by every call on a device; keeps the last call's contents.
static __device__ __align__(256) double g_na_scratch[kNaDoubles];

__global__ void k_na_dot(const double* __restrict__ v, const double* __restrict__ r, long long n, double* scratch) {
  double acc = 0.0;
  const long long base = (long long)blockIdx.x * kNaTile + threadIdx.x;
#pragma unroll
  for (int u = 0; u < kNaPerThread; ++u) {
    const long long i = base + (long long)u * kThreads;
    if (i < n) acc += v[i] * r[i];
  }
  double total;
  unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kNaCounter);
  if (reduce_grid(acc, scratch, counter, &total) && threadIdx.x == 0) scratch[kNaScalars] = total;
}

__global__ void k_na_update(const double* __restrict__ v, double* __restrict__ r, long long n, double* scratch) {
  const double alpha = scratch[kNaScalars];
  double acc = 0.0;
  const long long base = (long long)blockIdx.x * kNaTile + threadIdx.x;
#pragma unroll
  for (int u = 0; u < kNaPerThread; ++u) {
    const long long i = base + (long long)u * kThreads;
    if (i < n) {
      const double x = r[i] - alpha * v[i];
      r[i] = x;
      acc += x * x;
    }
  }
  double total;
  unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kNaCounter);
  if (reduce_grid(acc, scratch, counter, &total) && threadIdx.x == 0) {
    const double b = sqrt(total);
    scratch[kNaScalars + 1] = b;
    scratch[kNaScalars + 2] = total;
    scratch[kNaScalars + 3] = 1. / b;
  }
}

// v <- r / beta, r <- -beta v (the reference's scale then swap), and the
// scalars to the caller's buffer
__global__ void k_na_swap(double* __restrict__ v, double* __restrict__ r, long long n, const double* scratch,
                          double* abb) {
  const double b = scratch[kNaScalars + 1], inv = scratch[kNaScalars + 3];
  const long long base = (long long)blockIdx.x * kNaTile + threadIdx.x;
#pragma unroll
  for (int u = 0; u < kNaPerThread; ++u) {
    const long long i = base + (long long)u * kThreads;
    if (i < n) {
      const double vi = v[i];
      v[i] = inv * r[i];
      r[i] = (-b) * vi;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    abb[0] = scratch[kNaScalars];
    abb[1] = b;
    abb[2] = scratch[kNaScalars + 2];
  }
}

// Device address of the scratch array, looked up once per device with that
// device current (host code must not pass the symbol itself to a kernel).
std::mutex g_na_mutex;
double* g_na_ptr[64] = {nullptr};

int scratch_for_current_device(double** out) {
  int dev = 0;
  BSL_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(BSL_ERR_UNSUPPORTED, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static Lanczos scratch)");
    g_na_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_na_ptr[dev];
  return BSL_OK;
}

}  // namespace
}  // namespace bsl

using namespace bsl;

extern "C" int bsl_lanczos_orthonormalize_static(double* d_vec, double* d_rvec, long long n, double* d_abb,
                                                 void* stream) {
  if (!d_vec || !d_rvec || !d_abb) return fail(BSL_ERR_INPUT, "null device pointer");
  if (n < 1 || n > kNaMaxN)
    return fail(BSL_ERR_INPUT, "vector length " + std::to_string(n) +
                                   " is outside the static scratch capacity of 1.." + std::to_string(kNaMaxN));
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  // the counter must start at zero; a previous call that failed part-way may
  // have left it set
  BSL_CUDA(cudaMemsetAsync(scratch + kNaCounter, 0, sizeof(double), s));
  const unsigned int blocks = (unsigned int)((n + kNaTile - 1) / kNaTile);
  k_na_dot<<<blocks, kThreads, 0, s>>>(d_vec, d_rvec, n, scratch);
  k_na_update<<<blocks, kThreads, 0, s>>>(d_vec, d_rvec, n, scratch);
  k_na_swap<<<blocks, kThreads, 0, s>>>(d_vec, d_rvec, n, scratch, d_abb);
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}
