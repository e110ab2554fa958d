// Lanczos orthonormalisation step that allocates nothing: the reduction
// scratch (per-block partial sums, the scalars and the completion counter)
// lives in one file-scope static device array instead of memory obtained from
// cudaMalloc, so callers that cannot allocate device memory can still run the
// recurrence on buffers they own.  See bsl_lanczos_orthonormalize_static in
// include/bsl.h for the contract.
#include <cstdint>
#include <mutex>
#include <string>

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
    // a zero or non-finite beta (or alpha) is a breakdown: 1/beta = 0 tells the
    // next kernel to leave both vectors as they are
    const bool ok = b > 0.0 && isfinite(b) && isfinite(alpha);
    scratch[kNaScalars + 3] = ok ? 1. / b : 0.0;
  }
}

// v <- r / beta, r <- -beta v (the reference's scale then swap), and the
// scalars to the caller's buffer; nothing is moved after a breakdown
__global__ void k_na_swap(double* __restrict__ v, double* __restrict__ r, long long n, const double* scratch,
                          double* abb) {
  const double b = scratch[kNaScalars + 1], inv = scratch[kNaScalars + 3];
  if (inv != 0.0) {
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
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    abb[0] = scratch[kNaScalars];
    abb[1] = b;
    abb[2] = scratch[kNaScalars + 2];
  }
}

// Device address of the scratch array in the calling thread's current CUDA
// context.  A symbol's device address belongs to a context, not to a device
// ordinal: after cudaDeviceReset, or under another context on the same
// device, an address looked up earlier is stale.  The cache is therefore keyed
// by the context's unique id (cuCtxGetId, reached through the runtime's driver
// entry points so that the library does not link the driver library), and a
// context seen for the first time pays one cudaGetSymbolAddress.  Where the
// id cannot be read, the address is looked up on every call.  Host code must
// not pass the symbol itself to a kernel: in host code it names a host-side
// stand-in, not device memory.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

struct CtxEntry {
  unsigned long long id;
  double* ptr;
};

std::mutex g_na_mutex;
constexpr int kNaCacheSlots = 16;
CtxEntry g_na_cache[kNaCacheSlots] = {};
int g_na_next = 0;
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
bool g_ctx_resolved = false;

// the current context's id, or 0 when it cannot be read
unsigned long long current_context_id() {
  if (!g_ctx_resolved) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
      g_ctx_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    cudaGetLastError();
    g_ctx_resolved = true;
  }
  if (!g_ctx_current || !g_ctx_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_current(&ctx) != 0 || !ctx || g_ctx_id(ctx, &id) != 0) return 0;
  return id;
}

int scratch_for_current_context(double** out) {
  std::lock_guard<std::mutex> lock(g_na_mutex);
  unsigned long long id = current_context_id();
  if (id != 0)
    for (const CtxEntry& e : g_na_cache)
      if (e.id == id) {
        *out = e.ptr;
        return BSL_OK;
      }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static Lanczos scratch)");
  if (id == 0) id = current_context_id();  // the lookup made the device's primary context current
  if (id != 0) {
    g_na_cache[g_na_next] = CtxEntry{id, static_cast<double*>(p)};
    g_na_next = (g_na_next + 1) % kNaCacheSlots;
  }
  *out = static_cast<double*>(p);
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
  // the kernels read v and write r through restrict-qualified pointers
  const uintptr_t v0 = reinterpret_cast<uintptr_t>(d_vec), r0 = reinterpret_cast<uintptr_t>(d_rvec);
  const uintptr_t bytes = (uintptr_t)n * sizeof(double);
  if (v0 < r0 + bytes && r0 < v0 + bytes) return fail(BSL_ERR_INPUT, "d_vec and d_rvec overlap");
  const uintptr_t a0 = reinterpret_cast<uintptr_t>(d_abb);
  if ((a0 < v0 + bytes && v0 < a0 + 3 * sizeof(double)) || (a0 < r0 + bytes && r0 < a0 + 3 * sizeof(double)))
    return fail(BSL_ERR_INPUT, "d_abb overlaps d_vec or d_rvec");
  double* scratch = nullptr;
  int rc = scratch_for_current_context(&scratch);
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
