// Self-test of the tcgen05 plumbing on the current device: one 128 x 64 x 64
// kind::tf32 product from 128-byte-swizzled shared-memory operands into tensor
// memory, read back and compared with the exact result (the operands are small
// multiples of powers of two, so every product and sum is exact in FP32).
#include "bsl_tc.cuh"

namespace bsl {
namespace {

__device__ __forceinline__ float st_a(int m, int k) { return (float)(((m * 7 + k * 3) % 17) - 8) * 0.0625f; }
__device__ __forceinline__ float st_b(int n, int k) { return (float)(((n * 5 + k * 11) % 13) - 6) * 0.125f; }

__global__ void __launch_bounds__(128) k_tc_selftest(float* max_err, int* status) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
  uint8_t* A = sm;               // 128 x 64, 32 KiB
  uint8_t* B = sm + 128 * 256;   // 64 x 64, 16 KiB
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int e = tid; e < 128 * 64; e += blockDim.x) {
    const int r = e >> 6, k = e & 63;
    *reinterpret_cast<float*>(A + tc::sw128_offset(r, k, 128)) = st_a(r, k);
  }
  for (int e = tid; e < 64 * 64; e += blockDim.x) {
    const int r = e >> 6, k = e & 63;
    *reinterpret_cast<float*>(B + tc::sw128_offset(r, k, 64)) = st_b(r, k);
  }
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 64);
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_tf32(128, 64);
    const uint32_t a0 = tc::smem_u32(A), b0 = tc::smem_u32(B);
    for (int s = 0; s < 8; ++s) {
      const uint32_t ka = (uint32_t)((s >> 2) * 128 * 128 + (s & 3) * 32);
      const uint32_t kb = (uint32_t)((s >> 2) * 64 * 128 + (s & 3) * 32);
      tc::mma_tf32(tmem, tc::sw128_desc(a0 + ka), tc::sw128_desc(b0 + kb), idesc, s > 0 ? 1u : 0u);
    }
    tc::mma_commit(&bar);
  }
  const bool ok = tc::mbar_wait(&bar, 0);
  if (!ok && tid == 0) status[0] = 1;
  tc::fence_after_sync();
  float err = 0.f;
  if (ok) {
    const int m = tid;  // lane of this thread
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float d[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, d);
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        float ref = 0.f;
        for (int k = 0; k < 64; ++k) ref += st_a(m, k) * st_b(c0 + c, k);
        err = fmaxf(err, fabsf(d[c] - ref));
      }
    }
  }
  atomicMax(reinterpret_cast<int*>(max_err), __float_as_int(err));
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

}  // namespace
}  // namespace bsl

using namespace bsl;

extern "C" int bsl_selftest_tensor_core(double* max_abs_err) {
  if (!max_abs_err) return fail(BSL_ERR_INPUT, "null argument");
  float* d_err = nullptr;
  int* d_status = nullptr;
  BSL_CUDA(cudaMalloc(&d_err, sizeof(float)));
  BSL_CUDA(cudaMalloc(&d_status, sizeof(int)));
  cudaMemset(d_err, 0, sizeof(float));
  cudaMemset(d_status, 0, sizeof(int));
  const size_t smem = 128 * 256 + 64 * 256 + 1024;
  cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_tc_selftest<<<1, 128, smem>>>(d_err, d_status);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  float err = -1.f;
  int st = 0;
  if (e == cudaSuccess) {
    cudaMemcpy(&err, d_err, sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost);
  }
  cudaFree(d_err);
  cudaFree(d_status);
  if (e != cudaSuccess) return cuda_fail(e, "tensor-core self-test");
  if (st) return fail(BSL_ERR_CUDA, "tensor-core self-test: the MMA did not complete within its time limit");
  *max_abs_err = err;
  return BSL_OK;
}
