// Mixed-precision potential apply: the FP32 potential blocks are streamed from
// HBM with bulk asynchronous copies (cp.async.bulk, completion on an
// mbarrier) through a multi-stage shared-memory ring, so each CTA keeps
// tens of kilobytes in flight with one issuing thread.
//
// Reference: Vv_5D_oneCompositeIndex_NoQuad and the Hv sum/mask,
// Hv-calculators/linRotor/cartSphBasis/HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:675-796.
//
// Block layout (written by the block assembly): tile-major
//   vbt[tile][t][p_local], tile = p / kTilePts, t over s <= s' row by row,
// so one tile's ntri x kTilePts floats are contiguous and a chunk of kChunk
// rows is one contiguous copy of kChunk * 512 bytes.
//
// One CTA per tile of 128 grid points, one thread per point:
//   u(s) = ukin(s) + B l(l+1) v(s) + sum_s' V_ss' v(s')   (FP32 block product, FP32-pair sums)
//   mode 0: out = u (FP64);   mode 1: R += c u (FP64), partial alpha = V . R (deterministic grid reduction)
#include "bsl_device.cuh"

namespace bsl {
namespace {

constexpr int kTilePts = 128;
constexpr int kChunk = 16;    // block rows per copy (8 KiB)
constexpr int kStages = 4;    // ring depth (32 KiB of shared memory)
constexpr long long kSpinCycles = 1000000000ll;  // ~0.5 s at 2 GHz: bound on every wait

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait; false if the limit was reached
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > kSpinCycles) return false;
  return true;
}

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

template <int NN>
__global__ void __launch_bounds__(kTilePts) k_vstream(const StreamArgs A) {
  constexpr int NT = NN * (NN + 1) / 2;
  constexpr int NCH = (NT + kChunk - 1) / kChunk;
  extern __shared__ float4 ring4[];
  float* ring = reinterpret_cast<float*>(ring4);  // [kStages][kChunk][kTilePts]
  __shared__ uint64_t full[kStages];
  __shared__ int abort_flag, issued;
  const int tid = threadIdx.x;
  const long long tile = blockIdx.x;
  const long long npts = A.npts;
  const float* src_tile = A.vb + tile * (long long)NT * kTilePts;
  if (tid == 0) {
    // a stream that already timed out in an earlier launch disables the copies
    // (and every wait) of later launches until the host has seen the error
    abort_flag = *(volatile int*)(A.status + 2);
    issued = 0;
    for (int s = 0; s < kStages; ++s) mbar_init(&full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int c) {
    const int st = c % kStages;
    const int rows = (c == NCH - 1) ? (NT - c * kChunk) : kChunk;
    const uint32_t bytes = (uint32_t)rows * kTilePts * sizeof(float);
    mbar_expect_tx(&full[st], bytes);
    issued = c + 1;
    bulk_copy(ring + (size_t)st * kChunk * kTilePts, src_tile + (size_t)c * kChunk * kTilePts, bytes, &full[st]);
  };
  if (tid == 0 && !abort_flag)
    for (int c = 0; c < NCH && c < kStages; ++c) issue(c);

  const long long p = tile * kTilePts + tid;
  const bool valid = p < npts;
  if (valid) {
#pragma unroll
    for (int s = 0; s < NN; ++s) {
      asm volatile("prefetch.global.L2 [%0];" ::"l"(A.ukin + s * npts + p));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(A.out + s * npts + p));
    }
  }
  float vv[NN], va[NN];
#pragma unroll
  for (int s = 0; s < NN; ++s) {
    vv[s] = valid ? A.v32[s * npts + p] : 0.f;
    va[s] = 0.f;
  }
  int t = 0;
#pragma unroll
  for (int s = 0; s < NN; ++s) {
#pragma unroll
    for (int q = s; q < NN; ++q, ++t) {
      const int c = t / kChunk;
      const int st = c % kStages;
      if (t % kChunk == 0) {
        if (!abort_flag && !mbar_wait(&full[st], (uint32_t)((c / kStages) & 1))) abort_flag = 1;
      }
      const float x = ring[((size_t)st * kChunk + (t % kChunk)) * kTilePts + tid];
      va[s] = fmaf(x, vv[q], va[s]);
      if (q != s) va[q] = fmaf(x, vv[s], va[q]);
      if (t % kChunk == kChunk - 1 || t == NT - 1) {
        __syncthreads();  // every thread is done with this stage
        if (tid == 0 && !abort_flag && c + kStages < NCH) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue(c + kStages);
        }
      }
    }
  }
  // u = kinetic pair + B l(l+1) v + V v as an FP32 pair, then one FP64 value.
  // mode 1: the logical vectors are v = sv V and r = sr R; r + H v is kept as
  // sr (R + (sv/sr) H V), so R' = R + c H V and alpha = sv sr (V . R').
  const double c = A.mode ? A.scalars[6] : 1.0;
  double dot = 0.0;
  if (valid) {
#pragma unroll
    for (int s = 0; s < NN; ++s) {
      const float2 uk = A.ukin[s * npts + p];
      const float a = fmaf(__ldg(A.rot_hi + s), vv[s], va[s]);
      float hi, e;
      two_sum(uk.x, a, hi, e);
      const float lo = uk.y + e + __ldg(A.rot_lo + s) * vv[s];
      const double hv = f64_of(hi) + f64_of(lo);
      if (A.mode == 0) {
        A.out[s * npts + p] = hv;
      } else {
        const double r = fma(c, hv, A.out[s * npts + p]);
        A.out[s * npts + p] = r;
        dot = fma(A.vec[s * npts + p], r, dot);
      }
    }
  }
  if (abort_flag && tid == 0 && issued > 0) {
    // a copy did not complete in time: record it and give the copies still in
    // flight a bounded chance to land before the CTA's shared memory is released
    A.status[2] = 1;
    for (int cc = issued - kStages; cc < issued; ++cc)
      if (cc >= 0) mbar_wait(&full[cc % kStages], (uint32_t)((cc / kStages) & 1));
  }
  if (A.mode == 1) {
    if (p == 0) dot = fma(A.vec[A.dpk], A.out[A.dpk], dot);  // extra coordinate: H acts as 0, R' = R
    double total;
    if (reduce_grid(dot, A.partials, A.counter, &total) && threadIdx.x == 0) {
      const double alpha = A.scalars[7] * total;
      A.scalars[0] = alpha;
      A.hist[A.j - 1] = alpha;
    }
  }
}

template <int NN>
int launch_nn(const StreamArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)kStages * kChunk * kTilePts * sizeof(float);
  cudaFuncSetAttribute(k_vstream<NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const long long tiles = (a.npts + kTilePts - 1) / kTilePts;
  k_vstream<NN><<<(unsigned)tiles, kTilePts, smem, s>>>(a);
  return BSL_OK;
}

}  // namespace

long long vstream_tile_points() { return kTilePts; }

int launch_vapply_f32(const StreamArgs& a, int nn, cudaStream_t s) {
#define BSL_CASE(K)      \
  case K:                \
    launch_nn<K>(a, s);  \
    break;
  switch (nn) {
    BSL_CASE(1)
    BSL_CASE(3)
    BSL_CASE(4)
    BSL_CASE(6)
    BSL_CASE(9)
    BSL_CASE(10)
    BSL_CASE(15)
    BSL_CASE(16)
    BSL_CASE(21)
    BSL_CASE(25)
    BSL_CASE(28)
    BSL_CASE(36)
    default:
      return fail(BSL_ERR_UNSUPPORTED, "mixed precision needs a block size with a specialised kernel");
  }
#undef BSL_CASE
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace bsl
