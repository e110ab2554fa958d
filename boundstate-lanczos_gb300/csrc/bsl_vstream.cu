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
// A precision variant streams BF16 blocks in the same layout (each point's
// elements divided by its largest |element|, kept as one FP32 scale per point):
// 32 rows per 8 KiB copy, the block product scaled once per point.
//
// One thread per grid point of a tile of 128 points:
//   u(s) = ukin(s) + B l(l+1) v(s) + sum_s' V_ss' v(s')   (FP32 block product, FP32-pair sums)
//   mode 0: out = u (FP64);   mode 1: R += c u (FP64), partial alpha = V . R (deterministic grid reduction);
//   mode 2: mode 1 with V and R as double-float pairs
//
// The iterations of a Lanczos run (graph-replayed, the fused iteration) split
// this differently: the update streams the potential and forms the block
// product of the next v while that v is in registers (role 1 of vstream_body),
// and the next iteration's H v apply is element-wise (k_vapply_light).  The
// double-float Lanczos update of the four-kernel iteration (k_update_stream)
// and the closing kernel of the deferred beta are here too.
#include <cuda_bf16.h>

#include <type_traits>

#include "bsl_device.cuh"
#include "bsl_gaunt.h"

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

// L2 policy for the block stream: read once per iteration, so evicted first and
// the Lanczos vectors (about 90 MB at 54^3) have the best chance to stay in L2
__device__ __forceinline__ uint64_t evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

__device__ __forceinline__ void bulk_copy_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                               uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
      : "memory");
}

// Blocks of 21-28 functions: the register budget of three resident CTAs per SM
// (the launcher sizes the grid from the occupancy), which lets the epilogue
// keep 11 functions' loads in flight (measured: 102.7 instead of 106.1 us per
// 54^3 iteration, bit-identical); other sizes give no minimum (0) and keep the
// compiler's choice.
__host__ __device__ constexpr int vstream_min_ctas(int nn) { return nn >= 21 && nn <= 28 ? 3 : 0; }
__host__ __device__ constexpr int vstream_load_group(int nn) { return nn >= 21 && nn <= 28 ? 11 : 7; }

// Persistent: CTA b owns the contiguous tiles [b * A.tiles_per_cta, ...), and
// its copy ring runs across tile boundaries, so the next tile's blocks are in
// flight while the current tile finishes its epilogue.
// Roles (kRole): 0 the H v apply of the modes above; 1 the Lanczos update of a
// graph-replayed iteration fused with the next iteration's block product:
// R = g (R - alpha c V) (alpha from the light apply's block totals, beta's
// block totals deferred), and A.vprod = V_blocks hi(R), hi(R) being the FP32
// head of the next v; 2 A.vprod = V_blocks hi(V) only (before the first
// iteration of a run).
// Formats (kFmt): 0 FP32 blocks; 1 BF16 blocks (A.vb16) scaled per point by
// A.vscale, twice the rows per copy so that a copy still moves 8 KiB; 2 FP32
// spherical-harmonic coefficients (A.vc), from which each thread rebuilds its
// point's block elements (bsl_gaunt.h).
template <int NN, int kFmt>
__host__ __device__ constexpr int rows_per_tile() {
  if constexpr (kFmt == 2) {
    return gaunt::Apply<NN>::kNC;
  } else {
    return NN * (NN + 1) / 2;
  }
}

// The CTA's tiles are [t0, t1); it is block `index` of the `count` blocks that
// reduce alpha together (the grid for one problem; a problem's blocks in a
// grouped launch).
template <int NN, int kFmt, int kRole = 0>
__device__ __forceinline__ void vstream_body(const StreamArgs& A, long long t0, long long t1_arg, unsigned int index,
                                             unsigned int count) {
  constexpr bool kBF = kFmt == 1;
  using TB = typename std::conditional<kBF, uint16_t, float>::type;
  constexpr int NT = rows_per_tile<NN, kFmt>();  // rows streamed per tile
  constexpr int kCh = kBF ? 2 * kChunk : kChunk;  // rows per copy
  constexpr int NCH = (NT + kCh - 1) / kCh;
  extern __shared__ float4 ring4[];
  TB* ring = reinterpret_cast<TB*>(ring4);  // [kStages][kCh][kTilePts]
  __shared__ uint64_t full[kStages];
  __shared__ int abort_flag;
  __shared__ long long issued;
  const int tid = threadIdx.x;
  const long long npts = A.npts;
  const long long ntiles = (npts + kTilePts - 1) / kTilePts;
  const long long t1 = t1_arg < ntiles ? t1_arg : ntiles;
  const long long nchunks = (t1 > t0 ? t1 - t0 : 0) * NCH;
  const TB* src0 = reinterpret_cast<const TB*>(kFmt == 1 ? (const void*)A.vb16
                                                : kFmt == 2 ? (const void*)A.vc : (const void*)A.vb) +
                   t0 * (long long)NT * kTilePts;
  const uint64_t pol = evict_first_policy();
  if (tid == 0) {
    // a stream that already timed out in an earlier launch disables the copies
    // (and every wait) of later launches until the host has seen the error
    abort_flag = *(volatile int*)(A.status + 2);
    issued = 0;
    for (int s = 0; s < kStages; ++s) mbar_init(&full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // chunk g of this CTA: tile t0 + g / NCH, rows [c * kChunk, ...) with c = g % NCH
  auto issue = [&](long long g) {
    const int st = (int)(g % kStages);
    const int c = (int)(g % NCH);
    const int rows = (c == NCH - 1) ? (NT - c * kCh) : kCh;
    const uint32_t bytes = (uint32_t)rows * kTilePts * sizeof(TB);
    mbar_expect_tx(&full[st], bytes);
    issued = g + 1;
    bulk_copy_hint(ring + (size_t)st * kCh * kTilePts,
                   src0 + ((g / NCH) * NT + (long long)c * kCh) * kTilePts, bytes, &full[st], pol);
  };
  if (tid == 0 && !abort_flag)
    for (long long g = 0; g < nchunks && g < kStages; ++g) issue(g);
  // the potential blocks are constant: their first chunks stream in while the
  // kinetic kernel finishes; everything below reads that kernel's output
  pdl_launch_dependents();
  pdl_wait();

  const float2* Vp = reinterpret_cast<const float2*>(A.vec);
  float2* Rp = reinterpret_cast<float2*>(A.out);
  const double c = A.mode == 1 ? A.scalars[6] : 1.0;
  const float2 cc = reinterpret_cast<const float2*>(A.scalars)[8];  // c as a pair (mode 2)
  double dot = 0.0;
  float2 dacc = make_float2(0.f, 0.f);
  // role 1: -alpha c from the light apply's block totals (every CTA the same
  // fixed-order sum) and the update's scale g = 2^e
  float2 na = make_float2(0.f, 0.f);
  float gs = 1.f;
  if constexpr (kRole == 1) {
    __shared__ double sh4[kTilePts / 32];
    const int* si = reinterpret_cast<const int*>(A.scalars);
    const double total = sum_partials(A.partials, si[kAlphaCountSlot], tid, kTilePts, 1, sh4);
    const double alpha = A.scalars[7] * total;
    na = df_of(-alpha * A.scalars[6]);
    gs = ldexpf(1.f, si[20]);
    if (index == 0 && tid == 0) {
      A.scalars[0] = alpha;
      A.hist[*A.jdev - 1] = alpha;
      reinterpret_cast<float2*>(A.scalars)[9] = na;
    }
  }
  long long g0 = 0;  // first chunk of the current tile
  for (long long tile = t0; tile < t1; ++tile, g0 += NCH) {
    const long long p = tile * kTilePts + tid;
    const bool valid = p < npts;
    if (kRole == 0 && valid) {
#pragma unroll
      for (int s = 0; s < NN; ++s) {
        asm volatile("prefetch.global.L2 [%0];" ::"l"(A.ukin + s * npts + p));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(A.out + s * npts + p));
        if (A.mode == 1) asm volatile("prefetch.global.L2 [%0];" ::"l"(A.vec + s * npts + p));
      }
    }
    // mode 2 reads the pair of v once: its head is the FP32 copy (the block
    // product's operand) and its tail is kept for alpha
    float vv[NN], va[NN], vlo[NN];
    if constexpr (kRole == 1) {
      // R = g (R - alpha c V) (the arithmetic of the streamed update), stored;
      // its head is the operand of the next iteration's block product
      constexpr int kGroup = vstream_load_group(NN);
#pragma unroll
      for (int s0 = 0; s0 < NN; s0 += kGroup) {
        float2 vx[kGroup], rx[kGroup];
#pragma unroll
        for (int u = 0; u < kGroup; ++u)
          if (s0 + u < NN) {
            vx[u] = valid ? Vp[(s0 + u) * npts + p] : make_float2(0.f, 0.f);
            rx[u] = valid ? Rp[(s0 + u) * npts + p] : make_float2(0.f, 0.f);
          }
#pragma unroll
        for (int u = 0; u < kGroup; ++u)
          if (s0 + u < NN) {
            const float2 r = df_scale2(df_fma_fast(na, vx[u], rx[u]), gs);
            if (valid) Rp[(s0 + u) * npts + p] = r;
            dacc = df_add_fast(df_sqr(r), dacc);
            vv[s0 + u] = r.x;
            vlo[s0 + u] = 0.f;
            va[s0 + u] = 0.f;
          }
      }
    } else {
#pragma unroll
    for (int s = 0; s < NN; ++s) {
      if (kRole == 2) {
        vv[s] = valid ? Vp[s * npts + p].x : 0.f;
        vlo[s] = 0.f;
      } else if (A.mode == 2) {
        const float2 x = valid ? Vp[s * npts + p] : make_float2(0.f, 0.f);
        vv[s] = x.x;
        vlo[s] = x.y;
      } else {
        vv[s] = valid ? A.v32[s * npts + p] : 0.f;
        vlo[s] = 0.f;
      }
      va[s] = 0.f;
    }
    }
    if constexpr (kFmt == 2) {
      // the point's coefficients, chunk by chunk from the ring, then the block
      // elements rebuilt and multiplied in registers
      float cf[NT];
#pragma unroll
      for (int k = 0; k < NT; ++k) {
        const long long g = g0 + k / kCh;
        const int st = (int)(g % kStages);
        if (k % kCh == 0) {
          if (!abort_flag && !mbar_wait(&full[st], (uint32_t)((g / kStages) & 1))) abort_flag = 1;
        }
        cf[k] = ring[((size_t)st * kCh + (k % kCh)) * kTilePts + tid];
        if (k % kCh == kCh - 1 || k == NT - 1) {
          __syncthreads();  // every thread is done with this stage
          if (tid == 0 && !abort_flag && g + kStages < nchunks) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(g + kStages);
          }
        }
      }
      gaunt::Apply<NN>::run(cf, vv, va);
    } else {
      int t = 0;
  #pragma unroll
      for (int s = 0; s < NN; ++s) {
  #pragma unroll
        for (int q = s; q < NN; ++q, ++t) {
          const long long g = g0 + t / kCh;
          const int st = (int)(g % kStages);
          if (t % kCh == 0) {
            if (!abort_flag && !mbar_wait(&full[st], (uint32_t)((g / kStages) & 1))) abort_flag = 1;
          }
          const TB xr = ring[((size_t)st * kCh + (t % kCh)) * kTilePts + tid];
          float x;
          if constexpr (kBF) {
            x = __uint_as_float((uint32_t)xr << 16);
          } else {
            x = xr;
          }
          va[s] = fmaf(x, vv[q], va[s]);
          if (q != s) va[q] = fmaf(x, vv[s], va[q]);
          if (t % kCh == kCh - 1 || t == NT - 1) {
            __syncthreads();  // every thread is done with this stage
            if (tid == 0 && !abort_flag && g + kStages < nchunks) {
              asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
              issue(g + kStages);
            }
          }
        }
      }
    }
    if (kBF && valid) {
      const float sc = A.vscale[p];
#pragma unroll
      for (int s = 0; s < NN; ++s) va[s] *= sc;
    }
    if (kRole != 0) {
      if (valid) {
#pragma unroll
        for (int s = 0; s < NN; ++s) A.vprod[s * npts + p] = va[s];
      }
      continue;
    }
    // u = kinetic pair + B l(l+1) v + V v as an FP32 pair.
    // mode 1: the logical vectors are v = sv V and r = sr R; r + H v is kept as
    // sr (R + (sv/sr) H V), so R' = R + c H V and alpha = sv sr (V . R').
    // mode 2: the same with V and R stored as double-float pairs, all on the FP32 pipe.
    if (valid) {
      if (A.mode == 2) {
        constexpr int kGroup = vstream_load_group(NN);  // loads in flight before their arithmetic
#pragma unroll
        for (int s0 = 0; s0 < NN; s0 += kGroup) {
          float2 uk[kGroup], rr[kGroup];
#pragma unroll
          for (int u = 0; u < kGroup; ++u)
            if (s0 + u < NN) {
              uk[u] = A.ukin[(s0 + u) * npts + p];
              rr[u] = Rp[(s0 + u) * npts + p];
            }
#pragma unroll
          for (int u = 0; u < kGroup; ++u)
            if (s0 + u < NN) {
              const int s = s0 + u;
              const float a = fmaf(__ldg(A.rot_hi + s), vv[s], va[s]);
              float hi, e, lo;
              two_sum(uk[u].x, a, hi, e);
              two_sum(hi, uk[u].y + e + __ldg(A.rot_lo + s) * vv[s], hi, lo);
              const float2 r = df_fma_fast(cc, make_float2(hi, lo), rr[u]);
              Rp[s * npts + p] = r;
              dacc = df_fma_fast(make_float2(vv[s], vlo[s]), r, dacc);
            }
        }
      } else {
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
    }
  }
  if (abort_flag && tid == 0 && issued > 0) {
    // a copy did not complete in time: record it and give the copies still in
    // flight a bounded chance to land before the CTA's shared memory is released
    A.status[2] = 1;
    for (long long g = issued - kStages; g < issued; ++g)
      if (g >= 0) mbar_wait(&full[g % kStages], (uint32_t)((g / kStages) & 1));
  }
  if constexpr (kRole == 1) {
    // the coordinate outside the symmetry block, then beta's block total for
    // the next x/y kinetic (or the closing kernel)
    if (index == 0 && tid == 0) {
      const float2 r = df_scale2(df_fma_fast(na, Vp[A.dpk], Rp[A.dpk]), gs);
      Rp[A.dpk] = r;
      dacc = df_add_fast(df_sqr(r), dacc);
    }
    const double bt = block_total_df(dacc);
    if (tid == 0) {
      A.partials[kBetaPartials + index] = bt;
      if (index == 0) reinterpret_cast<int*>(A.scalars)[kPendingSlot] = 1;
    }
    return;
  }
  if (kRole == 0 && A.mode != 0) {
    // extra coordinate: H acts as 0, R' = R
    if (index == 0 && tid == 0) {
      if (A.mode == 2)
        dacc = df_fma(Vp[A.dpk], Rp[A.dpk], dacc);
      else
        dot = fma(A.vec[A.dpk], A.out[A.dpk], dot);
    }
    if (A.defer && A.mode == 2) {  // the update forms alpha from the block totals
      const double bt = block_total_df(dacc);
      if (tid == 0) {
        A.partials[index] = bt;
        if (index == 0) reinterpret_cast<int*>(A.scalars)[kAlphaCountSlot] = (int)count;
      }
      return;
    }
    double total;
    const bool last = A.mode == 2 ? reduce_group_df(dacc, A.partials, A.counter, count, index, &total)
                                  : reduce_group(dot, A.partials, A.counter, count, index, &total);
    if (last && threadIdx.x == 0) {
      const double alpha = A.scalars[7] * total;
      A.scalars[0] = alpha;
      A.hist[(A.j > 0 ? A.j : *A.jdev) - 1] = alpha;
      reinterpret_cast<float2*>(A.scalars)[9] = df_of(-alpha * A.scalars[6]);  // for the pair update
    }
  }
}

template <int NN, int kFmt, int kRole = 0>
__global__ void __launch_bounds__(kTilePts, vstream_min_ctas(NN)) k_vstream(const StreamArgs A) {
  const long long t0 = (long long)blockIdx.x * A.tiles_per_cta;
  vstream_body<NN, kFmt, kRole>(A, t0, t0 + A.tiles_per_cta, blockIdx.x, gridDim.x);
}

// The H v apply of a graph-replayed iteration whose block product was formed
// by the previous update (A.vprod): R += c (u_kin + B l(l+1) v + V_blocks hi(v))
// with the arithmetic of the stream's mode 2, one thread per grid point, and
// alpha's block totals stored for the update.  Point p of the problem; the CTA
// is block `index` of the `count` that reduce alpha.
constexpr int kLightThreads = 256;
template <int NN>
__device__ __forceinline__ void light_body(const StreamArgs& A, long long p, unsigned int index,
                                           unsigned int count) {
  const int tid = threadIdx.x;
  const long long npts = A.npts;
  pdl_launch_dependents();
  pdl_wait();
  const float2* Vp = reinterpret_cast<const float2*>(A.vec);
  float2* Rp = reinterpret_cast<float2*>(A.out);
  const float2 cc = reinterpret_cast<const float2*>(A.scalars)[8];
  float2 dacc = make_float2(0.f, 0.f);
  if (p < npts) {
    constexpr int kGroup = 7;
#pragma unroll
    for (int s0 = 0; s0 < NN; s0 += kGroup) {
      float2 vx[kGroup], uk[kGroup], rr[kGroup];
      float va[kGroup];
#pragma unroll
      for (int u = 0; u < kGroup; ++u)
        if (s0 + u < NN) {
          const long long i = (s0 + u) * npts + p;
          vx[u] = Vp[i];
          uk[u] = A.ukin[i];
          rr[u] = Rp[i];
          va[u] = A.vprod[i];
        }
#pragma unroll
      for (int u = 0; u < kGroup; ++u)
        if (s0 + u < NN) {
          const int s = s0 + u;
          const float a = fmaf(__ldg(A.rot_hi + s), vx[u].x, va[u]);
          float hi, e, lo;
          two_sum(uk[u].x, a, hi, e);
          two_sum(hi, uk[u].y + e + __ldg(A.rot_lo + s) * vx[u].x, hi, lo);
          const float2 r = df_fma_fast(cc, make_float2(hi, lo), rr[u]);
          Rp[s * npts + p] = r;
          dacc = df_fma_fast(vx[u], r, dacc);
        }
    }
  }
  // extra coordinate: H acts as 0, R' = R
  if (index == 0 && tid == 0) dacc = df_fma(Vp[A.dpk], Rp[A.dpk], dacc);
  const double bt = block_total_df(dacc);
  if (tid == 0) {
    A.partials[index] = bt;
    if (index == 0) reinterpret_cast<int*>(A.scalars)[kAlphaCountSlot] = (int)count;
  }
}

template <int NN>
__global__ void __launch_bounds__(kLightThreads) k_vapply_light(const StreamArgs A) {
  light_body<NN>(A, (long long)blockIdx.x * kLightThreads + threadIdx.x, blockIdx.x, gridDim.x);
}

// Grouped launches over problems with blocks of 15 or 21 functions (the fused
// iteration of a batch), CTA c working on problem work[c].x as block
// work[c].w of that problem's reduction (over probs[].red_count blocks): the
// light apply of the 256 points from work[c].y * 256, and the fused update of
// tiles [work[c].y, work[c].z).
__global__ void __launch_bounds__(kLightThreads) k_vapply_light_group(const StreamArgs* __restrict__ probs,
                                                                      const int4* __restrict__ work) {
  const int4 w = work[blockIdx.x];
  const StreamArgs A = probs[w.x];
  const long long p = (long long)w.y * kLightThreads + threadIdx.x;
  if (A.nn == 21)
    light_body<21>(A, p, (unsigned)w.w, (unsigned)A.red_count);
  else
    light_body<15>(A, p, (unsigned)w.w, (unsigned)A.red_count);
}

__global__ void __launch_bounds__(kTilePts, 3) k_vstream_group(const StreamArgs* __restrict__ probs,
                                                               const int4* __restrict__ work) {
  const int4 w = work[blockIdx.x];
  const StreamArgs A = probs[w.x];
  if (A.vformat == BSL_VFMT_GAUNT) {
    if (A.nn == 21)
      vstream_body<21, 2, 1>(A, w.y, w.z, (unsigned)w.w, (unsigned)A.red_count);
    else
      vstream_body<15, 2, 1>(A, w.y, w.z, (unsigned)w.w, (unsigned)A.red_count);
  } else {
    if (A.nn == 21)
      vstream_body<21, 0, 1>(A, w.y, w.z, (unsigned)w.w, (unsigned)A.red_count);
    else
      vstream_body<15, 0, 1>(A, w.y, w.z, (unsigned)w.w, (unsigned)A.red_count);
  }
}

// the grid of k_vstream<NN, kFmt, kRole> for a (and its tiles per CTA)
template <int NN, int kFmt, int kRole = 0>
long long vstream_grid(const StreamArgs& a, long long* tiles_per_cta) {
  const size_t smem = (size_t)kStages * kChunk * kTilePts * sizeof(float);
  cudaFuncSetAttribute(k_vstream<NN, kFmt, kRole>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const long long tiles = (a.npts + kTilePts - 1) / kTilePts;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vstream<NN, kFmt, kRole>, kTilePts, smem);
  if (a.ctas_per_sm > 0 && a.ctas_per_sm < per_sm) per_sm = a.ctas_per_sm;
  const long long slots = (long long)(sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  *tiles_per_cta = (tiles + slots - 1) / slots;
  return (tiles + *tiles_per_cta - 1) / *tiles_per_cta;
}

template <int NN, int kFmt = 0, int kRole = 0>
int launch_nn(StreamArgs a, cudaStream_t s) {
  const size_t smem = (size_t)kStages * kChunk * kTilePts * sizeof(float);
  const long long grid = vstream_grid<NN, kFmt, kRole>(a, &a.tiles_per_cta);
  const cudaError_t e = launch_pdl(k_vstream<NN, kFmt, kRole>, dim3((unsigned)grid), dim3(kTilePts), smem, s, a);
  return e == cudaSuccess ? BSL_OK : cuda_fail(e, "potential stream launch");
}

// ---------------------------------------------------------------------------
// Double-float Lanczos update R = g (R - alpha c V) and ||R||^2 (the same
// arithmetic as k_update_pair), streamed: CTA b owns a contiguous range of
// 16-byte units (two pairs) of V and R, brings them in chunks of kUpdUnits
// units per array through a kUpdStages-stage ring of bulk copies, updates R in
// shared memory and writes it back with bulk stores.
// ---------------------------------------------------------------------------
constexpr int kUpdThreads = 256;
constexpr int kUpdUnits = 1024;  // 16 KiB of V and 16 KiB of R per chunk
constexpr int kUpdStages = 3;

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
               "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

struct UpdArgs {
  const float4* V4;
  float4* R4;
  long long L;
  double* partials;
  unsigned int* counter;
  double* scalars;
  double* hist;
  int hist_stride;
  int* jdev;
  int* status;
  int defer;      // alpha from the stream's block totals here, beta's block totals left for the next kinetic
};

// The CTA's 16-byte units are [u0, u1_arg); it is block `index` of the
// `count` blocks that reduce beta together.
__device__ __forceinline__ void update_body(const UpdArgs& a, long long u0, long long u1_arg, unsigned int index,
                                            unsigned int count, int j_arg) {
  const float4* __restrict__ V4 = a.V4;
  float4* __restrict__ R4 = a.R4;
  const long long L = a.L;
  double* partials = a.partials;
  unsigned int* counter = a.counter;
  double* scalars = a.scalars;
  double* hist = a.hist;
  const int hist_stride = a.hist_stride;
  int* jdev = a.jdev;
  int* status = a.status;
  extern __shared__ float4 upd[];  // [stage][V, R][kUpdUnits]
  __shared__ uint64_t full[kUpdStages];
  __shared__ int failed;
  const int tid = threadIdx.x;
  const long long L2 = L / 2;
  const long long u1 = u1_arg < L2 ? u1_arg : L2;
  const long long nchunks = u1 > u0 ? (u1 - u0 + kUpdUnits - 1) / kUpdUnits : 0;
  if (tid == 0) {
    for (int s = 0; s < kUpdStages; ++s) mbar_init(&full[s], 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  pdl_launch_dependents();
  pdl_wait();  // R and alpha come from the potential stream
  const int j = j_arg > 0 ? j_arg : *jdev;
  const int e = reinterpret_cast<const int*>(scalars)[20];
  const float g = ldexpf(1.f, e);
  auto chunk_units = [&](long long k) { return (int)(u1 - (u0 + k * kUpdUnits) < kUpdUnits ? u1 - (u0 + k * kUpdUnits) : kUpdUnits); };
  long long issued = 0;
  auto issue = [&](long long k) {  // thread 0
    const int st = (int)(k % kUpdStages);
    const long long c0 = u0 + k * kUpdUnits;
    const uint32_t bytes = (uint32_t)chunk_units(k) * 16u;
    mbar_expect_tx(&full[st], 2 * bytes);
    bulk_copy(upd + (size_t)(2 * st) * kUpdUnits, V4 + c0, bytes, &full[st]);
    bulk_copy(upd + (size_t)(2 * st + 1) * kUpdUnits, R4 + c0, bytes, &full[st]);
    issued = k + 1;
  };
  if (tid == 0)
    for (long long k = 0; k < nchunks && k < kUpdStages; ++k) issue(k);
  // -alpha c: from the stream's scalars, or (deferred) summed here from its
  // block totals while the first copies are in flight -- every CTA the same
  // fixed-order sum
  float2 na;
  if (a.defer) {
    __shared__ double sh8[kUpdThreads / 32];
    const double total = sum_partials(partials, reinterpret_cast<const int*>(scalars)[kAlphaCountSlot], tid,
                                      kUpdThreads, 1, sh8);
    const double alpha = scalars[7] * total;
    na = df_of(-alpha * scalars[6]);
    if (index == 0 && tid == 0) {
      scalars[0] = alpha;
      hist[j - 1] = alpha;
      reinterpret_cast<float2*>(scalars)[9] = na;
    }
  } else {
    na = reinterpret_cast<const float2*>(scalars)[9];
  }
  float2 acc = make_float2(0.f, 0.f);
  for (long long k = 0; k < nchunks; ++k) {
    const int st = (int)(k % kUpdStages);
    if (!mbar_wait(&full[st], (uint32_t)((k / kUpdStages) & 1))) failed = 1;
    __syncthreads();
    if (failed) break;
    const int n = chunk_units(k);
    const float4* vs = upd + (size_t)(2 * st) * kUpdUnits;
    float4* rs = upd + (size_t)(2 * st + 1) * kUpdUnits;
    for (int q = tid; q < n; q += kUpdThreads) {
      const float4 v = vs[q], r = rs[q];
      const float2 r0 = df_scale2(df_fma_fast(na, make_float2(v.x, v.y), make_float2(r.x, r.y)), g);
      const float2 r1 = df_scale2(df_fma_fast(na, make_float2(v.z, v.w), make_float2(r.z, r.w)), g);
      rs[q] = make_float4(r0.x, r0.y, r1.x, r1.y);
      acc = df_add_fast(df_sqr(r0), acc);
      acc = df_add_fast(df_sqr(r1), acc);
    }
    __syncthreads();  // the chunk's new R is complete in shared memory
    if (tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_store(R4 + u0 + k * kUpdUnits, rs, (uint32_t)n * 16u);
      if (k + kUpdStages < nchunks) {
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // the store has read this stage
        issue(k + kUpdStages);
      }
    }
  }
  if (tid == 0) {
    if (failed) {  // let the copies in flight land (bounded) before the shared memory is released
      status[2] = 1;
      for (long long k = issued - kUpdStages; k < issued; ++k)
        if (k >= 0) mbar_wait(&full[k % kUpdStages], (uint32_t)((k / kUpdStages) & 1));
    }
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  if ((L & 1) && index == 0 && tid == 0) {  // the coordinate outside the symmetry block
    const long long i = L - 1;
    const float2* V = reinterpret_cast<const float2*>(V4);
    float2* R = reinterpret_cast<float2*>(R4);
    const float2 r = df_scale2(df_fma_fast(na, V[i], R[i]), g);
    R[i] = r;
    acc = df_add_fast(df_sqr(r), acc);
  }
  if (a.defer) {  // beta is formed by the next kinetic (or the closing kernel)
    const double bt = block_total_df(acc);
    if (tid == 0) {
      partials[kBetaPartials + index] = bt;
      if (index == 0) reinterpret_cast<int*>(scalars)[kPendingSlot] = 1;
    }
    return;
  }
  double total;
  if (reduce_group_df(acc, partials, counter, count, index, &total) && tid == 0) {
    finish_update_pair(total, e, scalars, hist, hist_stride, j, status);
    if (j_arg <= 0) *jdev = j + 1;  // every block has read j before the last one gets here
  }
}

// the deferred beta after the last iteration (one CTA of kUpdThreads threads)
__global__ void __launch_bounds__(kUpdThreads) k_finish_beta(double* partials, int count, double* scalars,
                                                             double* hist, int hist_stride, int* jdev, int* status) {
  __shared__ double sh8[kUpdThreads / 32];
  pdl_wait();
  finish_deferred_beta(partials + kBetaPartials, count, scalars, hist, hist_stride, jdev, status, threadIdx.x,
                       kUpdThreads, 1, sh8);
}

__global__ void __launch_bounds__(kUpdThreads, 2) k_update_stream(const UpdArgs a, long long units_per_cta, int j_arg) {
  const long long u0 = (long long)blockIdx.x * units_per_cta;
  update_body(a, u0, u0 + units_per_cta, blockIdx.x, gridDim.x, j_arg);
}


}  // namespace

int update_stream_ctas(int ctas_per_sm) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return (ctas_per_sm > 0 ? ctas_per_sm : 2) * (sms > 0 ? sms : 1);
}

int launch_update_stream(const float2* V, float2* R, long long L, double* partials, unsigned int* counter,
                         double* scalars, double* hist, int hist_stride, int j, int* jdev, int* status,
                         cudaStream_t s, int ctas_per_sm, int defer) {
  const size_t smem = (size_t)kUpdStages * 2 * kUpdUnits * sizeof(float4);
  cudaFuncSetAttribute(k_update_stream, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const long long grid = update_stream_ctas(ctas_per_sm);
  const long long L2 = L / 2;
  const long long per = (L2 + grid - 1) / grid;
  const UpdArgs a{reinterpret_cast<const float4*>(V), reinterpret_cast<float4*>(R), L, partials, counter, scalars,
                  hist, hist_stride, jdev, status, defer};
  BSL_CUDA(launch_pdl(k_update_stream, dim3((unsigned)grid), dim3(kUpdThreads), smem, s, a, per, j));
  return BSL_OK;
}

// ---- grouped launches of the fused iteration ---------------------------------
size_t vstream_group_arg_size() { return sizeof(StreamArgs); }
long long light_points_per_cta() { return kLightThreads; }

int launch_finish_beta(double* partials, int count, double* scalars, double* hist, int hist_stride, int* jdev,
                       int* status, cudaStream_t s) {
  BSL_CUDA(launch_pdl(k_finish_beta, dim3(1), dim3(kUpdThreads), 0, s, partials, count, scalars, hist, hist_stride,
                      jdev, status));
  return BSL_OK;
}

bool vstream_group_supported(int nn) { return nn == 15 || nn == 21; }

int vstream_group_ctas_per_sm() {
  const size_t smem = (size_t)kStages * kChunk * kTilePts * sizeof(float);
  cudaFuncSetAttribute(k_vstream_group, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vstream_group, kTilePts, smem);
  return per_sm > 0 ? per_sm : 1;
}

int launch_vstream_group(const void* d_args, const int4* d_work, int nctas, cudaStream_t s) {
  const size_t smem = (size_t)kStages * kChunk * kTilePts * sizeof(float);
  cudaFuncSetAttribute(k_vstream_group, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  BSL_CUDA(launch_pdl(k_vstream_group, dim3(nctas), dim3(kTilePts), smem, s,
                      static_cast<const StreamArgs*>(d_args), d_work));
  return BSL_OK;
}

int launch_light_group(const void* d_args, const int4* d_work, int nctas, cudaStream_t s) {
  BSL_CUDA(launch_pdl(k_vapply_light_group, dim3(nctas), dim3(kLightThreads), 0, s,
                      static_cast<const StreamArgs*>(d_args), d_work));
  return BSL_OK;
}

long long vstream_tile_points() { return kTilePts; }

// BF16 blocks: tile-major like the FP32 blocks, each point's elements divided
// by that point's largest |element| (the FP32 scale), rounded to nearest
__global__ void k_blocks_bf16(const double* __restrict__ vb64, long long npts, int ntri, uint16_t* vb16,
                              float* vscale) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npts;
       p += (long long)gridDim.x * blockDim.x) {
    double m = 0.0;
    for (int t = 0; t < ntri; ++t) m = fmax(m, fabs(vb64[(long long)t * npts + p]));
    const float sc = m > 0.0 ? (float)m : 1.f;
    vscale[p] = sc;
    const long long base = (p / kTilePts) * ntri * kTilePts + p % kTilePts;
    for (int t = 0; t < ntri; ++t) {
      const __nv_bfloat16 b = __double2bfloat16(vb64[(long long)t * npts + p] / (double)sc);
      vb16[base + (long long)t * kTilePts] = *reinterpret_cast<const uint16_t*>(&b);
    }
  }
}

// ---- the fused update path of graph-replayed iterations --------------------
// Supported block sizes and formats: the spherical-harmonic coefficients at 10,
// 15 and 21 functions, FP32 blocks at 15 and 21.
bool fused_update_supported(int vformat, int nn) {
  if (vformat == BSL_VFMT_GAUNT) return nn == 10 || nn == 15 || nn == 21;
  if (vformat == BSL_VFMT_FP32) return nn == 15 || nn == 21;
  return false;
}

#define BSL_FUSED_DISPATCH(ROLE, CALL)                                  \
  if (a.vformat == BSL_VFMT_GAUNT) {                                    \
    if (nn == 10) return CALL<10, 2, ROLE>(a, s);                             \
    if (nn == 15) return CALL<15, 2, ROLE>(a, s);                             \
    if (nn == 21) return CALL<21, 2, ROLE>(a, s);                             \
  } else if (a.vformat == BSL_VFMT_FP32) {                              \
    if (nn == 15) return CALL<15, 0, ROLE>(a, s);                             \
    if (nn == 21) return CALL<21, 0, ROLE>(a, s);                             \
  }

// CTAs of the fused update (the block totals of its deferred beta)
int fused_update_ctas(const StreamArgs& a, int nn) {
  long long tpc = 0;
#define BSL_GRID(NN_, F_, R_) (int)vstream_grid<NN_, F_, R_>(a, &tpc)
  if (a.vformat == BSL_VFMT_GAUNT) {
    if (nn == 10) return BSL_GRID(10, 2, 1);
    if (nn == 15) return BSL_GRID(15, 2, 1);
    if (nn == 21) return BSL_GRID(21, 2, 1);
  } else if (a.vformat == BSL_VFMT_FP32) {
    if (nn == 15) return BSL_GRID(15, 0, 1);
    if (nn == 21) return BSL_GRID(21, 0, 1);
  }
#undef BSL_GRID
  return 0;
}

// role 1: the fused update; role 2: the block product of V alone
int launch_update_fused(const StreamArgs& a, int nn, int role, cudaStream_t s) {
  if (!a.vprod) return fail(BSL_ERR_STATE, "fused update: no product buffer");
  if (role == 1) {
    if (fused_update_ctas(a, nn) > kBetaPartials) return fail(BSL_ERR_UNSUPPORTED, "fused update: too many CTAs");
    BSL_FUSED_DISPATCH(1, launch_nn)
  } else {
    BSL_FUSED_DISPATCH(2, launch_nn)
  }
  return fail(BSL_ERR_UNSUPPORTED, "fused update: unsupported block size or format");
}
#undef BSL_FUSED_DISPATCH

int launch_vapply_light(const StreamArgs& a, int nn, cudaStream_t s) {
  const long long grid = (a.npts + kLightThreads - 1) / kLightThreads;
  if (grid > kBetaPartials) return fail(BSL_ERR_UNSUPPORTED, "light apply: too many CTAs for the reduction slots");
  if (!a.vprod) return fail(BSL_ERR_STATE, "light apply: no product buffer");
  cudaError_t e;
  if (nn == 10)
    e = launch_pdl(k_vapply_light<10>, dim3((unsigned)grid), dim3(kLightThreads), 0, s, a);
  else if (nn == 15)
    e = launch_pdl(k_vapply_light<15>, dim3((unsigned)grid), dim3(kLightThreads), 0, s, a);
  else if (nn == 21)
    e = launch_pdl(k_vapply_light<21>, dim3((unsigned)grid), dim3(kLightThreads), 0, s, a);
  else
    return fail(BSL_ERR_UNSUPPORTED, "light apply: unsupported block size");
  return e == cudaSuccess ? BSL_OK : cuda_fail(e, "light apply launch");
}

int launch_vapply_f32(const StreamArgs& a, int nn, cudaStream_t s) {
  if (a.vformat == BSL_VFMT_BF16) {
    if (nn == 15) return launch_nn<15, 1>(a, s);
    if (nn == 21) return launch_nn<21, 1>(a, s);
    return fail(BSL_ERR_UNSUPPORTED, "BF16 potential blocks are built for blocks of 15 and 21 functions");
  }
  if (a.vformat == BSL_VFMT_GAUNT) {
    if (nn == 10) return launch_nn<10, 2>(a, s);
    if (nn == 15) return launch_nn<15, 2>(a, s);
    if (nn == 21) return launch_nn<21, 2>(a, s);
    return fail(BSL_ERR_UNSUPPORTED, "no spherical-harmonic stream for this block size");
  }
#define BSL_CASE(K)                          \
  case K:                                    \
    if (int rc = launch_nn<K>(a, s)) return rc; \
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

int dev_vblocks_bf16(bsl_handle* h) {
  DeviceState& d = h->d;
  const Tables& t = h->t;
  const long long N = t.npts, ntri = (long long)t.nn * (t.nn + 1) / 2;
  const long long tiled = (N + kTilePts - 1) / kTilePts * kTilePts;
  if (!d.vb64) return fail(BSL_ERR_STATE, "FP64 potential blocks are not on the device");
  cudaError_t e;
  if ((e = cudaMalloc(&d.vb16, (size_t)(ntri * tiled) * sizeof(uint16_t))) != cudaSuccess ||
      (e = cudaMalloc(&d.vscale, (size_t)tiled * sizeof(float))) != cudaSuccess) {
    cudaFree(d.vb16);
    d.vb16 = nullptr;
    return fail(BSL_ERR_NOMEM, std::string("BF16 potential blocks: ") + cudaGetErrorString(e));
  }
  BSL_CUDA(cudaMemsetAsync(d.vb16, 0, (size_t)(ntri * tiled) * sizeof(uint16_t), d.stream));
  BSL_CUDA(cudaMemsetAsync(d.vscale, 0, (size_t)tiled * sizeof(float), d.stream));
  k_blocks_bf16<<<grid_for(N), kThreads, 0, d.stream>>>(d.vb64, N, (int)ntri, d.vb16, d.vscale);
  BSL_CUDA(cudaGetLastError());
  BSL_CUDA(cudaStreamSynchronize(d.stream));
  return BSL_OK;
}

}  // namespace bsl
