// Sinc-DVR kinetic contractions on the fifth-generation tensor cores
// (tcgen05.mma kind::f16, accumulators in tensor memory), sm_103a, with
// exact accumulation.
//
// Reference: Tv_5D_oneCompositeIndex / Mv_5D_oneCompositeIndex,
// Hv-calculators/linRotor/cartSphBasis/HvCalc/linRotCartSphHvRoutines.cpp:1807-1969.
//
// Work unit: a pair of planes.  The accumulator D has M = 128 rows (p, x) --
// plane p of the pair, grid column x -- and N = 64 columns (the other in-plane
// index), K = 64 per contraction:
//   x and y (k_kin_xy_tc), planes (y, x) of fixed (s, z); both directions
//     accumulate into the same D[(p, x)][y]:
//       y:  sum_q v_p(q, x) Ty[y][q]      A = v tile read MN-major, B = T
//       x:  sum_q Tx[x][q] v_p(y, q)      A = diag(Tx, Tx) over K = (p', q), B = v tile
//     (the block-diagonal A is two 128-row tiles [T; 0] and [0; T] made from the
//     T tile and zero tiles laid out around it);
//   z (k_kin_z_tc), planes (z, x) of fixed (s, y):
//       sum_q v_p(q, x) Tz[z][q]           A = v tile read MN-major, B = T
//     and the result is added to the x/y result.
// Every v tile is stored once, row by row as it lies in memory (64 FP16 per
// 128-byte swizzled row), and read by both terms; the output rows of D are
// grid columns, so the epilogue's stores are coalesced along x.
//
// Exactness (error-free slicing after Ozaki, Ogita, Oishi and Rump,
// Numer. Algorithms 59, 2012, here with 9-bit fixed-point slices): each plane
// of the double-float Lanczos vector is scaled by a power of two to below 1 in
// magnitude and cut into four 9-bit signed integer slices,
// v = 2^(e - 8) (a1 + 2^-9 a2 + 2^-18 a3 + 2^-27 a4) (36 bits relative to the
// plane's maximum); T is scaled from its largest element and cut the same way,
// rounded to nearest so that the symmetric T stays exactly symmetric.  The
// slices are integers in [-256, 256], exact in FP16, their products are exact,
// and the products of each scale class k + l <= 3 (10 products) share one
// accumulator.  A class sum is bounded by 2 * sum_{k+l=c} 256 max_x sum_q |b_l[x][q]|,
// below 2^23.6 for the sinc-DVR T (its first slice decays as 1/(x - q)^2), so
// the FP32 accumulation in tensor memory is exact whatever its internal
// rounding.  The four classes are combined on the CUDA cores into a
// double-float pair.
//
// Pipeline: one persistent CTA per SM with three roles.  Eight producer warps
// load a plane pair, find each plane's scale and write the slices into one of
// two 64 KiB shared-memory stages; one thread issues the pair's 72 (x/y) or
// 16 (z) MMAs into one of two 256-column accumulator stages; eight epilogue
// warps read the finished accumulators and store (x/y) or add (z) the
// double-float results.  mbarriers hand the stages over; every wait is bounded
// and a timeout sets status[3].
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "bsl_device.cuh"
#include "bsl_internal.h"
#include "bsl_tc.cuh"

namespace bsl {
namespace {

constexpr int kVS = 4;                        // slices of v
constexpr int kTS = 4;                        // slices of T
constexpr uint32_t kTile = 64 * 128;          // 8 KiB: 64 rows x 64 FP16, one 128-byte swizzled row each
constexpr uint32_t kPlaneSlices = kVS * kTile;  // the v slices of one plane, contiguous
constexpr uint32_t kStage = 2 * kPlaneSlices;   // v slices of a plane pair: [plane][slice] tiles
constexpr int kStages = 2;                    // shared-memory stages and accumulator stages
constexpr uint32_t kAccCols = 4 * 64;         // accumulator columns of one pair (classes 0..3)
constexpr int kEpiWarps = 8;                  // warps 0-7
constexpr int kProdWarps = 8;                 // warps 8-15
constexpr int kMmaWarp = kEpiWarps + kProdWarps;  // warp 16: MMA issue and tensor-memory owner
constexpr int kWsThreads = (kMmaWarp + 1) * 32;
constexpr int kProdThreads = kProdWarps * 32;
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr int kMaxItems = 64 * 16 / kProdThreads;  // (row, 4-column group) items per producer thread

struct KinTC {
  const uint4* timage;      // the T tiles as laid out in shared memory (kinetic_smem_image)
  int timage16;             // its size in 16-byte units
  int e_t;                  // T = 2^(e_t - 8) (b1 + 2^-9 b2 + 2^-18 b3 + 2^-27 b4)
  const float2* v;          // the Lanczos v as double-float pairs
  float2* out;
  int nx, ny, nz, nplanes;
  int* status;
  int nslices;              // slices of v and of T kept (1-4; 4 = exact), classes k + l < nslices
  // x/y of a graph-replayed iteration: the first CTA's epilogue warps finish
  // the previous update's deferred beta (null: nothing deferred)
  double* fin_partials;
  double* scalars;
  double* hist;
  int* jdev;
  int fin_count, hist_stride;
};

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~(uintptr_t)1023);
}

// byte offset of element k (a multiple of 4) of row r in an SW128 tile of 64 FP16 per row
__device__ __forceinline__ uint32_t quad_offset(int r, int k) {
  return (uint32_t)(r * 128 + (((k >> 3) ^ (r & 7)) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// exponent e with max|x| 2^-e in [0.5, 1]; 0 for an all-zero plane
__device__ __forceinline__ int plane_exponent(float maxabs) {
  if (!(maxabs > 0.f)) return 0;
  return max(-100, ilogbf(maxabs) + 1);
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((min(max(e, -126), 127) + 127) << 23); }

// Four 9-bit slices of a double-float value already scaled to |y| < 256 (hi and
// lo multiplied by the same power of two): y = a1 + 2^-9 a2 + 2^-18 a3 +
// 2^-27 a4 + O(2^-28), each a an integer in [-256, 256].  Every step is exact
// except the last rounding.
__device__ __forceinline__ void slice4(float yh, float yl, float (&a)[kVS]) {
  a[0] = rintf(yh);
  float r = __fmul_rn(__fadd_rn(__fsub_rn(yh, a[0]), yl), 512.f);
  a[1] = rintf(r);
  r = __fmul_rn(__fsub_rn(r, a[1]), 512.f);
  a[2] = rintf(r);
  r = __fmul_rn(__fsub_rn(r, a[2]), 512.f);
  a[3] = rintf(r);
}

// the four class accumulators of 8 consecutive columns combined into
// double-float pairs and multiplied by `scale` (a power of two).  The classes
// are exact integers below 2^24: the head is c0 + 2^-9 c1 with its rounding
// error, the tail collects that error and the two smaller classes (its own
// rounding is ~2^-33 of the head); the pair is left unnormalised (|lo| may
// slightly exceed half an ulp of hi), which the double-float additions accept.
// With fewer than four slices the classes at and above `nslices` were never
// written and are taken as zero.
__device__ __forceinline__ void load_pairs8(uint32_t taddr, float scale, int nslices, float2 (&out)[8]) {
  float c0[8], c1[8], c2[8], c3[8];
  tc::tmem_ld8_nowait(taddr, c0);
  tc::tmem_ld8_nowait(taddr + 64u, c1);
  tc::tmem_ld8_nowait(taddr + 128u, c2);
  tc::tmem_ld8_nowait(taddr + 192u, c3);
  tc::tmem_wait_ld();
  if (nslices < 4) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      c3[u] = 0.f;
      c2[u] = nslices > 2 ? c2[u] : 0.f;
      c1[u] = nslices > 1 ? c1[u] : 0.f;
    }
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    float h, e;
    two_sum(c0[u], __fmul_rn(c1[u], 0x1p-9f), h, e);
    const float l = __fmaf_rn(c3[u], 0x1p-27f, __fmaf_rn(c2[u], 0x1p-18f, e));
    out[u] = make_float2(__fmul_rn(h, scale), __fmul_rn(l, scale));
  }
}

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }


// Plane geometry: x/y planes are the contiguous (y, x) planes of fixed (s, z);
// z planes are the (z, x) planes of fixed (s, y), rows nx * ny apart.
template <bool kXY>
struct Planes {
  int nx, ny, nz, nplanes;
  __device__ __forceinline__ long long base(int plane) const {
    if (kXY) return (long long)plane * nx * ny;
    return (long long)(plane / ny) * nz * nx * ny + (long long)(plane % ny) * nx;
  }
  __device__ __forceinline__ long long row_stride() const { return kXY ? (long long)nx : (long long)nx * ny; }
  __device__ __forceinline__ int rows() const { return kXY ? ny : nz; }
};

// The CTA's plane pairs: p_first, p_first + p_stride, ... below p_end (the
// single-problem launch strides over the grid; a grouped launch gives each CTA
// one contiguous range of one problem).
template <bool kXY>
__device__ __forceinline__ void kin_ws_body(const KinTC& a, int p_first, int p_stride, int p_end) {
  extern __shared__ uint8_t smraw[];
  uint8_t* sm = align1024(smraw);
  // T tiles: x/y as Z T0 T1 T2 T3 Z (Z = zero tile), z as T0 T1 T2 T3; then
  // the v stages
  constexpr int kTTiles = kXY ? kTS + 2 : kTS;
  uint8_t* V = sm + kTTiles * kTile;
  __shared__ uint64_t v_full[kStages], v_empty[kStages], acc_full[kStages], acc_empty[kStages], e_full[kStages];
  __shared__ uint64_t stages_zeroed, t_ready;  // setup by the epilogue warps
  __shared__ uint32_t tmem_slot;
  __shared__ int e_stage[kStages][2], e_acc[kStages][2];
  __shared__ float red[2][kProdWarps];
  __shared__ int prod_go, failed, skip;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const Planes<kXY> pg{a.nx, a.ny, a.nz, a.nplanes};
  const int npairs = min((a.nplanes + 1) / 2, p_end);

  // a kinetic time-out recorded before this launch (an earlier launch of the
  // run, or the host's injection) makes the CTA leave before it allocates
  // tensor memory, loads, issues an MMA or waits; one thread reads the flag so
  // that the whole CTA takes the same branch
  if (tid == 0) skip = *(volatile int*)(a.status + 3);
  __syncthreads();
  if (skip) return;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&v_full[s], kProdThreads);
      tc::mbar_init(&v_empty[s], 1);
      tc::mbar_init(&acc_full[s], 1);
      tc::mbar_init(&acc_empty[s], kEpiThreads);
      tc::mbar_init(&e_full[s], 1);
    }
    tc::mbar_init(&stages_zeroed, kEpiThreads);
    tc::mbar_init(&t_ready, kEpiThreads);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaWarp) tc::tmem_alloc(&tmem_slot, kStages * kAccCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  pdl_launch_dependents();

  if (warp < kEpiWarps) {
    // ---- epilogue: TMEM lane quadrant warp % 4 = (plane p, 32-column block of
    // x), columns [32 half, 32 half + 32) ----
    const int quad = warp & 3, half = warp >> 2;
    const int p = quad >> 1, x = ((quad & 1) << 5) + lane;
    const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
    const int ncols = pg.rows();
    const long long cstride = pg.row_stride();
    const int c_begin = half * 32, c_end = min(half * 32 + 32, ncols);
    {  // setup while the producers' first planes are in flight: zeroed v stages
       // (the producers write only the rows and 4-column groups that hold data,
       // so the padding of every stage stays zero), then the T tiles (a
       // prebuilt image of that region) for the MMA thread
      for (int e = tid; e < (int)(kStages * kStage / 16); e += kEpiThreads)
        reinterpret_cast<uint4*>(V)[e] = make_uint4(0u, 0u, 0u, 0u);
      tc::fence_smem_to_async();
      tc::mbar_arrive(&stages_zeroed);
      constexpr int kBatch = 6;
      for (int e0 = tid; e0 < a.timage16; e0 += kBatch * kEpiThreads) {
        uint4 img[kBatch];
#pragma unroll
        for (int r = 0; r < kBatch; ++r) {
          const int e = e0 + r * kEpiThreads;
          img[r] = e < a.timage16 ? a.timage[e] : make_uint4(0u, 0u, 0u, 0u);
        }
#pragma unroll
        for (int r = 0; r < kBatch; ++r) {
          const int e = e0 + r * kEpiThreads;
          if (e < a.timage16) reinterpret_cast<uint4*>(sm)[e] = img[r];
        }
      }
      tc::fence_smem_to_async();
      tc::mbar_arrive(&t_ready);
    }
    pdl_wait();  // the output (and, for z, the values added to) belong to earlier kernels
    if (kXY && a.fin_partials && p_first == 0) {
      __shared__ double fin8[kEpiWarps];
      finish_deferred_beta(a.fin_partials + kBetaPartials, a.fin_count, a.scalars, a.hist, a.hist_stride, a.jdev,
                           a.status, tid, kEpiThreads, 2, fin8);
    }
    // z: the values the epilogue adds to, 8 columns of this thread's x
    auto load8 = [&](long long ob, bool valid, int c0, float2 (&u0)[8]) {
#pragma unroll
      for (int u = 0; u < 8; ++u)
        u0[u] = (valid && c0 + u < c_end) ? a.out[ob + (c0 + u) * cstride] : make_float2(0.f, 0.f);
    };
    for (int it = 0, pair = p_first; pair < npairs; pair += p_stride, ++it) {
      const int st = it & 1;
      const uint32_t par = (uint32_t)(it >> 1) & 1u;
      const int plane = 2 * pair + p;
      const bool valid = plane < a.nplanes && x < a.nx;
      const long long ob = valid ? pg.base(plane) + x : 0;
      float2 nxt[8];  // z: first chunk loaded while the products run
      if (!kXY) load8(ob, valid, c_begin, nxt);
      // lane 0 waits (bounded) and the warp leaves together on a timeout; once the
      // phases are complete every lane's own wait returns at once and orders its
      // reads after the producers' and the MMA thread's writes
      int ok = 1;
      if (lane == 0) ok = tc::mbar_wait(&acc_full[st], par) && tc::mbar_wait(&e_full[st], par);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) {
        failed = 1;
        break;
      }
      tc::mbar_wait(&acc_full[st], par);
      tc::mbar_wait(&e_full[st], par);
      tc::fence_after_sync();
      const float scale = pow2f(e_acc[st][p] + a.e_t - 16);
      const uint32_t tbase = tmem + (uint32_t)st * kAccCols + lane_base;
#pragma unroll 1
      for (int c0 = c_begin; c0 < c_end; c0 += 8) {
        float2 v[8];
        if (kXY) {
          load_pairs8(tbase + (uint32_t)c0, scale, a.nslices, v);
          if (valid)
#pragma unroll
            for (int u = 0; u < 8; ++u)
              if (c0 + u < c_end) a.out[ob + (c0 + u) * cstride] = v[u];
        } else {
          float2 cur[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) cur[u] = nxt[u];
          if (c0 + 8 < c_end) load8(ob, valid, c0 + 8, nxt);  // the next chunk, in flight meanwhile
          load_pairs8(tbase + (uint32_t)c0, scale, a.nslices, v);
          if (valid)
#pragma unroll
            for (int u = 0; u < 8; ++u)
              if (c0 + u < c_end) a.out[ob + (c0 + u) * cstride] = df_add_fast(cur[u], v[u]);
        }
      }
      tc::fence_before_sync();
      tc::mbar_arrive(&acc_empty[st]);
    }
  } else if (warp < kMmaWarp) {
    // ---- producers: item i = (row i / ncg, 4-column group i % ncg) of a plane,
    // items ptid, ptid + 256, ...; the next plane's items are loaded into
    // registers while this one is sliced ----
    const int ptid = tid - kEpiThreads, pw = ptid >> 5;
    const int nrows = pg.rows(), nx = a.nx, ncg = (nx + 3) >> 2, nitems = nrows * ncg;
    const long long rstride = pg.row_stride();
    // per item: offset in a plane, offset in a shared-memory tile, values present
    int goff[kMaxItems], cnt[kMaxItems];
    uint32_t soff[kMaxItems];
#pragma unroll
    for (int t = 0; t < kMaxItems; ++t) {
      const int i = ptid + t * kProdThreads;
      const int j = i / ncg, c = (i - j * ncg) * 4;
      const bool iv = i < nitems;
      goff[t] = iv ? (int)(j * rstride) + c : 0;
      soff[t] = iv ? quad_offset(j, c) : 0u;
      cnt[t] = iv ? min(4, nx - c) : 0;
    }
    auto load_items = [&](int plane, float2 (&x)[kMaxItems][4]) {
      const bool pv = plane < a.nplanes;
      const float2* src = a.v + (pv ? pg.base(plane) : 0);
#pragma unroll
      for (int t = 0; t < kMaxItems; ++t)
#pragma unroll
        for (int u = 0; u < 4; ++u)
          x[t][u] = (pv && u < cnt[t]) ? __ldg(src + goff[t] + u) : make_float2(0.f, 0.f);
    };
    auto prefetch_plane = [&](int plane) {  // into L2, one 16-value row segment per thread
      if (plane >= a.nplanes) return;
      const int j = ptid >> 2, i = (ptid & 3) * 16;
      if (j < nrows && i < nx) prefetch_l2(a.v + pg.base(plane) + j * rstride + i);
    };
    float2 x[kMaxItems][4];
    pdl_wait();  // v is written by the previous iteration's update
    load_items(2 * p_first, x);  // in flight during the setup
    int slot = 0;
    for (int it = 0, pair = p_first; pair < npairs; pair += p_stride, ++it) {
      const int st = it & 1;
      const uint32_t par = (uint32_t)(it >> 1) & 1u;
      if (ptid == 0)
        prod_go = ((it > 0 || tc::mbar_wait(&stages_zeroed, 0u)) && tc::mbar_wait(&v_empty[st], par ^ 1u)) ? 1 : 0;
      tc::named_sync(1, kProdThreads);
      if (!prod_go) {
        if (ptid == 0) failed = 1;
        break;
      }
      {  // the pair after next into L2
        const int far = 2 * (pair + 2 * p_stride);
        prefetch_plane(far);
        prefetch_plane(far + 1);
      }
      uint8_t* vs = V + st * kStage;
#pragma unroll 1
      for (int pl = 0; pl < 2; ++pl) {
        float2 y[kMaxItems][4];  // the next plane, in flight while this one is sliced
        load_items(pl == 0 ? 2 * pair + 1 : 2 * (pair + p_stride), y);
        float mx = 0.f;
#pragma unroll
        for (int t = 0; t < kMaxItems; ++t)
#pragma unroll
          for (int u = 0; u < 4; ++u) mx = fmaxf(mx, fabsf(x[t][u].x));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) red[slot][pw] = mx;
        tc::named_sync(1, kProdThreads);
#pragma unroll
        for (int w = 0; w < kProdWarps; ++w) mx = fmaxf(mx, red[slot][w]);
        slot ^= 1;
        const int e = plane_exponent(mx);
        if (ptid == 0) e_stage[st][pl] = e;
        const float sc = pow2f(8 - e);
        uint8_t* vp = vs + pl * kPlaneSlices;
#pragma unroll
        for (int t = 0; t < kMaxItems; ++t) {
          if (cnt[t] > 0) {
            float sl[4][kVS];
#pragma unroll
            for (int u = 0; u < 4; ++u) slice4(__fmul_rn(x[t][u].x, sc), __fmul_rn(x[t][u].y, sc), sl[u]);
#pragma unroll
            for (int k = 0; k < kVS; ++k)
              if (k < a.nslices)
                *reinterpret_cast<uint2*>(vp + k * kTile + soff[t]) =
                  make_uint2(pack_h2(sl[0][k], sl[1][k]), pack_h2(sl[2][k], sl[3][k]));
          }
        }
#pragma unroll
        for (int t = 0; t < kMaxItems; ++t)
#pragma unroll
          for (int u = 0; u < 4; ++u) x[t][u] = y[t][u];
      }
      tc::fence_smem_to_async();
      tc::mbar_arrive(&v_full[st]);
    }
  } else if (lane == 0) {
    // ---- MMA issue ----
    const uint32_t tb = tc::smem_u32(sm);
    if (!tc::mbar_wait(&t_ready, 0u)) failed = 1;
    for (int it = 0, pair = p_first; pair < npairs && !failed; pair += p_stride, ++it) {
      const int st = it & 1;
      const uint32_t par = (uint32_t)(it >> 1) & 1u;
      if (!tc::mbar_wait(&v_full[st], par) || !tc::mbar_wait(&acc_empty[st], par ^ 1u)) {
        failed = 1;
        break;
      }
      tc::fence_after_sync();
      e_acc[st][0] = e_stage[st][0];
      e_acc[st][1] = e_stage[st][1];
      tc::mbar_arrive(&e_full[st]);
      const uint32_t d0 = tmem + (uint32_t)st * kAccCols;
      const uint32_t vb = tc::smem_u32(V + st * kStage);
      // Class c accumulates in columns [64 c, 64 c + 64).  An MMA whose B stacks
      // the slices l = 0 .. ns - 1 - k of one operand along N (rows 64 l ..) and
      // whose D starts at column 64 k puts product (k, l) into class k + l
      // (ns = 4 slices, the exact default: classes 0..3, 10 products).
      // Contraction over the rows of each plane (y for x/y, z for z): A = v
      // slice k (M = (p, x), MN-major, the planes kPlaneSlices apart), B = T
      // slices 0 .. ns - 1 - k; 16 rows (2 KiB) per K step.  The first MMA
      // (k = 0, N = 64 ns) sets every class.
      const uint32_t t0 = tb + (kXY ? kTile : 0u);
      const int ns = a.nslices;
#pragma unroll 1
      for (int k = 0; k < ns; ++k) {
        const uint32_t idesc = tc::idesc_f16(128, 64 * (ns - k)) | tc::kIdescAMajorMN;
#pragma unroll
        for (int s = 0; s < 4; ++s)
          tc::mma_f16(d0 + (uint32_t)k * 64u,
                      tc::sw128_mn_desc(vb + (uint32_t)k * kTile + (uint32_t)s * 2048u, kPlaneSlices, 1024u),
                      tc::sw128_desc(t0 + (uint32_t)s * 32u), idesc, (k == 0 && s == 0) ? 0u : 1u);
      }
      if (kXY) {
        // contraction along x: A = diag(T_l, T_l) over K = (p', q), read MN-major
        // (T is symmetric) with its two 64-row blocks chosen by the start address
        // and the block stride: [T_l; 0] = (T_l, the zero tile above) and
        // [0; T_l] = (the zero tile below, T_l); B = v slices 0 .. 3 - l of plane p'
        // stacked along N
        const uint32_t zlo = tb, zhi = tb + (uint32_t)(kTS + 1) * kTile;
#pragma unroll 1
        for (int l = 0; l < ns; ++l) {
          const uint32_t tl = t0 + (uint32_t)l * kTile;
          const uint32_t idesc = tc::idesc_f16(128, 64 * (ns - l)) | tc::kIdescAMajorMN;
#pragma unroll
          for (int s = 0; s < 8; ++s) {
            const uint32_t pp = (uint32_t)(s >> 2), q = (uint32_t)(s & 3);
            const uint64_t adesc = pp ? tc::sw128_mn_desc(zlo + q * 2048u, tl - zlo, 1024u)
                                      : tc::sw128_mn_desc(tl + q * 2048u, zhi - tl, 1024u);
            tc::mma_f16(d0 + (uint32_t)l * 64u, adesc, tc::sw128_desc(vb + pp * kPlaneSlices + q * 32u), idesc, 1u);
          }
        }
      }
      tc::mma_commit(&v_empty[st]);
      tc::mma_commit(&acc_full[st]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (failed && tid == 0) a.status[3] = 1;
  if (warp == kMmaWarp) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kStages * kAccCols);
  }
}

// x and y contractions: out(y, x) = (Tx v + Ty v) as double-float pairs
__global__ void __launch_bounds__(kWsThreads, 1) k_kin_xy_tc(KinTC a) {
  kin_ws_body<true>(a, blockIdx.x, gridDim.x, 1 << 30);
}

// z contraction added into the pairs: out(z, x) += Tz v
__global__ void __launch_bounds__(kWsThreads, 1) k_kin_z_tc(KinTC a) {
  kin_ws_body<false>(a, blockIdx.x, gridDim.x, 1 << 30);
}

// Grouped launch over several problems (each with its own grid, T image and
// vectors): CTA c works on problem work[c].x, pairs [work[c].y, work[c].z).
__global__ void __launch_bounds__(kWsThreads, 1) k_kin_xy_tc_group(const KinTC* __restrict__ probs,
                                                                    const int4* __restrict__ work) {
  const int4 w = work[blockIdx.x];
  const KinTC a = probs[w.x];
  kin_ws_body<true>(a, w.y, 1, w.z);
}
__global__ void __launch_bounds__(kWsThreads, 1) k_kin_z_tc_group(const KinTC* __restrict__ probs,
                                                                   const int4* __restrict__ work) {
  const int4 w = work[blockIdx.x];
  const KinTC a = probs[w.x];
  kin_ws_body<false>(a, w.y, 1, w.z);
}

constexpr size_t kSmemXY = 1024 + (kTS + 2) * kTile + kStages * kStage;
constexpr size_t kSmemZ = 1024 + kTS * kTile + kStages * kStage;
static_assert(kSmemXY + 512 <= 227 * 1024, "x/y T tiles and stages must fit in one CTA's shared memory");
static_assert(kStages * kAccCols <= 512, "the accumulator stages must fit in tensor memory");

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, sms);
}

uint16_t half_bits(float x) {  // FP16 bits of a small integer (|x| <= 2048: exact)
  const __half h = __float2half_rn(x);
  uint16_t u;
  std::memcpy(&u, &h, 2);
  return u;
}

}  // namespace

// Fixed-point FP16 slices of an n x n kinetic matrix, T = 2^(e_t - 8) (b1 +
// 2^-9 b2 + 2^-18 b3 + 2^-27 b4) + O(2^(e_t - 36)), each b an integer in
// [-256, 256] rounded to nearest (a symmetric T stays symmetric), as the bytes
// of the kernels' shared-memory T region: tiles of 64 rows (output index) x 64
// FP16 (contraction index), zero padded, 128-byte rows with 16-byte chunk c of
// row r at chunk c ^ (r % 8); with_zero_tiles adds a zero tile before and after
// the four slice tiles (the x/y layout).
void kinetic_smem_image(const std::vector<double>& T, int n, bool with_zero_tiles, std::vector<uint16_t>* image,
                        int* e_t) {
  double m = 0.0;
  for (double x : T) m = std::max(m, std::fabs(x));
  int e = 0;
  if (m > 0.0) std::frexp(m, &e);  // m = f 2^e, f in [0.5, 1)
  *e_t = e;
  const int first = with_zero_tiles ? 1 : 0, ntiles = kTS + 2 * first;
  image->assign((size_t)ntiles * kTile / 2, half_bits(0.f));
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < n; ++q) {
      double r = std::ldexp(T[(size_t)i * n + q], 8 - e);
      for (int l = 0; l < kTS; ++l) {
        const double b = std::nearbyint(r);
        const size_t byte = (size_t)(first + l) * kTile + (size_t)i * 128 + (size_t)(((q >> 3) ^ (i & 7)) << 4) +
                            (size_t)(q & 7) * 2;
        (*image)[byte / 2] = half_bits((float)b);
        r = (r - b) * 512.0;
      }
    }
}

bool kinetic_tc_supported(const Tables& t) { return t.nx <= 64 && t.ny <= 64 && t.nz <= 64 && t.tx == t.ty; }

namespace {
// the kernel arguments of one problem's x/y (xy = true) or z contraction of v
// (fin_count > 0: the x/y launch finishes a deferred beta of that many block totals)
KinTC kin_tc_args(bsl_handle* h, const float2* v, bool xy, int fin_count) {
  const Tables& t = h->t;
  DeviceState& d = h->d;
  KinTC a{};
  a.v = v;
  a.out = reinterpret_cast<float2*>(d.ukin);
  a.nx = t.nx;
  a.ny = t.ny;
  a.nz = t.nz;
  a.status = d.status;
  a.nslices = h->kin_slices;
  if (xy) {
    a.timage = reinterpret_cast<const uint4*>(d.kxy_slices);
    a.timage16 = (int)((kTS + 2) * kTile / 16);
    a.e_t = d.e_txy;
    a.nplanes = t.nz * t.nn;
    if (fin_count > 0) {
      a.fin_partials = d.partials;
      a.scalars = d.scalars;
      a.hist = d.hist;
      a.jdev = d.jdev;
      a.fin_count = fin_count;
      a.hist_stride = d.hist_cap;
    }
  } else {
    a.timage = reinterpret_cast<const uint4*>(d.kz_slices);
    a.timage16 = (int)(kTS * kTile / 16);
    a.e_t = d.e_tz;
    a.nplanes = t.ny * t.nn;
  }
  return a;
}
}  // namespace

size_t kin_group_arg_size() { return sizeof(KinTC); }

// the plane pairs of one problem's x/y or z contraction (the work units)
long long kin_tc_pairs(const bsl_handle* h, bool xy) {
  const Tables& t = h->t;
  return ((long long)(xy ? t.nz : t.ny) * t.nn + 1) / 2;
}

// fill args[b] (kin_group_arg_size() bytes each) for the problems' vectors v[b]
void kin_tc_group_args(bsl_handle** hs, int n, const float2* const* v, bool xy, const int* fin_counts, void* args) {
  KinTC* a = static_cast<KinTC*>(args);
  for (int b = 0; b < n; ++b) a[b] = kin_tc_args(hs[b], v[b], xy, fin_counts ? fin_counts[b] : 0);
}

int launch_kin_tc_group(bool xy, const void* d_args, const int4* d_work, int nctas, cudaStream_t s) {
  const size_t smem = xy ? kSmemXY : kSmemZ;
  if (xy) {
    cudaFuncSetAttribute(k_kin_xy_tc_group, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    BSL_CUDA(launch_pdl(k_kin_xy_tc_group, dim3(nctas), dim3(kWsThreads), smem, s,
                        static_cast<const KinTC*>(d_args), d_work));
  } else {
    cudaFuncSetAttribute(k_kin_z_tc_group, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    BSL_CUDA(launch_pdl(k_kin_z_tc_group, dim3(nctas), dim3(kWsThreads), smem, s,
                        static_cast<const KinTC*>(d_args), d_work));
  }
  return BSL_OK;
}

int launch_kin_xy_tc(bsl_handle* h, const float2* v, cudaStream_t s) {
  cudaFuncSetAttribute(k_kin_xy_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemXY);
  const KinTC a = kin_tc_args(h, v, true, h->defer_reductions ? deferred_beta_count(h) : 0);
  BSL_CUDA(launch_pdl(k_kin_xy_tc, dim3(std::min((a.nplanes + 1) / 2, sm_count())), dim3(kWsThreads), kSmemXY, s, a));
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

int launch_kin_z_tc(bsl_handle* h, const float2* v, cudaStream_t s) {
  cudaFuncSetAttribute(k_kin_z_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemZ);
  const KinTC a = kin_tc_args(h, v, false, 0);
  BSL_CUDA(launch_pdl(k_kin_z_tc, dim3(std::min((a.nplanes + 1) / 2, sm_count())), dim3(kWsThreads), kSmemZ, s, a));
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace bsl
