// wk_spmv_core.cuh -- device building blocks shared by the SpMV kernels and
// the solver kernels: streaming loads with L2 eviction hints, x gathers, and
// the per-warp row sums of a WPK1/WPK2 layout warp.
//
// Layout: layout warp w owns slots [o_w, o_w + 32*A_w); entry i of layout lane
// l sits at o_w + l + 32*i (warpkernel.hpp:65-71, 360-361).  Layout lane l
// belongs to sorted row first_row_w + l / T_w; the T_w lanes of a row are
// summed by a tree (T_w = 1 for WPK1).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <type_traits>

namespace wk {
namespace core {

constexpr int WS = 32;

__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// ---- cp.async: global -> shared copies tracked by commit groups ----------------
// 16 bytes, L2-only (.cg) with an L2 cache-policy hint; both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, uint64_t pol) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(sa), "l"(gmem), "l"(pol)
               : "memory");
}
// N = 4, 8 or 16 bytes through L1 (.ca); both addresses N-byte aligned.
template <int N>
__device__ __forceinline__ void cp_async_ca(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(sa), "l"(gmem), "n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Waits until at most N of this thread's committed groups are pending.
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// ---- streaming loads (matrix), ld.global.nc.L1::no_allocate + evict_first ------
template <typename T>
__device__ __forceinline__ T ld_stream1(const T *p, uint64_t pol);
template <>
__device__ __forceinline__ double ld_stream1(const double *p, uint64_t pol) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
template <>
__device__ __forceinline__ float ld_stream1(const float *p, uint64_t pol) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}
template <>
__device__ __forceinline__ int32_t ld_stream1(const int32_t *p, uint64_t pol) {
  int v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
template <>
__device__ __forceinline__ __nv_bfloat16 ld_stream1(const __nv_bfloat16 *p, uint64_t pol) {
  unsigned short v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(pol));
  return __ushort_as_bfloat16(v);
}

template <>
__device__ __forceinline__ __half ld_stream1(const __half *p, uint64_t pol) {
  unsigned short v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(pol));
  return __ushort_as_half(v);
}

// ---- type traits: value/vector element -> accumulator ------------------------------
template <typename V>
struct Tr;
template <>
struct Tr<double> {
  typedef double Acc;
  static __device__ __forceinline__ double acc(double v) { return v; }
};
template <>
struct Tr<float> {
  typedef float Acc;
  static __device__ __forceinline__ float acc(float v) { return v; }
};
template <>
struct Tr<__nv_bfloat16> {
  typedef float Acc;
  static __device__ __forceinline__ float acc(__nv_bfloat16 v) { return __bfloat162float(v); }
};
// WK_F16S values: FP16 relative to the layout warp's power-of-two scale; the
// kernels sum h * x in FP32 and multiply the row total by the scale (exact).
template <>
struct Tr<__half> {
  typedef float Acc;
  static __device__ __forceinline__ float acc(__half v) { return __half2float(v); }
};
template <typename V>
struct Scaled {
  static constexpr bool value = std::is_same<V, __half>::value;
};

// ---- gathers (x).  `cache` (the reference's texture fetch, fetch_cache<true>
// in warpkernel.hpp:41-49) reads through the non-coherent read-only path
// (ld.global.nc); without it the reference reads x[i] with a plain global
// load, which on sm_103a caches in L1 (ld.global.ca).  (On the Kepler parts
// the reference targeted a plain load bypassed L1; an L2-only gather here
// measured 3.6x slower on split rows, whose lanes revisit the same x sectors
// step after step.)
template <bool L1>
__device__ __forceinline__ double gather(const double *x, int i) { return L1 ? __ldg(x + i) : __ldca(x + i); }
template <bool L1>
__device__ __forceinline__ float gather(const float *x, int i) { return L1 ? __ldg(x + i) : __ldca(x + i); }
template <bool L1>
__device__ __forceinline__ __nv_bfloat16 gather(const __nv_bfloat16 *x, int i) {
  const unsigned short *u = reinterpret_cast<const unsigned short *>(x);
  return __ushort_as_bfloat16(L1 ? __ldg(u + i) : __ldca(u + i));
}

// x gather from global memory (gather<L1>) or, with SX, from an x window
// staged in shared memory (stage_window): x then points at the window and i
// is a window position.
template <bool L1, bool SX, typename X>
__device__ __forceinline__ X gx(const X *__restrict__ x, int i) {
  if constexpr (SX)
    return x[i];
  else
    return gather<L1>(x, i);
}

// Copies a layout warp's x window into shared memory `win` (the warp's
// region, WIN_MAX values): wd = {first chunk, chunks, window size, 0}; chunk
// q = {first column, window position | length << 16} holds at most 32
// consecutive columns and is copied by one warp-wide load (lane j: column
// first + j).  SW chunks' loads are issued before their stores, so a window
// of up to SW chunks costs one round trip to L2.
template <bool L1, typename X, int SW = 16>
__device__ __forceinline__ void stage_window(X *win, const int2 *__restrict__ chunks, int4 wd,
                                             const X *__restrict__ x, uint32_t lane) {
  const int nch = wd.y;
  const int2 mine = lane < (uint32_t)nch ? chunks[wd.x + lane] : make_int2(0, 0);
  for (int q0 = 0; q0 < nch; q0 += SW) {
    X v[SW];
    int dst[SW];
#pragma unroll
    for (int j = 0; j < SW; j++) {
      const int q = q0 + j;
      const int c0 = __shfl_sync(0xffffffffu, mine.x, q & 31);
      const int pl = __shfl_sync(0xffffffffu, mine.y, q & 31);
      const int pos = (pl & 0xffff) + (int)lane;
      const bool ok = q < nch && lane < (uint32_t)(pl >> 16) && pos < WIN_MAX;
      dst[j] = ok ? pos : -1;
      v[j] = ok ? gather<L1>(x, c0 + (int)lane) : X(0.0f);
    }
#pragma unroll
    for (int j = 0; j < SW; j++)
      if (dst[j] >= 0) win[dst[j]] = v[j];
  }
  __syncwarp();
}

// The same copy for 4-byte x by cp.async, one warp-wide copy per chunk in a
// rolled loop, committed as one group: the caller issues its first stream
// loads and then waits (cp_async_wait<0> + __syncwarp) before the first
// gather, so the window's L2 round trip overlaps the stream's.
template <typename X>
__device__ __forceinline__ void stage_window_async(X *win, const int2 *__restrict__ chunks, int4 wd,
                                                   const X *__restrict__ x, uint32_t lane) {
  static_assert(sizeof(X) == 4, "cp.async copies 4-byte x values");
  const int nch = wd.y;
  const int2 mine = lane < (uint32_t)nch ? chunks[wd.x + lane] : make_int2(0, 0);
  for (int q = 0; q < nch; q++) {
    const int c0 = __shfl_sync(0xffffffffu, mine.x, q);
    const int pl = __shfl_sync(0xffffffffu, mine.y, q);
    const int pos = (pl & 0xffff) + (int)lane;
    if (lane < (uint32_t)(pl >> 16) && pos < WIN_MAX) cp_async_ca<4>(win + pos, x + c0 + (int)lane);
  }
  cp_async_commit();
}

__device__ __forceinline__ double fma_acc(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_acc(float a, float b, float c) { return fmaf(a, b, c); }

// Tree over the T lanes of a row: lockstep semantics of warpkernel.hpp:157-162,
// i.e. s_l <- s_l + s_{l+k} for k = 1, 2, 4, ... (all reads before writes).
template <typename Acc>
__device__ __forceinline__ Acc row_tree(Acc s, uint32_t T) {
  for (uint32_t k = 1; k < T; k <<= 1) s += __shfl_down_sync(0xffffffffu, s, k);
  return s;
}

// Exact order: layout lane `lane` sums its slots first product, then fma per
// step (warpkernel.hpp:147-153).  Returns 0 for lanes of absent rows.
template <typename V, typename X, bool L1>
__device__ __forceinline__ typename Tr<V>::Acc lane_sum_exact(const V *__restrict__ pv,
                                                             const int32_t *__restrict__ pc, int4 d,
                                                             const X *__restrict__ x, uint32_t lane,
                                                             bool valid) {
  typedef typename Tr<V>::Acc Acc;
  Acc s = Acc(0);
  if (valid) {
    size_t o = (size_t)(uint32_t)d.x + lane;
    const size_t end = o + (size_t)WS * (uint32_t)d.y;
    if constexpr (sizeof(V) == 8 || Scaled<V>::value) {
      // 8-byte values and scaled FP16 (FP32 x): streaming loads with
      // evict_first measured up to 25 % faster (hex 64^3, 2-D Q1 1024^2);
      // for fp32 and bf16 the plain loads were faster (up to 33 %), so those
      // keep them.
      const uint64_t pol = policy_evict_first();
      s = Tr<V>::acc(ld_stream1(pv + o, pol)) * (Acc)Tr<X>::acc(gather<L1>(x, ld_stream1(pc + o, pol)));
      for (o += WS; o < end; o += WS)
        s = fma_acc(Tr<V>::acc(ld_stream1(pv + o, pol)), (Acc)Tr<X>::acc(gather<L1>(x, ld_stream1(pc + o, pol))), s);
    } else {
      s = Tr<V>::acc(pv[o]) * (Acc)Tr<X>::acc(gather<L1>(x, pc[o]));
      for (o += WS; o < end; o += WS) s = fma_acc(Tr<V>::acc(pv[o]), (Acc)Tr<X>::acc(gather<L1>(x, pc[o])), s);
    }
  }
  return s;
}

// ---- word loads (streaming) and unpacking ----------------------------------------
__device__ __forceinline__ void ld_words(const void *p, uint32_t (&w)[1], uint64_t pol) {
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(w[0]) : "l"(p), "l"(pol));
}
__device__ __forceinline__ void ld_words(const void *p, uint32_t (&w)[2], uint64_t pol) {
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.b32 {%0,%1}, [%2], %3;"
               : "=r"(w[0]), "=r"(w[1])
               : "l"(p), "l"(pol));
}
__device__ __forceinline__ void ld_words(const void *p, uint32_t (&w)[4], uint64_t pol) {
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.b32 {%0,%1,%2,%3}, [%4], %5;"
               : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3])
               : "l"(p), "l"(pol));
}
__device__ __forceinline__ void ld_words(const void *p, uint32_t (&w)[8], uint64_t pol) {
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
               : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
               : "l"(p), "l"(pol));
}
__device__ __forceinline__ void ld_words(const void *p, uint32_t (&w)[16], uint64_t pol) {
  ld_words(p, *reinterpret_cast<uint32_t(*)[8]>(&w[0]), pol);
  ld_words((const char *)p + 32, *reinterpret_cast<uint32_t(*)[8]>(&w[8]), pol);
}
template <typename V>
__device__ __forceinline__ V word_val(const uint32_t *w, int k);
template <>
__device__ __forceinline__ double word_val<double>(const uint32_t *w, int k) {
  return __hiloint2double((int)w[2 * k + 1], (int)w[2 * k]);
}
template <>
__device__ __forceinline__ float word_val<float>(const uint32_t *w, int k) {
  return __uint_as_float(w[k]);
}
template <>
__device__ __forceinline__ __nv_bfloat16 word_val<__nv_bfloat16>(const uint32_t *w, int k) {
  return __ushort_as_bfloat16((unsigned short)((k & 1) ? (w[k >> 1] >> 16) : (w[k >> 1] & 0xffffu)));
}
template <>
__device__ __forceinline__ __half word_val<__half>(const uint32_t *w, int k) {
  return __ushort_as_half((unsigned short)((k & 1) ? (w[k >> 1] >> 16) : (w[k >> 1] & 0xffffu)));
}
template <typename C>
__device__ __forceinline__ int word_col(const uint32_t *w, int k, int base);
template <>
__device__ __forceinline__ int word_col<int32_t>(const uint32_t *w, int k, int) {
  return (int)w[k];
}
template <>
__device__ __forceinline__ int word_col<uint16_t>(const uint32_t *w, int k, int base) {
  return base + (int)((k & 1) ? (w[k >> 1] >> 16) : (w[k >> 1] & 0xffffu));
}
__device__ __forceinline__ int ld_col1(const int32_t *p, int, uint64_t pol) { return ld_stream1(p, pol); }
__device__ __forceinline__ int ld_col1(const uint16_t *p, int base, uint64_t pol) {
  unsigned short v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(pol));
  return base + (int)v;
}

// Base slots per lane and iteration: 32 B of values for fp64 (4 slots), 32 B
// for fp32 and 16 B for 2-byte values (8 slots).  The adjoint and the CG's
// SpMV-dot use it as is; VecPlan below adjusts it for wk_run.
template <typename V>
struct SlotsPerLane {
  static constexpr int value = sizeof(V) == 8 ? 4 : 8;
};
// Per (value, column) type: slots per lane and whether the next unit's
// loads are issued before this unit's gathers (software pipelining), chosen
// by measurement on hex 96^3 (3 dof) on four GB300s.  bf16 streams 16 slots
// per lane (32 B of values, 256-bit loads): 3 % faster with 32-bit columns,
// 1-11 % with 16-bit ones, and the same slot count for both column types
// keeps their sums bit-identical.  fp32 with 32-bit columns is pipelined
// (3 % faster on every box).  Pipelining the other forms was faster on some
// boxes and slower on others, so they keep the plain loop.
template <typename V, typename C>
struct VecPlan {
  static constexpr int slots =
      (std::is_same<V, __nv_bfloat16>::value || std::is_same<V, __half>::value) ? 16 : SlotsPerLane<V>::value;
  // units unrolled in the plain loop: fp64 runs 1.3 % faster with 1 (2 and 3
  // unrolled units cost registers and 1-6 %) except on layouts of long warps,
  // where k_spmv_fast overrides it with 2; bf16 with 16-bit columns lost 2 %
  // with 4, so the others keep 2.  Scaled FP16 takes 16 slots per lane like
  // bf16 (32-byte value loads): with 16-bit columns 3.6 % faster than 8 slots
  // with 4 units unrolled, 0.5 % slower with 32-bit columns.
  static constexpr int unroll = sizeof(V) == 8 ? 1 : 2;
  static constexpr bool pipelined = sizeof(V) == 4 && sizeof(C) == 4;
};
// The CG's SpMV-dot (FP32 p for every narrow value type, plus the dot
// product) keeps the base slot count and the plain loop: the plan above
// raised its registers from 40-48 to 64 and slowed the FP32 / bf16 inner
// solves by 4 %.  fp64 runs without unrolling, as above (1.4 % per CG
// iteration).
template <typename V, typename C>
struct PlainPlan {
  static constexpr int slots = SlotsPerLane<V>::value;
  static constexpr int unroll = sizeof(V) == 8 ? 1 : 2;
  static constexpr bool pipelined = false;
};

// Cross-lane combine of the vector path.  Lane j holds S partial sums a[k]
// for layout lanes S*(j%R)+k (R = 32/S); the S lanes j%R + R*q (q < S) hold
// the same layout lanes.  Reduce-scatter: in round r the lanes pair across
// xor distance R<<r, each keeps half of its accumulators and adds its
// partner's copies of them (the pairs and their order are those of a
// butterfly over the same distances, so the sums are the same bits), so a
// lane ends with the total of one layout lane after S-1 additions instead of
// S*log2(S).  Lane j then holds layout lane S*(j%R) + brev(j/R) (brev over
// log2(S) bits); one shuffle moves each total to its owning lane.  Returns
// layout lane `lane`'s total.
template <int S, typename Acc>
__device__ __forceinline__ Acc combine_lanes(Acc (&a)[S], uint32_t lane) {
  constexpr int R = 32 / S;
  constexpr int LOG = S == 2 ? 1 : S == 4 ? 2 : S == 8 ? 3 : S == 16 ? 4 : 5;
  static_assert((1 << LOG) == S, "S must be a power of two up to 32");
#pragma unroll
  for (int r = 0; r < LOG; r++) {
    const int n = S >> r, dist = R << r;
    const bool hi = ((lane / (uint32_t)dist) & 1u) != 0;
#pragma unroll
    for (int k = 0; k < n / 2; k++) {
      const Acc send = hi ? a[k] : a[k + n / 2];
      const Acc keep = hi ? a[k + n / 2] : a[k];
      a[k] = keep + __shfl_xor_sync(0xffffffffu, send, dist);
    }
  }
  const uint32_t src = lane / S + R * (__brev(lane % S) >> (32 - LOG));
  return __shfl_sync(0xffffffffu, a[0], (int)src);
}

// Block sum of one value per thread for kernels that share GB300's FP64
// pipe with their DFMAs: the values go to shared memory (sh: NT values) and
// warp 0 adds NT / 32 of them per lane, then a shuffle tree -- 3 + 5 FP64
// warp instructions for NT = 128 instead of 25 for a tree in every warp (the
// per-warp trees cost 5 % of a CG iteration at hex 96^3).  Fixed order; the
// result is valid in thread 0.
template <int NT, typename T = double>
__device__ __forceinline__ T block_sum_staged(T v, T *sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  T t = T(0);
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    t = sh[lane];
#pragma unroll
    for (int k = 1; k < NT / 32; k++) t += sh[lane + 32 * k];
#pragma unroll
    for (int off = 16; off; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  }
  return t;
}

// Fast order: with S slots per lane, a unit of S steps is 32*S consecutive
// slots; lane j streams slots S*j .. S*j+S-1 (layout lanes S*(j%R) .. +S-1 at
// step j/R, R = 32/S) with one vector load of values and one of columns.
// Partials are combined across the S lanes holding the same layout lanes
// (combine_lanes) and moved to the owning lane, whose FMA chain then takes
// the A_w % S remaining steps one slot per lane.  Returns layout lane
// `lane`'s total.
// cp0 points at the warp's first column entry (slot o_w of a slot-indexed
// array, or the warp's start in a compact array); base is added to 16-bit
// offsets.
// UNR (if non-zero) replaces the plan's unroll factor.  SX: x is the warp's
// x window in shared memory and the columns are window positions (base 0).
struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};
template <typename V, typename X, bool L1, typename C, bool TUNED = true, int UNR = 0, bool SX = false,
          typename Hook = NoHook>
__device__ __forceinline__ typename Tr<V>::Acc lane_sum_vec(const V *__restrict__ pv, const C *__restrict__ cp0, int base,
                                                           int4 d, const X *__restrict__ x, uint32_t lane,
                                                           uint64_t pol, Hook hook = Hook()) {
  typedef typename Tr<V>::Acc Acc;
  typedef typename std::conditional<TUNED, VecPlan<V, C>, PlainPlan<V, C>>::type Plan;
  constexpr int S = Plan::slots;
  constexpr int NWV = S * (int)sizeof(V) / 4, NWC = S * (int)sizeof(C) / 4;
  const uint32_t A = (uint32_t)d.y;
  const size_t o = (size_t)(uint32_t)d.x;
  const uint32_t units = A / S, rem = A % S;
  Acc a[S];
#pragma unroll
  for (int k = 0; k < S; k++) a[k] = Acc(0);
  const V *vp = pv + o + S * lane;
  const C *cp = cp0 + S * lane;
  if constexpr (Plan::pipelined) {
    uint32_t wv[NWV], wc[NWC];
    if (units) {
      ld_words(vp, wv, pol);
      ld_words(cp, wc, pol);
    }
#pragma unroll 1
    for (uint32_t u = 0; u < units; u++) {
      uint32_t nv[NWV], nc[NWC];
      if (u + 1 < units) {
        ld_words(vp + S * WS, nv, pol);
        ld_words(cp + S * WS, nc, pol);
      }
#pragma unroll
      for (int k = 0; k < S; k++)
        a[k] = fma_acc(Tr<V>::acc(word_val<V>(wv, k)), (Acc)Tr<X>::acc(gx<L1, SX>(x, word_col<C>(wc, k, base))), a[k]);
#pragma unroll
      for (int q = 0; q < NWV; q++) wv[q] = nv[q];
#pragma unroll
      for (int q = 0; q < NWC; q++) wc[q] = nc[q];
      vp += S * WS;
      cp += S * WS;
    }
  } else {
    constexpr int U = UNR ? UNR : Plan::unroll;
#pragma unroll U
  for (uint32_t u = 0; u < units; u++) {
    uint32_t wv[NWV], wc[NWC];
    ld_words(vp, wv, pol);
    ld_words(cp, wc, pol);
    if (u == 0) hook();  // e.g. completing the x window, once the first unit's loads are in flight
#pragma unroll
    for (int k = 0; k < S; k++)
      a[k] = fma_acc(Tr<V>::acc(word_val<V>(wv, k)), (Acc)Tr<X>::acc(gx<L1, SX>(x, word_col<C>(wc, k, base))), a[k]);
    vp += S * WS;
    cp += S * WS;
  }
  }
  // the A_w % S remaining steps continue the combined total's FMA chain (no
  // separate tail sum to add: one FP64 add less per lane on GB300's FP64
  // pipe).  With 4 slots per lane (fp64) their operands are loaded before the
  // combine, whose shuffles then overlap the loads: loading them after it
  // made layouts of long warps 15 % slower; with 8 slots the 14 preloaded
  // registers made scaled FP16 with 16-bit columns (then on 8 slots) 10 %
  // slower.
  if (units == 0) hook();
  const size_t ut = (size_t)units * S * WS + lane;
  if constexpr (S <= 4) {
    Acc tv[S - 1], tx[S - 1];
#pragma unroll
    for (int i = 0; i < S - 1; i++) {
      tv[i] = Acc(0);
      tx[i] = Acc(0);
      if ((uint32_t)i < rem) {
        const size_t k = ut + (size_t)i * WS;
        tv[i] = Tr<V>::acc(ld_stream1(pv + o + k, pol));
        tx[i] = (Acc)Tr<X>::acc(gx<L1, SX>(x, ld_col1(cp0 + k, base, pol)));
      }
    }
    Acc s = combine_lanes<S>(a, lane);
#pragma unroll
    for (int i = 0; i < S - 1; i++)
      if ((uint32_t)i < rem) s = fma_acc(tv[i], tx[i], s);
    return s;
  } else if constexpr (S <= 8) {
    Acc s = combine_lanes<S>(a, lane);
    for (uint32_t i = 0; i < rem; i++) {
      const int c = ld_col1(cp0 + ut + (size_t)i * WS, base, pol);
      s = fma_acc(Tr<V>::acc(ld_stream1(pv + o + ut + (size_t)i * WS, pol)), (Acc)Tr<X>::acc(gx<L1, SX>(x, c)), s);
    }
    return s;
  } else {
    // 16 slots per lane (bf16, scaled FP16): the tail can be up to 15 steps, so it is summed
    // before the combine (its loads overlap the combine's shuffles) and added
    // after it -- an FP32 add, not one on the FP64 pipe; 5-9 % faster on
    // layouts of 27-41 steps (with 8 slots the fold measured faster for fp32)
    Acc tail = Acc(0);
    for (uint32_t i = 0; i < rem; i++) {
      const int c = ld_col1(cp0 + ut + (size_t)i * WS, base, pol);
      tail = fma_acc(Tr<V>::acc(ld_stream1(pv + o + ut + (size_t)i * WS, pol)), (Acc)Tr<X>::acc(gx<L1, SX>(x, c)), tail);
    }
    return combine_lanes<S>(a, lane) + tail;
  }
}

template <typename V, typename X, bool L1, bool TUNED = true, int UNR = 0>
__device__ __forceinline__ typename Tr<V>::Acc lane_sum_fast(const V *__restrict__ pv, const int32_t *__restrict__ pc,
                                                            int4 d, const X *__restrict__ x, uint32_t lane,
                                                            uint64_t pol) {
  return lane_sum_vec<V, X, L1, int32_t, TUNED, UNR>(pv, pc + (uint32_t)d.x, 0, d, x, lane, pol);
}

// ---- compressed column indices ---------------------------------------------------
// A layout warp whose column indices span less than 65,536 stores them as
// 16-bit offsets from a per-warp base (2 bytes per slot instead of 4); other
// warps keep 32-bit indices in a compact side array.  cdesc = {base, mode
// (0 = 16-bit, 1 = 32-bit), offset of the warp in the 32-bit array, 0}.
template <typename V, typename X, bool L1, bool TUNED = true>
__device__ __forceinline__ typename Tr<V>::Acc lane_sum_compressed(const V *__restrict__ pv,
                                                                  const uint16_t *__restrict__ c16,
                                                                  const int32_t *__restrict__ c32, int4 d,
                                                                  int4 cd, const X *__restrict__ x,
                                                                  uint32_t lane, uint64_t pol) {
  if (cd.y == 0) return lane_sum_vec<V, X, L1, uint16_t, TUNED>(pv, c16 + (uint32_t)d.x, cd.x, d, x, lane, pol);
  return lane_sum_vec<V, X, L1, int32_t, TUNED>(pv, c32 + (uint32_t)cd.z, 0, d, x, lane, pol);
}

}  // namespace core
}  // namespace wk
