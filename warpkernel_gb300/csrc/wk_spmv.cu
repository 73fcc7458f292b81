// wk_spmv.cu -- WPK1/WPK2 SpMV kernels for sm_103a (engine::run / run_x).
//
// Layout (from the scan): layout warp w owns slots [o_w, o_w + 32*A_w); entry
// i of layout lane l sits at o_w + l + 32*i (warpkernel.hpp:65-71, 360-361).
// Layout lane l belongs to sorted row row_start_w + l / T_w, and the T_w lanes
// of a row are summed by a tree (T_w = 1 for WPK1).
//
// Two kernels per configuration:
//  * exact: one slot per lane per step in the reference's order
//    (first product, then fma per step, then the tree) -- bit-identical to the
//    oracle and to the reference kernels compiled with contraction;
//  * fast: each lane streams 4 consecutive slots of a 4-step unit with one
//    256-bit value load (fp64) or 128-bit load (fp32) and one 128-bit column
//    load, so a warp moves 128 slots per iteration with two memory
//    instructions.  Slot 4j..4j+3 of a unit belongs to layout lanes
//    4(j%8)..4(j%8)+3 at step j/8; per-lane partials are combined across the
//    four lanes holding the same layout lanes (xor 8, xor 16) and moved to the
//    owning lane with four shuffles.  This re-associates each row's sum.
// The matrix stream is loaded with ld.global.nc.L1::no_allocate and an
// L2 evict_first policy so that x (gathered through L1 with cache != 0, or L2
// only with cache == 0) stays resident in L2.
#include <cuda_bf16.h>

#include "wk_internal.cuh"

namespace wk {
namespace {

constexpr int WS = 32;

__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// ---- streaming loads (matrix) ----------------------------------------------------
__device__ __forceinline__ void ld_stream(const double *p, double (&v)[4], uint64_t pol) {
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f64 {%0,%1,%2,%3}, [%4], %5;"
               : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3])
               : "l"(p), "l"(pol));
}
__device__ __forceinline__ void ld_stream(const float *p, float (&v)[4], uint64_t pol) {
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
               : "l"(p), "l"(pol));
}
__device__ __forceinline__ void ld_stream(const __nv_bfloat16 *p, __nv_bfloat16 (&v)[4], uint64_t pol) {
  unsigned a, b;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.b32 {%0,%1}, [%2], %3;"
               : "=r"(a), "=r"(b)
               : "l"(p), "l"(pol));
  v[0] = __ushort_as_bfloat16((unsigned short)(a & 0xffffu));
  v[1] = __ushort_as_bfloat16((unsigned short)(a >> 16));
  v[2] = __ushort_as_bfloat16((unsigned short)(b & 0xffffu));
  v[3] = __ushort_as_bfloat16((unsigned short)(b >> 16));
}
__device__ __forceinline__ void ld_stream4(const int32_t *p, int (&c)[4], uint64_t pol) {
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.s32 {%0,%1,%2,%3}, [%4], %5;"
               : "=r"(c[0]), "=r"(c[1]), "=r"(c[2]), "=r"(c[3])
               : "l"(p), "l"(pol));
}
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

// ---- gathers (x) -------------------------------------------------------------------
template <bool L1, typename T>
__device__ __forceinline__ T gather(const T *x, int i) {
  if (L1) return __ldg(x + i);
  return __ldcg(x + i);
}
template <bool L1>
__device__ __forceinline__ __nv_bfloat16 gather(const __nv_bfloat16 *x, int i) {
  const unsigned short *u = reinterpret_cast<const unsigned short *>(x);
  return __ushort_as_bfloat16(L1 ? __ldg(u + i) : __ldcg(u + i));
}

// Type traits: storage V, accumulator Acc, output Y.
template <typename V>
struct Tr;
template <>
struct Tr<double> {
  typedef double Acc;
  typedef double Y;
  static __device__ __forceinline__ double acc(double v) { return v; }
};
template <>
struct Tr<float> {
  typedef float Acc;
  typedef float Y;
  static __device__ __forceinline__ float acc(float v) { return v; }
};
template <>
struct Tr<__nv_bfloat16> {
  typedef float Acc;
  typedef float Y;
  static __device__ __forceinline__ float acc(__nv_bfloat16 v) { return __bfloat162float(v); }
};

__device__ __forceinline__ double fma_acc(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_acc(float a, float b, float c) { return fmaf(a, b, c); }

// Tree over the T lanes of a row, lockstep semantics of warpkernel.hpp:157-162.
template <typename Acc>
__device__ __forceinline__ Acc row_tree(Acc s, uint32_t T) {
  for (uint32_t k = 1; k < T; k <<= 1) s += __shfl_down_sync(0xffffffffu, s, k);
  return s;
}

template <typename V, bool MAPPED>
__device__ __forceinline__ void store_row(typename Tr<V>::Y *y, const int32_t *row_map, uint32_t p,
                                          typename Tr<V>::Acc s) {
  if (MAPPED)
    y[row_map[p]] = (typename Tr<V>::Y)s;
  else
    y[p] = (typename Tr<V>::Y)s;
}

// ------------------------------------------------------------------------------------
// Exact-order kernel.
// ------------------------------------------------------------------------------------
template <typename V, bool MAPPED, bool L1>
__global__ void __launch_bounds__(1024) k_spmv_exact(const V *__restrict__ pv, const int32_t *__restrict__ pc,
                                                     const int4 *__restrict__ desc, uint32_t W,
                                                     const int32_t *__restrict__ row_map, uint32_t nzr,
                                                     const V *__restrict__ x, typename Tr<V>::Y *__restrict__ y) {
  typedef typename Tr<V>::Acc Acc;
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w >= W) return;
  const int4 d = desc[w];
  const uint32_t T = (uint32_t)d.z;
  const uint32_t p = (uint32_t)d.w + lane / T;
  const bool valid = p < nzr;
  Acc s = Acc(0);
  if (valid) {
    size_t o = (size_t)(uint32_t)d.x + lane;
    const size_t end = o + (size_t)WS * (uint32_t)d.y;
    s = Tr<V>::acc(pv[o]) * Tr<V>::acc(gather<L1>(x, pc[o]));
    for (o += WS; o < end; o += WS) s = fma_acc(Tr<V>::acc(pv[o]), Tr<V>::acc(gather<L1>(x, pc[o])), s);
  }
  s = row_tree<Acc>(s, T);
  if (valid && (lane & (T - 1)) == 0) store_row<V, MAPPED>(y, row_map, p, s);
}

// ------------------------------------------------------------------------------------
// Fast kernel: 4 slots per lane per iteration.
// ------------------------------------------------------------------------------------
template <typename V, bool MAPPED, bool L1>
__global__ void __launch_bounds__(1024) k_spmv_fast(const V *__restrict__ pv, const int32_t *__restrict__ pc,
                                                    const int4 *__restrict__ desc, uint32_t W,
                                                    const int32_t *__restrict__ row_map, uint32_t nzr,
                                                    const V *__restrict__ x, typename Tr<V>::Y *__restrict__ y) {
  typedef typename Tr<V>::Acc Acc;
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w >= W) return;
  const uint64_t pol = policy_evict_first();
  const int4 d = desc[w];
  const uint32_t A = (uint32_t)d.y, T = (uint32_t)d.z;
  const size_t o = (size_t)(uint32_t)d.x;
  const uint32_t units = A >> 2, rem = A & 3u;

  Acc a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  const V *vp = pv + o + 4 * lane;
  const int32_t *cp = pc + o + 4 * lane;
#pragma unroll 2
  for (uint32_t u = 0; u < units; u++) {
    V v[4];
    int c[4];
    ld_stream(vp, v, pol);
    ld_stream4(cp, c, pol);
    a0 = fma_acc(Tr<V>::acc(v[0]), Tr<V>::acc(gather<L1>(x, c[0])), a0);
    a1 = fma_acc(Tr<V>::acc(v[1]), Tr<V>::acc(gather<L1>(x, c[1])), a1);
    a2 = fma_acc(Tr<V>::acc(v[2]), Tr<V>::acc(gather<L1>(x, c[2])), a2);
    a3 = fma_acc(Tr<V>::acc(v[3]), Tr<V>::acc(gather<L1>(x, c[3])), a3);
    vp += 4 * WS;
    cp += 4 * WS;
  }
  // combine the four lanes that hold the same layout lanes
  a0 += __shfl_xor_sync(0xffffffffu, a0, 8);
  a1 += __shfl_xor_sync(0xffffffffu, a1, 8);
  a2 += __shfl_xor_sync(0xffffffffu, a2, 8);
  a3 += __shfl_xor_sync(0xffffffffu, a3, 8);
  a0 += __shfl_xor_sync(0xffffffffu, a0, 16);
  a1 += __shfl_xor_sync(0xffffffffu, a1, 16);
  a2 += __shfl_xor_sync(0xffffffffu, a2, 16);
  a3 += __shfl_xor_sync(0xffffffffu, a3, 16);
  // layout lane `lane` = register lane%4 of lane lane/4
  const int src = (int)(lane >> 2);
  Acc t0 = __shfl_sync(0xffffffffu, a0, src);
  Acc t1 = __shfl_sync(0xffffffffu, a1, src);
  Acc t2 = __shfl_sync(0xffffffffu, a2, src);
  Acc t3 = __shfl_sync(0xffffffffu, a3, src);
  const uint32_t k = lane & 3u;
  Acc s = k == 0 ? t0 : k == 1 ? t1 : k == 2 ? t2 : t3;
  // remaining steps, one slot per lane
  size_t ot = o + (size_t)units * 4 * WS + lane;
  for (uint32_t i = 0; i < rem; i++, ot += WS)
    s = fma_acc(Tr<V>::acc(ld_stream1(pv + ot, pol)), Tr<V>::acc(gather<L1>(x, ld_stream1(pc + ot, pol))), s);

  const uint32_t p = (uint32_t)d.w + lane / T;
  s = row_tree<Acc>(s, T);
  if (p < nzr && (lane & (T - 1)) == 0) store_row<V, MAPPED>(y, row_map, p, s);
}

template <typename V>
wk_status dispatch(const RunArgs &a, unsigned grid, unsigned block) {
  const wk_engine *e = a.e;
  const wk_layout *l = e->layout;
  const V *pv = e->vals.as<V>();
  const int32_t *pc = e->cols.as<int32_t>();
  const V *x = (const V *)a.x;
  typename Tr<V>::Y *y = (typename Tr<V>::Y *)a.y;
  const int4 *desc = l->d.warp_desc;
  const int32_t *rm = l->d.row_map;
  const uint32_t W = l->info.nwarps, nzr = l->info.nznrows;
#define WK_LAUNCH(K, M, C) K<V, M, C><<<grid, block, 0, a.stream>>>(pv, pc, desc, W, rm, nzr, x, y)
  const bool c = a.cache != 0;
  if (a.order == WK_ORDER_EXACT) {
    if (a.mapped) {
      if (c) WK_LAUNCH(k_spmv_exact, true, true); else WK_LAUNCH(k_spmv_exact, true, false);
    } else {
      if (c) WK_LAUNCH(k_spmv_exact, false, true); else WK_LAUNCH(k_spmv_exact, false, false);
    }
  } else {
    if (a.mapped) {
      if (c) WK_LAUNCH(k_spmv_fast, true, true); else WK_LAUNCH(k_spmv_fast, true, false);
    } else {
      if (c) WK_LAUNCH(k_spmv_fast, false, true); else WK_LAUNCH(k_spmv_fast, false, false);
    }
  }
#undef WK_LAUNCH
  WK_CHECK_LAUNCH();
  return WK_OK;
}

}  // namespace

wk_status launch_spmv(const RunArgs &a) {
  const wk_layout *l = a.e->layout;
  const uint32_t W = l->info.nwarps;
  int block = a.blocksize, nblocks = a.nblocks;
  if (block <= 0 || nblocks <= 0) {
    block = 256;
    nblocks = 0;
  }
  if (block % WS != 0 || block > 1024)
    return set_error(WK_ERR_INVALID, "blocksize %d is not a multiple of 32 in [32, 1024]", block);
  const uint32_t wpb = (uint32_t)block / WS;
  const size_t need = (W + wpb - 1) / wpb;
  if (nblocks == 0) nblocks = (int)(need ? need : 1);
  if ((size_t)nblocks < need)
    return set_error(WK_ERR_INVALID,
                     "nblocks = %d covers %zu warps but the layout has %u (need >= %zu blocks of %d)",
                     nblocks, (size_t)nblocks * wpb, W, need, block);
  if (W == 0) return WK_OK;
  switch (a.e->dtype) {
    case WK_F64: return dispatch<double>(a, (unsigned)nblocks, (unsigned)block);
    case WK_F32: return dispatch<float>(a, (unsigned)nblocks, (unsigned)block);
    case WK_BF16: return dispatch<__nv_bfloat16>(a, (unsigned)nblocks, (unsigned)block);
  }
  return set_error(WK_ERR_INVALID, "unknown dtype %d", a.e->dtype);
}

}  // namespace wk
