// wk_spmv.cu -- WPK1/WPK2 SpMV kernels for sm_103a (engine::run / run_x).
//
// Two kernels per configuration (building blocks in wk_spmv_core.cuh):
//  * exact: one slot per lane per step in the reference's order (first
//    product, then fma per step, then the tree) -- bit-identical to the oracle
//    and to the reference kernels compiled with contraction;
//  * fast: several slots per lane per iteration (VecPlan: 4 for fp64, 8 for
//    fp32, 16 for bf16 and scaled FP16) with 256/128-bit loads, rows
//    re-associated.
// The matrix stream is loaded with ld.global.nc.L1::no_allocate and an L2
// evict_first policy so that x (gathered with ld.global.nc with cache != 0,
// ld.global.ca with cache == 0) stays resident in L2.  One warp per layout
// warp.
#include "wk_internal.cuh"
#include "wk_spmv_core.cuh"

namespace wk {
namespace {

using namespace core;

template <typename Acc, bool MAPPED>
__device__ __forceinline__ void store_row(Acc *y, const int32_t *row_map, uint32_t p, Acc s) {
  if (MAPPED)
    y[row_map[p]] = s;
  else
    y[p] = s;
}

template <typename V, typename X, bool MAPPED, bool L1>
__global__ void __launch_bounds__(1024) k_spmv_exact(const V *__restrict__ pv, const int32_t *__restrict__ pc,
                                                     const int4 *__restrict__ desc, uint32_t W,
                                                     const int32_t *__restrict__ row_map, uint32_t nzr,
                                                     const X *__restrict__ x, typename Tr<V>::Acc *__restrict__ y,
                                                     const float *__restrict__ wscale) {
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w >= W) return;
  const int4 d = desc[w];
  const uint32_t T = (uint32_t)d.z;
  const uint32_t p = (uint32_t)d.w + lane / T;
  const bool valid = p < nzr;
  typename Tr<V>::Acc s = lane_sum_exact<V, X, L1>(pv, pc, d, x, lane, valid);
  s = row_tree(s, T);
  if constexpr (Scaled<V>::value) s *= wscale[w];
  if (valid && (lane & (T - 1)) == 0) store_row<typename Tr<V>::Acc, MAPPED>(y, row_map, p, s);
}

// UNR: unroll factor replacing the plan's (0: the plan's), for layouts of
// long warps (long_warps): fp64 takes 2 there.
template <typename V, typename X, bool MAPPED, bool L1, int UNR = 0>
__global__ void __launch_bounds__(1024) k_spmv_fast(const V *__restrict__ pv, const int32_t *__restrict__ pc,
                                                    const int4 *__restrict__ desc, uint32_t W,
                                                    const int32_t *__restrict__ row_map, uint32_t nzr,
                                                    const X *__restrict__ x, typename Tr<V>::Acc *__restrict__ y,
                                                    const float *__restrict__ wscale) {
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w >= W) return;
  const int4 d = desc[w];
  const uint32_t T = (uint32_t)d.z;
  typename Tr<V>::Acc s = lane_sum_fast<V, X, L1, true, UNR>(pv, pc, d, x, lane, policy_evict_first());
  const uint32_t p = (uint32_t)d.w + lane / T;
  s = row_tree(s, T);
  if constexpr (Scaled<V>::value) s *= wscale[w];
  if (p < nzr && (lane & (T - 1)) == 0) store_row<typename Tr<V>::Acc, MAPPED>(y, row_map, p, s);
}

// warpKernel_nocoalesced (optimization.cu:91-114) for the non-interleaved
// ablation layout: lane l of a WPK1 warp owns slots o + l * A ... o + l * A +
// A - 1 and sums them in order (first product, then fma).  Neighbouring lanes
// read addresses A slots apart, so a warp load touches up to 32 sectors.
template <typename V, typename X, bool MAPPED, bool L1>
__global__ void __launch_bounds__(1024) k_spmv_nocoal(const V *__restrict__ pv, const int32_t *__restrict__ pc,
                                                      const int4 *__restrict__ desc, uint32_t W,
                                                      const int32_t *__restrict__ row_map, uint32_t nzr,
                                                      const X *__restrict__ x, typename Tr<V>::Acc *__restrict__ y,
                                                      const float *__restrict__ wscale) {
  typedef typename Tr<V>::Acc Acc;
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w >= W) return;
  const int4 d = desc[w];
  const uint32_t p = (uint32_t)d.w + lane;
  if (p >= nzr) return;
  const uint32_t A = (uint32_t)d.y;
  const size_t o = (size_t)(uint32_t)d.x + (size_t)lane * A;
  Acc s = Tr<V>::acc(pv[o]) * (Acc)Tr<X>::acc(gather<L1>(x, pc[o]));
  for (uint32_t i = 1; i < A; i++)
    s = fma_acc(Tr<V>::acc(pv[o + i]), (Acc)Tr<X>::acc(gather<L1>(x, pc[o + i])), s);
  if constexpr (Scaled<V>::value) s *= wscale[w];
  store_row<Acc, MAPPED>(y, row_map, p, s);
}

// Fast order with the 16-bit column storage of wk_engine_compress_cols.  With
// WIN (dynamic shared memory of WIN_MAX x values per warp of the block), the
// warps that have an x window stage it in shared memory and gather from
// there; the sums are the same bits as without.
template <typename V, typename X, bool MAPPED, bool L1, bool WIN>
__global__ void __launch_bounds__(1024) k_spmv_fast_c(const V *__restrict__ pv, const uint16_t *__restrict__ c16,
                                                      const int32_t *__restrict__ c32, const int4 *__restrict__ cdesc,
                                                      const uint16_t *__restrict__ w16, const int2 *__restrict__ wch,
                                                      const int4 *__restrict__ wdesc,
                                                      const int4 *__restrict__ desc, uint32_t W,
                                                      const int32_t *__restrict__ row_map, uint32_t nzr,
                                                      const X *__restrict__ x, typename Tr<V>::Acc *__restrict__ y,
                                                      const float *__restrict__ wscale) {
  extern __shared__ __align__(16) unsigned char wk_dyn_smem[];
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w >= W) return;
  const int4 d = desc[w];
  const uint32_t T = (uint32_t)d.z;
  typename Tr<V>::Acc s;
  const uint64_t pol = policy_evict_first();
  int4 wd = make_int4(0, 0, 0, 0);
  if constexpr (WIN) wd = wdesc[w];
  if (WIN && wd.y != 0) {
    X *win = reinterpret_cast<X *>(wk_dyn_smem) + (threadIdx.x / WS) * WIN_MAX;
    // 4-byte x: the window is copied asynchronously and waited for once the
    // first unit's loads are in flight; 2-byte x (no cp.async of that size)
    // is staged by the warp's loads and stores first
    if constexpr (sizeof(X) == 4) {
      stage_window_async(win, wch, wd, x, lane);
      s = lane_sum_vec<V, X, L1, uint16_t, true, 0, true>(pv, w16 + (uint32_t)d.x, 0, d, win, lane, pol, [] {
        cp_async_wait<0>();
        __syncwarp();
      });
    } else {  // staged in four-chunk rounds once the first loads were out: 0.179 ms against 0.158 (bf16, hex 96^3)
      stage_window<L1>(win, wch, wd, x, lane);
      s = lane_sum_vec<V, X, L1, uint16_t, true, 0, true>(pv, w16 + (uint32_t)d.x, 0, d, win, lane, pol);
    }
  } else {
    s = lane_sum_compressed<V, X, L1>(pv, c16, c32, d, cdesc[w], x, lane, pol);
  }
  const uint32_t p = (uint32_t)d.w + lane / T;
  s = row_tree(s, T);
  if constexpr (Scaled<V>::value) s *= wscale[w];
  if (p < nzr && (lane & (T - 1)) == 0) store_row<typename Tr<V>::Acc, MAPPED>(y, row_map, p, s);
}

template <typename V, typename X>
wk_status dispatch(const RunArgs &a, unsigned grid, unsigned block) {
  const wk_engine *e = a.e;
  const wk_layout *l = e->layout;
  const V *pv = e->vals.as<V>();
  const int32_t *pc = e->cols.as<int32_t>();
  const X *x = (const X *)a.x;
  typedef typename Tr<V>::Acc Acc;
  Acc *y = (Acc *)a.y;
  const int4 *desc = l->d.warp_desc;
  const int32_t *rm = l->d.row_map;
  const uint32_t W = l->info.nwarps, nzr = l->info.nznrows;
  const float *ws = e->scale.as<float>();
#define WK_LAUNCH(K, M, C) K<V, X, M, C><<<grid, block, 0, a.stream>>>(pv, pc, desc, W, rm, nzr, x, y, ws)
  const bool c = a.cache != 0;
  if (l->info.variant & WK_ABL_NOCOALESCE) {  // one order only: the reference's
    if (a.mapped) {
      if (c) WK_LAUNCH(k_spmv_nocoal, true, true); else WK_LAUNCH(k_spmv_nocoal, true, false);
    } else {
      if (c) WK_LAUNCH(k_spmv_nocoal, false, true); else WK_LAUNCH(k_spmv_nocoal, false, false);
    }
    WK_CHECK_LAUNCH();
    return WK_OK;
  }
  // Fast order on layouts of short warps: the one-slot-per-step kernel beats
  // the vector path's cross-lane combine (short_steps gives the crossovers).
  const bool use_exact = a.order == WK_ORDER_EXACT || short_layout(l, e->dtype);
  // fp64 keeps 32-bit columns: its SpMV is bound by the FP64 rate, and the
  // 16-bit offsets (fewer bytes, more integer work) measured 7 % slower
  if (e->compressed && !use_exact && sizeof(V) < 8) {
    const uint16_t *c16 = e->c16.as<uint16_t>();
    const int32_t *c32 = e->c32.as<int32_t>();
    const int4 *cd = e->cdesc.as<int4>();
    const uint16_t *w16 = e->w16.as<uint16_t>();
    const int2 *wch = e->wchunks.as<int2>();
    const int4 *wd = e->wdesc.as<int4>();
    const bool win = e->use_windows && e->windows_built && e->window_warps > 0;
    const size_t smem = win ? (size_t)(block / WS) * WIN_MAX * sizeof(X) : 0;
#define WK_LAUNCH_C(M, C, WN)                                                                              \
  do {                                                                                                     \
    if (smem > 48 * 1024)                                                                                  \
      WK_CUDA(cudaFuncSetAttribute(k_spmv_fast_c<V, X, M, C, WN>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                   (int)smem));                                                            \
    k_spmv_fast_c<V, X, M, C, WN><<<grid, block, smem, a.stream>>>(pv, c16, c32, cd, w16, wch, wd, desc, W, rm, \
                                                                   nzr, x, y, ws);                         \
  } while (0)
#define WK_LAUNCH_CW(M, C)                                                                                 \
  do {                                                                                                     \
    if (win) WK_LAUNCH_C(M, C, true); else WK_LAUNCH_C(M, C, false);                                       \
  } while (0)
    if (a.mapped) {
      if (c) WK_LAUNCH_CW(true, true); else WK_LAUNCH_CW(true, false);
    } else {
      if (c) WK_LAUNCH_CW(false, true); else WK_LAUNCH_CW(false, false);
    }
#undef WK_LAUNCH_CW
#undef WK_LAUNCH_C
    WK_CHECK_LAUNCH();
    return WK_OK;
  }
  if (use_exact) {
    if (a.mapped) {
      if (c) WK_LAUNCH(k_spmv_exact, true, true); else WK_LAUNCH(k_spmv_exact, true, false);
    } else {
      if (c) WK_LAUNCH(k_spmv_exact, false, true); else WK_LAUNCH(k_spmv_exact, false, false);
    }
  } else if (sizeof(V) == 8 && long_warps(l)) {
    // fp64 runs its unit loop without unrolling (fewer registers, 1.3 % faster
    // on FE layouts); a layout whose longest warps set the time keeps two
    // units in flight per warp (power-law WPK1, 1 M rows: 0.57 -> 0.43 ms)
#define WK_LAUNCH2(M, C) k_spmv_fast<V, X, M, C, 2><<<grid, block, 0, a.stream>>>(pv, pc, desc, W, rm, nzr, x, y, ws)
    if (a.mapped) {
      if (c) WK_LAUNCH2(true, true); else WK_LAUNCH2(true, false);
    } else {
      if (c) WK_LAUNCH2(false, true); else WK_LAUNCH2(false, false);
    }
#undef WK_LAUNCH2
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

wk_status launch_shape(uint32_t W, int nblocks, int blocksize, unsigned *grid, unsigned *block) {
  int bs = blocksize, nb = nblocks;
  if (bs <= 0 || nb <= 0) {
    bs = 128;
    nb = 0;
  }
  if (bs % WS != 0 || bs > 1024)
    return set_error(WK_ERR_INVALID, "blocksize %d is not a multiple of 32 in [32, 1024]", bs);
  const uint32_t wpb = (uint32_t)bs / WS;
  const size_t need = (W + wpb - 1) / wpb;
  if (nb == 0) nb = (int)(need ? need : 1);
  if ((size_t)nb < need)
    return set_error(WK_ERR_INVALID,
                     "nblocks = %d covers %zu warps but the layout has %u (need >= %zu blocks of %d)", nb,
                     (size_t)nb * wpb, W, need, bs);
  *grid = (unsigned)nb;
  *block = (unsigned)bs;
  return WK_OK;
}

wk_status launch_spmv(const RunArgs &a) {
  const wk_layout *l = a.e->layout;
  unsigned grid = 0, block = 0;
  WK_TRY(launch_shape(l->info.nwarps, a.nblocks, a.blocksize, &grid, &block));
  if (l->info.nwarps == 0) return WK_OK;
  switch (a.e->dtype) {
    case WK_F64: return dispatch<double, double>(a, grid, block);
    case WK_F32: return dispatch<float, float>(a, grid, block);
    case WK_BF16: return dispatch<__nv_bfloat16, __nv_bfloat16>(a, grid, block);
    case WK_F16S: return dispatch<__half, float>(a, grid, block);
  }
  return set_error(WK_ERR_INVALID, "unknown dtype %d", a.e->dtype);
}

}  // namespace wk
