// wk_solve.cu -- solver building blocks on the WPK layout: the fp64 residual
// r = b - A x fused with its squared norm.
//
// The norm is reduced deterministically: each block writes one partial
// (warp shuffles, then the block's warps in index order) and a second kernel
// sums the partials in a fixed order, so repeated calls give identical bits.
#include "wk_internal.cuh"
#include "wk_spmv_core.cuh"

namespace wk {
namespace {

using namespace core;

constexpr int RES_BLOCK = 128;

__device__ __forceinline__ double block_sum(double v, double *sh) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if (lane == 0) sh[wib] = v;
  __syncthreads();
  double t = 0.0;
  if (wib == 0) {
    t = lane < nw ? sh[lane] : 0.0;
#pragma unroll
    for (int off = 16; off; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  }
  return t;  // valid in thread 0
}

// One warp per layout warp; rows without entries (sorted positions
// [nzr, nrows)) get r = b.  partials[blockIdx.x] = sum of r^2 over the block.
template <bool L1>
__global__ void __launch_bounds__(RES_BLOCK) k_residual(const double *__restrict__ pv, const int32_t *__restrict__ pc,
                                                        const int4 *__restrict__ desc, uint32_t W,
                                                        const int32_t *__restrict__ row_map, uint32_t nzr,
                                                        uint32_t nrows, const double *__restrict__ x,
                                                        const double *__restrict__ b, double *__restrict__ r,
                                                        double *__restrict__ partials) {
  __shared__ double sh[RES_BLOCK];
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  double part = 0.0;
  if (w < W) {
    const int4 d = desc[w];
    const uint32_t T = (uint32_t)d.z;
    double s = lane_sum_fast<double, double, L1>(pv, pc, d, x, lane, policy_evict_first());
    s = row_tree(s, T);
    const uint32_t p = (uint32_t)d.w + lane / T;
    if (p < nzr && (lane & (T - 1)) == 0) {
      const int32_t row = row_map[p];
      const double rr = b[row] - s;
      r[row] = rr;
      part = rr * rr;
    }
  }
  for (size_t q = (size_t)nzr + (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nrows;
       q += (size_t)gridDim.x * blockDim.x) {
    const int32_t row = row_map[q];
    const double bb = b[row];
    r[row] = bb;
    part = fma(bb, bb, part);
  }
  const double t = block_sum_staged<RES_BLOCK>(part, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// out[0] = sum of partials[0..n) in a fixed order (one block).
__global__ void __launch_bounds__(1024) k_sum_partials(const double *__restrict__ partials, unsigned n,
                                                       double *__restrict__ out) {
  __shared__ double sh[32];
  double v = 0.0;
  for (unsigned i = threadIdx.x; i < n; i += blockDim.x) v += partials[i];
  const double t = block_sum(v, sh);
  if (threadIdx.x == 0) out[0] = t;
}

}  // namespace

// Launch shape of the residual: 4 warps per block, at least one block.
unsigned residual_grid(const wk_layout *l) {
  const uint32_t W = l->info.nwarps;
  unsigned g = (unsigned)((W + RES_BLOCK / WS - 1) / (RES_BLOCK / WS));
  return g ? g : 1u;
}

wk_status launch_residual(const wk_engine *e, const double *x, const double *b, double *r, double *partials,
                          unsigned grid, double *norm2, cudaStream_t st) {
  const wk_layout *l = e->layout;
  k_residual<true><<<grid, RES_BLOCK, 0, st>>>(e->vals.as<double>(), e->cols.as<int32_t>(), l->d.warp_desc,
                                               l->info.nwarps, l->d.row_map, l->info.nznrows, l->info.nrows, x,
                                               b, r, partials);
  WK_CHECK_LAUNCH();
  if (norm2) {
    k_sum_partials<<<1, 1024, 0, st>>>(partials, grid, norm2);
    WK_CHECK_LAUNCH();
  }
  return WK_OK;
}

}  // namespace wk

// ---- residual without any device allocation -------------------------------------
// The partial sums of wk_residual_static live in this fixed array instead of
// an engine-owned buffer.  Every GPU that loads the library holds it (512 KiB)
// until the process exits.  All calls share it: each call first writes
// partials[0, grid) and only then sums them, so no contents need clearing,
// but calls whose kernels overlap on the GPU race on it.
namespace wk {
namespace {
constexpr unsigned kResidualStaticBlocks = 65536;  // one double per block
static __device__ __align__(256) double g_residual_partials[kResidualStaticBlocks];

// Device address of g_residual_partials for engine e, looked up with
// cudaGetSymbolAddress on the engine's first wk_residual_static call (with
// the engine's device current, as for every call on the engine) and kept in
// the engine.  Caching it per engine, not per device number, keeps it valid
// across cudaDeviceReset: a reset frees the engine as well, and an engine
// created afterwards looks the address up again in the new context.
wk_status static_partials(wk_engine *e, double **out) {
  if (!e->static_partials) {
    double *p = nullptr;
    cudaError_t err = cudaGetSymbolAddress((void **)&p, g_residual_partials);
    if (err != cudaSuccess || !p) {
      cudaGetLastError();
      return set_error(WK_ERR_CUDA, "cudaGetSymbolAddress(g_residual_partials) failed: %s", cudaGetErrorString(err));
    }
    e->static_partials = p;
  }
  *out = e->static_partials;
  return WK_OK;
}
}  // namespace
}  // namespace wk

using namespace wk;

extern "C" wk_status wk_residual_static(wk_engine *e, const double *x, const double *b, double *r,
                                        double *norm2, void *stream) {
  if (!e || !x || !b || !r) return set_error(WK_ERR_INVALID, "NULL argument");
  if (e->dtype != WK_F64) return set_error(WK_ERR_INVALID, "wk_residual_static needs a WK_F64 engine");
  WK_TRY(require_interleaved(e->layout, "wk_residual_static"));
  const unsigned grid = residual_grid(e->layout);
  if (grid > kResidualStaticBlocks)
    return set_error(WK_ERR_INVALID,
                     "wk_residual_static: the layout has %u warps and needs %u partial sums, but the static "
                     "scratch holds %u (at most %u layout warps); use wk_residual",
                     e->layout->info.nwarps, grid, kResidualStaticBlocks, kResidualStaticBlocks * (128u / 32u));
  double *partials = nullptr;
  WK_TRY(static_partials(e, &partials));
  return launch_residual(e, x, b, r, partials, grid, norm2, (cudaStream_t)stream);
}

extern "C" wk_status wk_residual(wk_engine *e, const double *x, const double *b, double *r, double *norm2,
                                 void *stream) {
  if (!e || !x || !b || !r) return set_error(WK_ERR_INVALID, "NULL argument");
  if (e->dtype != WK_F64) return set_error(WK_ERR_INVALID, "wk_residual needs a WK_F64 engine");
  WK_TRY(require_interleaved(e->layout, "wk_residual"));
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned grid = residual_grid(e->layout);
  if (e->scratch.bytes < (size_t)grid * sizeof(double)) WK_TRY(e->scratch.alloc((size_t)grid * sizeof(double)));
  return launch_residual(e, x, b, r, e->scratch.as<double>(), grid, norm2, st);
}
