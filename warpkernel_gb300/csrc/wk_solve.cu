// wk_solve.cu -- solver building blocks on the WPK layout: the fp64 residual
// r = b - A x fused with its squared norm.
//
// The norm is reduced deterministically: each block writes one partial
// (warp shuffles, then the block's warps in index order) and a second kernel
// sums the partials in a fixed order, so repeated calls give identical bits.
#include <algorithm>
#include <cmath>

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
  __shared__ double sh[32];
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
  const double t = block_sum(part, sh);
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

constexpr int kMaxDevices = 64;
std::atomic<double *> g_residual_partials_addr[kMaxDevices];

// Device address of g_residual_partials on the current device, looked up on
// the first call per device (cudaGetSymbolAddress with that device current).
wk_status static_partials(double **out) {
  int dev = 0;
  WK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(WK_ERR_STATE, "device %d beyond the supported %d", dev, kMaxDevices);
  double *p = g_residual_partials_addr[dev].load();
  if (!p) {
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_residual_partials);
    if (e != cudaSuccess || !p)
      return set_error(WK_ERR_CUDA, "cudaGetSymbolAddress(g_residual_partials) on device %d failed: %s", dev,
                       cudaGetErrorString(e));
    g_residual_partials_addr[dev].store(p);
  }
  *out = p;
  return WK_OK;
}
}  // namespace
}  // namespace wk

using namespace wk;

extern "C" wk_status wk_residual_static(wk_engine *e, const double *x, const double *b, double *r,
                                        double *norm2, void *stream) {
  if (!e || !x || !b || !r) return set_error(WK_ERR_INVALID, "NULL argument");
  if (e->dtype != WK_F64) return set_error(WK_ERR_INVALID, "wk_residual_static needs a WK_F64 engine");
  const unsigned grid = residual_grid(e->layout);
  if (grid > kResidualStaticBlocks)
    return set_error(WK_ERR_INVALID,
                     "wk_residual_static: the layout has %u warps and needs %u partial sums, but the static "
                     "scratch holds %u (at most %u layout warps); use wk_residual",
                     e->layout->info.nwarps, grid, kResidualStaticBlocks, kResidualStaticBlocks * (128u / 32u));
  double *partials = nullptr;
  WK_TRY(static_partials(&partials));
  return launch_residual(e, x, b, r, partials, grid, norm2, (cudaStream_t)stream);
}

extern "C" wk_status wk_residual(wk_engine *e, const double *x, const double *b, double *r, double *norm2,
                                 void *stream) {
  if (!e || !x || !b || !r) return set_error(WK_ERR_INVALID, "NULL argument");
  if (e->dtype != WK_F64) return set_error(WK_ERR_INVALID, "wk_residual needs a WK_F64 engine");
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned grid = residual_grid(e->layout);
  if (e->scratch.bytes < (size_t)grid * sizeof(double)) WK_TRY(e->scratch.alloc((size_t)grid * sizeof(double)));
  return launch_residual(e, x, b, r, e->scratch.as<double>(), grid, norm2, st);
}

// ==================================================================================
// Conjugate gradient (fp64) and iterative-refinement CG (fp64 outer, fp32 inner).
//
// Scalars stay on the device: every reduction writes block partials that a
// single-block kernel sums in a fixed order into a slot of `scal`; the update
// kernels read alpha / beta from those slots, so an iteration needs no host
// round trip.  The host reads the residual norm every `check_every`
// iterations to decide convergence.
// ==================================================================================
namespace wk {
namespace {

constexpr int VEC_BLOCK = 256;
constexpr unsigned VEC_GRID = 152 * 8;  // fixed: the partial count is part of the summation order

// scal slots
enum { S_RHO0 = 0, S_RHO1 = 1, S_PQ = 2, S_BB = 3, S_RR64 = 4, S_RR0 = 5 };

// q = A p (rows without entries get 0) and block partials of p . q
template <typename V, typename X, bool COMP>
__global__ void __launch_bounds__(RES_BLOCK) k_cg_spmv_dot(const V *__restrict__ pv, const int32_t *__restrict__ pc,
                                                           const uint16_t *__restrict__ c16,
                                                           const int32_t *__restrict__ c32,
                                                           const int4 *__restrict__ cdesc, const int4 *__restrict__ desc,
                                                           uint32_t W, const int32_t *__restrict__ row_map,
                                                           uint32_t nzr, uint32_t nrows, const X *__restrict__ p,
                                                           X *__restrict__ q, double *__restrict__ partials) {
  __shared__ double sh[32];
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  double part = 0.0;
  if (w < W) {
    const int4 d = desc[w];
    const uint32_t T = (uint32_t)d.z;
    typename Tr<V>::Acc s;
    if constexpr (COMP)
      s = lane_sum_compressed<V, X, true>(pv, c16, c32, d, cdesc[w], p, lane, policy_evict_first());
    else
      s = lane_sum_fast<V, X, true>(pv, pc, d, p, lane, policy_evict_first());
    s = row_tree(s, T);
    const uint32_t r = (uint32_t)d.w + lane / T;
    if (r < nzr && (lane & (T - 1)) == 0) {
      const int32_t row = row_map[r];
      const X qv = (X)s;
      q[row] = qv;
      part = (double)p[row] * (double)qv;
    }
  }
  for (size_t k = (size_t)nzr + (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nrows;
       k += (size_t)gridDim.x * blockDim.x)
    q[row_map[k]] = X(0);
  const double t = block_sum(part, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

__device__ __forceinline__ double safe_div(double a, double b) { return b != 0.0 ? a / b : 0.0; }

// x += alpha p, r -= alpha q, partials of r . r; alpha = scal[rho] / scal[pq]
template <typename T>
__global__ void __launch_bounds__(VEC_BLOCK) k_cg_update(T *__restrict__ x, T *__restrict__ r, const T *__restrict__ p,
                                                         const T *__restrict__ q, uint32_t n,
                                                         const double *__restrict__ scal, int i_rho,
                                                         double *__restrict__ partials) {
  __shared__ double sh[32];
  const double alpha = safe_div(scal[i_rho], scal[S_PQ]);
  double part = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const T ri = (T)((double)r[i] - alpha * (double)q[i]);
    x[i] = (T)((double)x[i] + alpha * (double)p[i]);
    r[i] = ri;
    part = fma((double)ri, (double)ri, part);
  }
  const double t = block_sum(part, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// p = r + beta p, beta = scal[rr] / scal[rho]
template <typename T>
__global__ void __launch_bounds__(VEC_BLOCK) k_cg_pupdate(T *__restrict__ p, const T *__restrict__ r, uint32_t n,
                                                          const double *__restrict__ scal, int i_rr, int i_rho) {
  const double beta = safe_div(scal[i_rr], scal[i_rho]);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = (T)((double)r[i] + beta * (double)p[i]);
}

// partials of a . a
template <typename T>
__global__ void __launch_bounds__(VEC_BLOCK) k_dot_self(const T *__restrict__ a, uint32_t n,
                                                        double *__restrict__ partials) {
  __shared__ double sh[32];
  double part = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    part = fma((double)a[i], (double)a[i], part);
  const double t = block_sum(part, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// IR: r32 = r64, d = 0, p = r32
__global__ void __launch_bounds__(VEC_BLOCK) k_ir_prepare(const double *__restrict__ r64, float *__restrict__ r32,
                                                          float *__restrict__ d, float *__restrict__ p, uint32_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float v = (float)r64[i];
    r32[i] = v;
    p[i] = v;
    d[i] = 0.f;
  }
}

// IR: x64 += d (fp64 update)
__global__ void __launch_bounds__(VEC_BLOCK) k_ir_correct(double *__restrict__ x, const float *__restrict__ d,
                                                          uint32_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    x[i] += (double)d[i];
}

// One CG iteration on engine e with vectors of type X (rho slot alternates).
template <typename X>
wk_status cg_iteration(const wk_engine *e, X *x, X *r, X *p, X *q, double *scal, double *partials, int it,
                       cudaStream_t st) {
  const wk_layout *l = e->layout;
  const unsigned g = residual_grid(l);
  const int i_rho = it & 1 ? S_RHO1 : S_RHO0, i_next = it & 1 ? S_RHO0 : S_RHO1;
  const uint32_t n = l->info.nrows;
#define WK_SPMV_DOT(V, COMP)                                                                                    \
  k_cg_spmv_dot<V, X, COMP><<<g, RES_BLOCK, 0, st>>>(e->vals.as<V>(), e->cols.as<int32_t>(), e->c16.as<uint16_t>(), \
                                                     e->c32.as<int32_t>(), e->cdesc.as<int4>(), l->d.warp_desc,     \
                                                     l->info.nwarps, l->d.row_map, l->info.nznrows, n, p, q, partials)
  if constexpr (sizeof(X) == 8) {
    if (e->compressed) WK_SPMV_DOT(double, true); else WK_SPMV_DOT(double, false);
  } else {
    if (e->dtype == WK_F32) {
      if (e->compressed) WK_SPMV_DOT(float, true); else WK_SPMV_DOT(float, false);
    } else {
      if (e->compressed) WK_SPMV_DOT(__nv_bfloat16, true); else WK_SPMV_DOT(__nv_bfloat16, false);
    }
  }
#undef WK_SPMV_DOT
  k_sum_partials<<<1, 1024, 0, st>>>(partials, g, scal + S_PQ);
  k_cg_update<X><<<VEC_GRID, VEC_BLOCK, 0, st>>>(x, r, p, q, n, scal, i_rho, partials);
  k_sum_partials<<<1, 1024, 0, st>>>(partials, VEC_GRID, scal + i_next);
  k_cg_pupdate<X><<<VEC_GRID, VEC_BLOCK, 0, st>>>(p, r, n, scal, i_next, i_rho);
  WK_CHECK_LAUNCH();
  return WK_OK;
}

template <typename X>
wk_status dot_self(const X *a, uint32_t n, double *partials, double *out, cudaStream_t st) {
  k_dot_self<X><<<VEC_GRID, VEC_BLOCK, 0, st>>>(a, n, partials);
  k_sum_partials<<<1, 1024, 0, st>>>(partials, VEC_GRID, out);
  WK_CHECK_LAUNCH();
  return WK_OK;
}

wk_status check_square(const wk_engine *e) {
  if (e->ncols != e->layout->info.nrows)
    return set_error(WK_ERR_INVALID, "CG needs a square matrix (ncols %u, nrows %u)", e->ncols, e->layout->info.nrows);
  return WK_OK;
}

// Inner fp32 CG on engine `lo` for A d = r32 starting from d = 0 (p = r32).
// Runs until ||r||^2 <= tol2 or maxit iterations; returns the count.
wk_status inner_cg(const wk_engine *lo, float *d, float *r, float *p, float *q, double *scal, double *partials,
                   double tol2, int maxit, int check_every, int *iters, cudaStream_t st) {
  int it = 0;
  while (it < maxit) {
    const int m = std::min(check_every, maxit - it);
    for (int j = 0; j < m; j++, it++) WK_TRY((cg_iteration<float>(lo, d, r, p, q, scal, partials, it, st)));
    double rr = 0.0;
    WK_CUDA(cudaMemcpyAsync(&rr, scal + (it & 1 ? S_RHO1 : S_RHO0), 8, cudaMemcpyDeviceToHost, st));
    WK_CUDA(cudaStreamSynchronize(st));
    if (!(rr > tol2)) break;
  }
  *iters = it;
  return WK_OK;
}

}  // namespace
}  // namespace wk

extern "C" wk_status wk_cg(wk_engine *e, const double *b, double *x, wk_cg_params *prm, void *stream) {
  if (!e || !b || !x || !prm) return set_error(WK_ERR_INVALID, "NULL argument");
  if (e->dtype != WK_F64) return set_error(WK_ERR_INVALID, "wk_cg needs a WK_F64 engine");
  WK_TRY(check_square(e));
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t n = e->layout->info.nrows;
  const int check_every = prm->check_every > 0 ? prm->check_every : 10;
  const unsigned np = std::max(residual_grid(e->layout), VEC_GRID);
  DevBuf rb, pb, qb, sb, part;
  WK_TRY(rb.alloc((size_t)n * 8));
  WK_TRY(pb.alloc((size_t)n * 8));
  WK_TRY(qb.alloc((size_t)n * 8));
  WK_TRY(sb.alloc(16 * 8));
  WK_TRY(part.alloc((size_t)np * 8));
  double *r = rb.as<double>(), *p = pb.as<double>(), *q = qb.as<double>(), *scal = sb.as<double>();
  cudaEvent_t t0, t1;
  WK_CUDA(cudaEventCreate(&t0));
  WK_CUDA(cudaEventCreate(&t1));
  WK_CUDA(cudaEventRecord(t0, st));
  WK_TRY(dot_self<double>(b, n, part.as<double>(), scal + S_BB, st));
  WK_TRY(launch_residual(e, x, b, r, part.as<double>(), residual_grid(e->layout), scal + S_RHO0, st));
  WK_CUDA(cudaMemcpyAsync(p, r, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
  double hs[2];
  WK_CUDA(cudaMemcpyAsync(hs, scal + S_RHO0, 16, cudaMemcpyDeviceToHost, st));  // rho0 (slot 0), skip
  WK_CUDA(cudaMemcpyAsync(&hs[1], scal + S_BB, 8, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  const double bb = hs[1] > 0 ? hs[1] : 1.0, tol2 = prm->tol * prm->tol * bb;
  int it = 0;
  double rr = hs[0];
  while (rr > tol2 && it < prm->max_iter) {
    const int m = std::min(check_every, prm->max_iter - it);
    for (int j = 0; j < m; j++, it++) WK_TRY((cg_iteration<double>(e, x, r, p, q, scal, part.as<double>(), it, st)));
    WK_CUDA(cudaMemcpyAsync(&rr, scal + (it & 1 ? S_RHO1 : S_RHO0), 8, cudaMemcpyDeviceToHost, st));
    WK_CUDA(cudaStreamSynchronize(st));
  }
  // true residual of the returned x
  WK_TRY(launch_residual(e, x, b, r, part.as<double>(), residual_grid(e->layout), scal + S_RR64, st));
  WK_CUDA(cudaEventRecord(t1, st));
  double r64 = 0.0;
  WK_CUDA(cudaMemcpyAsync(&r64, scal + S_RR64, 8, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  prm->iters = it;
  prm->outer = 0;
  prm->relres = std::sqrt(r64 / bb);
  prm->seconds = ms * 1e-3;
  return prm->relres <= prm->tol ? WK_OK
                                 : set_error(WK_ERR_NOTCONV, "CG stopped after %d iterations at relative residual %.3e",
                                             it, prm->relres);
}

extern "C" wk_status wk_ir_cg(wk_engine *e64, wk_engine *lo, const double *b, double *x, wk_cg_params *prm,
                              void *stream) {
  if (!e64 || !lo || !b || !x || !prm) return set_error(WK_ERR_INVALID, "NULL argument");
  if (e64->dtype != WK_F64) return set_error(WK_ERR_INVALID, "wk_ir_cg: the residual engine must be WK_F64");
  if (lo->dtype != WK_F32 && lo->dtype != WK_BF16)
    return set_error(WK_ERR_INVALID, "wk_ir_cg: the inner engine must be WK_F32 or WK_BF16");
  WK_TRY(check_square(e64));
  if (lo->layout->info.nrows != e64->layout->info.nrows || lo->ncols != e64->ncols)
    return set_error(WK_ERR_INVALID, "wk_ir_cg: engines of different sizes");
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t n = e64->layout->info.nrows;
  const int check_every = prm->check_every > 0 ? prm->check_every : 10;
  const int max_inner = prm->max_inner > 0 ? prm->max_inner : 1000;
  const double inner_tol = prm->inner_tol > 0 ? prm->inner_tol : 1e-4;
  const unsigned np = std::max(std::max(residual_grid(e64->layout), residual_grid(lo->layout)), VEC_GRID);
  DevBuf r64b, r32b, db, pb, qb, sb, part;
  WK_TRY(r64b.alloc((size_t)n * 8));
  WK_TRY(r32b.alloc((size_t)n * 4));
  WK_TRY(db.alloc((size_t)n * 4));
  WK_TRY(pb.alloc((size_t)n * 4));
  WK_TRY(qb.alloc((size_t)n * 4));
  WK_TRY(sb.alloc(16 * 8));
  WK_TRY(part.alloc((size_t)np * 8));
  double *r64 = r64b.as<double>(), *scal = sb.as<double>(), *pp = part.as<double>();
  float *r32 = r32b.as<float>(), *d = db.as<float>(), *p = pb.as<float>(), *q = qb.as<float>();
  cudaEvent_t t0, t1;
  WK_CUDA(cudaEventCreate(&t0));
  WK_CUDA(cudaEventCreate(&t1));
  WK_CUDA(cudaEventRecord(t0, st));
  WK_TRY(dot_self<double>(b, n, pp, scal + S_BB, st));
  double bb = 0.0;
  WK_CUDA(cudaMemcpyAsync(&bb, scal + S_BB, 8, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  if (!(bb > 0)) bb = 1.0;
  const double tol2 = prm->tol * prm->tol * bb;
  int outer = 0, inner_total = 0;
  double rr64 = 0.0;
  for (;;) {
    // fp64 residual r = b - A x and its norm
    WK_TRY(launch_residual(e64, x, b, r64, pp, residual_grid(e64->layout), scal + S_RR64, st));
    WK_CUDA(cudaMemcpyAsync(&rr64, scal + S_RR64, 8, cudaMemcpyDeviceToHost, st));
    WK_CUDA(cudaStreamSynchronize(st));
    if (!(rr64 > tol2) || outer >= prm->max_iter) break;
    // inner solve A d = r in fp32 from d = 0
    k_ir_prepare<<<VEC_GRID, VEC_BLOCK, 0, st>>>(r64, r32, d, p, n);
    WK_CHECK_LAUNCH();
    WK_TRY(dot_self<float>(r32, n, pp, scal + S_RHO0, st));
    double rr0 = 0.0;
    WK_CUDA(cudaMemcpyAsync(&rr0, scal + S_RHO0, 8, cudaMemcpyDeviceToHost, st));
    WK_CUDA(cudaStreamSynchronize(st));
    int its = 0;
    WK_TRY(inner_cg(lo, d, r32, p, q, scal, pp, inner_tol * inner_tol * rr0, max_inner, check_every, &its, st));
    inner_total += its;
    k_ir_correct<<<VEC_GRID, VEC_BLOCK, 0, st>>>(x, d, n);
    WK_CHECK_LAUNCH();
    outer++;
  }
  WK_CUDA(cudaEventRecord(t1, st));
  WK_CUDA(cudaEventSynchronize(t1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  prm->iters = inner_total;
  prm->outer = outer;
  prm->relres = std::sqrt(rr64 / bb);
  prm->seconds = ms * 1e-3;
  return prm->relres <= prm->tol
             ? WK_OK
             : set_error(WK_ERR_NOTCONV, "IR-CG stopped after %d outer / %d inner iterations at %.3e", outer,
                         inner_total, prm->relres);
}
