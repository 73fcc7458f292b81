// wk_cg.cu -- conjugate gradient (fp64) and iterative-refinement CG (fp64
// outer loop, fp32 inner CG on an FP32 / BF16 / scaled-FP16 engine, its dot
// products summed in FP64 unless the caller asks for FP32) on the WPK layout.
//
// All scalars stay on the device, and every reduction is summed in a fixed
// order, so results are bit-reproducible.  An iteration is three kernels:
// the SpMV-dot (q = A p, block partials of p.q, each group of 64 blocks
// summed by its last block to finish), the vector update (every block sums
// the group sums for alpha; block partials of r.r) and the p update (every
// block sums those partials for beta; block 0 stores r.r, counts the
// iteration and sets the done flag: converged, or the iteration limit
// reached).  Every CG kernel returns at once when the flag is set.  A batch
// of iterations is captured once in a CUDA graph and replayed; the host
// reads the flag after each batch.
#include <algorithm>
#include <cmath>

#include "wk_internal.cuh"
#include "wk_spmv_core.cuh"

namespace wk {
namespace {

using namespace core;

constexpr int CG_BLOCK = 128;              // 4 warps per block in the SpMV-dot kernel, one per layout warp
constexpr int VEC_BLOCK = 256;
constexpr unsigned VEC_GRID = 152 * 8;     // blocks of the vector kernels

// Blocks of the SpMV-dot kernel (one warp per layout warp, like wk_run: a
// grid-stride loop over layout warps measured 37 % slower at hex 96^3).
unsigned spmv_dot_grid(const wk_layout *l) {
  const size_t g = ((size_t)l->info.nwarps + CG_BLOCK / WS - 1) / (CG_BLOCK / WS);
  return (unsigned)std::max<size_t>(1, g);
}
// Partial sums a CG run needs room for.
size_t cg_partials(const wk_layout *l, unsigned residual_blocks) {
  return std::max<size_t>({residual_blocks, VEC_GRID, spmv_dot_grid(l)});
}
// The SpMV-dot's block partials are summed in groups of DOT_GROUP blocks by
// the last block of each group to finish (a counter per group); the vector
// update then sums the group sums.  Both orders are fixed.
constexpr unsigned DOT_GROUP = 64;
unsigned dot_groups(const wk_layout *l) { return (spmv_dot_grid(l) + DOT_GROUP - 1) / DOT_GROUP; }

// Scratch of one CG run: block partials, the SpMV-dot's group sums and their
// arrival counters (zero between iterations).
struct CgScratch {
  double *partials, *gsum;
  unsigned *gcnt;
};

// slots of `scal`
enum { S_RHO0, S_RHO1, S_PQ, S_BB, S_RR64, S_TOL2, S_DONE, S_ITERS, S_MAXIT, S_COUNT };

__device__ __forceinline__ bool done(const double *scal) { return scal[S_DONE] != 0.0; }
__device__ __forceinline__ double safe_div(double a, double b) { return b != 0.0 ? a / b : 0.0; }

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

// q = A p (rows without entries get 0) and block partials of p . q.  MODE 0:
// vector path, 1: vector path on 16-bit columns, 2: one slot per step (short
// warps, as wk_run's fast order chooses), 3: 16-bit columns with the
// engine's x windows (4-byte vectors; dynamic shared memory of WIN_MAX
// values per warp), the window copied asynchronously as in wk_run.  D64: p . q accumulated in FP64
// (each row's p and q converted once), else in the vectors' precision.
template <typename V, typename X, int MODE, bool D64>
__global__ void __launch_bounds__(CG_BLOCK) k_spmv_dot(const V *__restrict__ pv, const int32_t *__restrict__ pc,
                                                       const uint16_t *__restrict__ c16, const int32_t *__restrict__ c32,
                                                       const int4 *__restrict__ cdesc, const int4 *__restrict__ desc,
                                                       uint32_t W, const int32_t *__restrict__ row_map, uint32_t nzr,
                                                       uint32_t nrows, const X *__restrict__ p, X *__restrict__ q,
                                                       const double *__restrict__ scal, double *__restrict__ partials,
                                                       double *__restrict__ gsum, unsigned *__restrict__ gcnt,
                                                       const float *__restrict__ wscale, const uint16_t *__restrict__ w16,
                                                       const int2 *__restrict__ wch, const int4 *__restrict__ wdesc) {
  if (done(scal)) return;
  extern __shared__ __align__(16) unsigned char cg_dyn_smem[];
  __shared__ double sh[CG_BLOCK];
  __shared__ bool s_last;
  const uint32_t lane = threadIdx.x & 31;
  // p . q in FP64 (fp64 vectors, or D64), else in FP32 for the inner solve
  // (then no float <-> double conversions per row on GB300's FP64 pipe)
  typedef typename std::conditional<sizeof(X) == 8 || D64, double, float>::type D;
  D part = D(0);
  const uint64_t pol = policy_evict_first();
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w < W) {
    const int4 d = desc[w];
    const uint32_t T = (uint32_t)d.z;
    const uint32_t r = (uint32_t)d.w + lane / T;
    typename Tr<V>::Acc s;
    if constexpr (MODE == 3 && sizeof(X) == 4) {
      const int4 wd = wdesc[w];
      if (wd.y != 0) {
        X *win = reinterpret_cast<X *>(cg_dyn_smem) + (threadIdx.x / WS) * WIN_MAX;
        stage_window_async(win, wch, wd, p, lane);
        s = lane_sum_vec<V, X, true, uint16_t, false, 0, true>(pv, w16 + (uint32_t)d.x, 0, d, win, lane, pol, [] {
          cp_async_wait<0>();
          __syncwarp();
        });
      } else {
        s = lane_sum_compressed<V, X, true, false>(pv, c16, c32, d, cdesc[w], p, lane, pol);
      }
    } else if constexpr (MODE == 1 || MODE == 3)
      s = lane_sum_compressed<V, X, true, false>(pv, c16, c32, d, cdesc[w], p, lane, pol);
    else if constexpr (MODE == 2)
      s = lane_sum_exact<V, X, true>(pv, pc, d, p, lane, r < nzr);
    else
      s = lane_sum_fast<V, X, true, false>(pv, pc, d, p, lane, pol);
    s = row_tree(s, T);
    if constexpr (Scaled<V>::value) s *= wscale[w];
    if (r < nzr && (lane & (T - 1)) == 0) {
      const int32_t row = row_map[r];
      const X qv = (X)s;
      q[row] = qv;
      part = fma((D)p[row], (D)qv, part);
    }
  }
  for (size_t k = (size_t)nzr + (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nrows;
       k += (size_t)gridDim.x * blockDim.x)
    q[row_map[k]] = X(0);
  const D t = block_sum_staged<CG_BLOCK, D>(part, reinterpret_cast<D *>(sh));
  // the last block of each group of DOT_GROUP sums the group's partials
  const unsigned grp = blockIdx.x / DOT_GROUP;
  const unsigned gsize = min(DOT_GROUP, gridDim.x - grp * DOT_GROUP);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = (double)t;
    __threadfence();
    s_last = atomicAdd(&gcnt[grp], 1u) == gsize - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x < WS) {
    __threadfence();
    const uint32_t lane = threadIdx.x;
    const double *gp = partials + (size_t)grp * DOT_GROUP;
    double a = (lane < gsize ? __ldcg(gp + lane) : 0.0) + (lane + WS < gsize ? __ldcg(gp + lane + WS) : 0.0);
#pragma unroll
    for (int off = 16; off; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
    if (lane == 0) {
      gsum[grp] = a;
      gcnt[grp] = 0u;  // ready for the next iteration
    }
  }
}

// Fixed-order sum of v[0..n) by one warp (lane-strided partials, then the
// xor tree); every lane gets the total.
__device__ __forceinline__ double warp_sum_array(const double *__restrict__ v, unsigned n, uint32_t lane) {
  double a = 0.0;
  for (unsigned i = lane; i < n; i += WS) a += __ldcg(v + i);
#pragma unroll
  for (int off = 16; off; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
  return a;
}

// x += alpha p, r -= alpha q, partials of r . r; alpha = scal[rho] / (p . q),
// p . q summed by every block from the SpMV-dot's group sums.
// FP32 vectors (the inner solve of IR-CG, whose tolerance is loose) are
// updated in FP32 arithmetic: on GB300 the float <-> double conversions of an
// FP64 update run at the FP64 rate and made these vector kernels FP64-bound.
// Each thread's share of r . r is summed in FP64 with D64 (one conversion per
// element), else in FP32.
template <typename T, bool D64>
__global__ void __launch_bounds__(VEC_BLOCK) k_update(T *__restrict__ x, T *__restrict__ r, const T *__restrict__ p,
                                                      const T *__restrict__ q, uint32_t n, const double *__restrict__ scal,
                                                      int i_rho, const double *__restrict__ gsum, unsigned ngroups,
                                                      double *__restrict__ partials) {
  if (done(scal)) return;
  __shared__ double sh[VEC_BLOCK];
  __shared__ double s_alpha;
  if (threadIdx.x < WS) {
    const double pq = warp_sum_array(gsum, ngroups, threadIdx.x);
    if (threadIdx.x == 0) s_alpha = safe_div(scal[i_rho], pq);
  }
  __syncthreads();
  const double alpha = s_alpha;
  double part = 0.0;
  if constexpr (sizeof(T) == 8) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
      const T ri = r[i] - alpha * q[i];
      x[i] = x[i] + alpha * p[i];
      r[i] = ri;
      part = fma(ri, ri, part);
    }
  } else {
    const float a = (float)alpha;
    float part32 = 0.f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
      const float ri = r[i] - a * q[i];
      x[i] = x[i] + a * p[i];
      r[i] = ri;
      if constexpr (D64) {
        const double rd = (double)ri;
        part = fma(rd, rd, part);
      } else {
        part32 = fmaf(ri, ri, part32);
      }
    }
    if constexpr (!D64) part = (double)part32;
  }
  const double t = block_sum_staged<VEC_BLOCK>(part, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// p = r + beta p, beta = r.r / scal[rho], r.r summed by every block from
// k_update's partials; block 0 stores it in scal[rr], counts the iteration
// and sets the done flag (1: r.r <= tol2, 2: iteration limit).
template <typename T>
__global__ void __launch_bounds__(VEC_BLOCK) k_pupdate(T *__restrict__ p, const T *__restrict__ r, uint32_t n,
                                                       double *scal, int i_rr, int i_rho,
                                                       const double *__restrict__ partials, unsigned nparts) {
  if (done(scal)) return;
  __shared__ double s_beta;
  if (threadIdx.x < WS) {
    const double rr = warp_sum_array(partials, nparts, threadIdx.x);
    if (threadIdx.x == 0) {
      s_beta = safe_div(rr, scal[i_rho]);
      if (blockIdx.x == 0) {
        scal[i_rr] = rr;
        const double it = scal[S_ITERS] + 1.0;
        scal[S_ITERS] = it;
        if (rr <= scal[S_TOL2])
          scal[S_DONE] = 1.0;
        else if (it >= scal[S_MAXIT])
          scal[S_DONE] = 2.0;
      }
    }
  }
  __syncthreads();
  const double beta = s_beta;
  const T b = (T)beta;  // FP32 vectors: FP32 arithmetic (see k_update)
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = r[i] + b * p[i];
}

// partials of a . a, each thread's share in FP64 (fp64 vectors, or D64)
// or in the vector's precision (see k_update), the block sum in fp64
template <typename T, bool D64>
__global__ void __launch_bounds__(VEC_BLOCK) k_dot_self(const T *__restrict__ a, uint32_t n,
                                                        double *__restrict__ partials) {
  __shared__ double sh[VEC_BLOCK];
  typedef typename std::conditional<sizeof(T) == 8 || D64, double, T>::type D;
  D part = D(0);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const D v = (D)a[i];
    part = fma(v, v, part);
  }
  const double t = block_sum_staged<VEC_BLOCK>((double)part, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

__global__ void k_sum_to(const double *__restrict__ partials, unsigned n, double *out) {
  __shared__ double sh[32];
  double v = 0.0;
  for (unsigned i = threadIdx.x; i < n; i += blockDim.x) v += partials[i];
  const double t = block_sum(v, sh);
  if (threadIdx.x == 0) *out = t;
}

// Start of a CG run: tol2 = tol^2 * scal[ref]; counters cleared.
__global__ void k_start(double *scal, int ref, double tol_sq, double maxit) {
  scal[S_TOL2] = tol_sq * scal[ref];
  scal[S_ITERS] = 0.0;
  scal[S_MAXIT] = maxit;
  scal[S_DONE] = scal[S_RHO0] <= scal[S_TOL2] ? 1.0 : 0.0;
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

// IR: x64 += d
__global__ void __launch_bounds__(VEC_BLOCK) k_ir_correct(double *__restrict__ x, const float *__restrict__ d,
                                                          uint32_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    x[i] += (double)d[i];
}

template <typename X>
struct CgVectors {
  X *x, *r, *p, *q;
};

// One CG iteration; `parity` selects which rho slot is current.  d64: the
// dot products p . q and r . r of FP32 vectors summed in FP64.
template <typename X>
void cg_iteration(const wk_engine *e, const CgVectors<X> &v, double *scal, const CgScratch &sc, int parity, bool d64,
                  cudaStream_t st) {
  const wk_layout *l = e->layout;
  const uint32_t W = l->info.nwarps, n = l->info.nrows;
  const unsigned g = spmv_dot_grid(l);
  const int i_rho = parity ? S_RHO1 : S_RHO0, i_next = parity ? S_RHO0 : S_RHO1;
  int mode = short_layout(l, e->dtype) ? 2 : (e->compressed && e->dtype != WK_F64 ? 1 : 0);
  // the engine's x windows for 4-byte vectors (FP32 and scaled-FP16 engines)
  if (mode == 1 && sizeof(X) == 4 && e->dtype != WK_BF16 && e->use_windows && e->windows_built && e->window_warps)
    mode = 3;
  const size_t smem = mode == 3 ? (size_t)(CG_BLOCK / WS) * WIN_MAX * sizeof(X) : 0;
#define WK_SPMV_DOT2(V, M, D)                                                                                       \
  k_spmv_dot<V, X, M, D><<<g, CG_BLOCK, smem, st>>>(                                                                \
      e->vals.as<V>(), e->cols.as<int32_t>(), e->c16.as<uint16_t>(), e->c32.as<int32_t>(), e->cdesc.as<int4>(),     \
      l->d.warp_desc, W, l->d.row_map, l->info.nznrows, n, v.p, v.q, scal, sc.partials, sc.gsum, sc.gcnt,           \
      e->scale.as<float>(), e->w16.as<uint16_t>(), e->wchunks.as<int2>(), e->wdesc.as<int4>())
#define WK_SPMV_DOT1(V, M)                                                                                          \
  do {                                                                                                              \
    if (d64) WK_SPMV_DOT2(V, M, true); else WK_SPMV_DOT2(V, M, false);                                              \
  } while (0)
#define WK_SPMV_DOT(V)                                                                                              \
  do {                                                                                                              \
    if (mode == 2) WK_SPMV_DOT1(V, 2); else if (mode == 1) WK_SPMV_DOT1(V, 1);                                      \
    else if (mode == 3) WK_SPMV_DOT1(V, 3); else WK_SPMV_DOT1(V, 0);                                                \
  } while (0)
  if constexpr (sizeof(X) == 8) {
    WK_SPMV_DOT(double);
  } else {
    if (e->dtype == WK_F32)
      WK_SPMV_DOT(float);
    else if (e->dtype == WK_F16S)
      WK_SPMV_DOT(__half);
    else
      WK_SPMV_DOT(__nv_bfloat16);
  }
#undef WK_SPMV_DOT
#undef WK_SPMV_DOT1
#undef WK_SPMV_DOT2
  const unsigned ng = (g + DOT_GROUP - 1) / DOT_GROUP;
  if (d64)
    k_update<X, true><<<VEC_GRID, VEC_BLOCK, 0, st>>>(v.x, v.r, v.p, v.q, n, scal, i_rho, sc.gsum, ng, sc.partials);
  else
    k_update<X, false><<<VEC_GRID, VEC_BLOCK, 0, st>>>(v.x, v.r, v.p, v.q, n, scal, i_rho, sc.gsum, ng, sc.partials);
  k_pupdate<X><<<VEC_GRID, VEC_BLOCK, 0, st>>>(v.p, v.r, n, scal, i_next, i_rho, sc.partials, VEC_GRID);
}

template <typename X>
wk_status dot_self(const X *a, uint32_t n, double *partials, double *out, bool d64, cudaStream_t st) {
  if (d64)
    k_dot_self<X, true><<<VEC_GRID, VEC_BLOCK, 0, st>>>(a, n, partials);
  else
    k_dot_self<X, false><<<VEC_GRID, VEC_BLOCK, 0, st>>>(a, n, partials);
  k_sum_to<<<1, 1024, 0, st>>>(partials, VEC_GRID, out);
  WK_CHECK_LAUNCH();
  return WK_OK;
}

// A batch of `iters` (even) CG iterations captured once as a CUDA graph.
struct IterGraph {
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  ~IterGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (cap) cudaStreamDestroy(cap);
  }
  template <typename X>
  wk_status build(const wk_engine *e, const CgVectors<X> &v, double *scal, const CgScratch &sc, int iters, bool d64) {
    WK_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    WK_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < iters; i++) cg_iteration<X>(e, v, scal, sc, i & 1, d64, cap);
    cudaGraph_t g = nullptr;
    cudaError_t err = cudaStreamEndCapture(cap, &g);
    if (err != cudaSuccess) {
      cudaGetLastError();
      return set_error(WK_ERR_CUDA, "CG graph capture failed: %s", cudaGetErrorString(err));
    }
    err = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) return set_error(WK_ERR_CUDA, "CG graph instantiation failed: %s", cudaGetErrorString(err));
    return WK_OK;
  }
};

// Replays the graph until the done flag is set; returns the iteration count.
wk_status run_until_done(IterGraph &gr, double *scal, cudaStream_t st, int *iters, int *flag) {
  double h[2] = {0, 0};
  for (;;) {
    WK_CUDA(cudaGraphLaunch(gr.exec, st));
    WK_CUDA(cudaMemcpyAsync(h, scal + S_DONE, 16, cudaMemcpyDeviceToHost, st));  // S_DONE, S_ITERS
    WK_CUDA(cudaStreamSynchronize(st));
    if (h[0] != 0.0) break;
  }
  *iters = (int)h[1];
  *flag = (int)h[0];
  return WK_OK;
}

wk_status check_square(const wk_engine *e) {
  if (e->ncols != e->layout->info.nrows)
    return set_error(WK_ERR_INVALID, "CG needs a square matrix (ncols %u, nrows %u)", e->ncols, e->layout->info.nrows);
  return WK_OK;
}

int batch_of(const wk_cg_params *p) {
  int b = p->check_every > 0 ? p->check_every : 16;
  return b + (b & 1);  // even: the rho slots alternate
}

}  // namespace
}  // namespace wk

using namespace wk;

extern "C" wk_status wk_cg(wk_engine *e, const double *b, double *x, wk_cg_params *prm, void *stream) {
  if (!e || !b || !x || !prm) return set_error(WK_ERR_INVALID, "NULL argument");
  if (e->dtype != WK_F64) return set_error(WK_ERR_INVALID, "wk_cg needs a WK_F64 engine");
  WK_TRY(require_interleaved(e->layout, "wk_cg"));
  WK_TRY(check_square(e));
  if (prm->max_iter <= 0) return set_error(WK_ERR_INVALID, "max_iter must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t n = e->layout->info.nrows;
  const unsigned rg = residual_grid(e->layout);
  DevBuf rb, pb, qb, sb, part;
  WK_TRY(rb.alloc((size_t)n * 8));
  WK_TRY(pb.alloc((size_t)n * 8));
  WK_TRY(qb.alloc((size_t)n * 8));
  WK_TRY(sb.alloc(S_COUNT * 8));
  WK_TRY(part.alloc(cg_partials(e->layout, rg) * 8));
  DevBuf gs, gc;
  WK_TRY(gs.alloc((size_t)dot_groups(e->layout) * 8));
  WK_TRY(gc.alloc((size_t)dot_groups(e->layout) * 4));
  WK_CUDA(cudaMemsetAsync(gc.p, 0, (size_t)dot_groups(e->layout) * 4, st));
  double *scal = sb.as<double>(), *pp = part.as<double>();
  const CgScratch sc{pp, gs.as<double>(), gc.as<unsigned>()};
  CgVectors<double> v{x, rb.as<double>(), pb.as<double>(), qb.as<double>()};
  IterGraph gr;
  WK_TRY(gr.build<double>(e, v, scal, sc, batch_of(prm), true));
  cudaEvent_t t0, t1;
  WK_CUDA(cudaEventCreate(&t0));
  WK_CUDA(cudaEventCreate(&t1));
  WK_CUDA(cudaEventRecord(t0, st));
  WK_TRY(dot_self<double>(b, n, pp, scal + S_BB, true, st));
  WK_TRY(launch_residual(e, x, b, v.r, pp, rg, scal + S_RHO0, st));
  WK_CUDA(cudaMemcpyAsync(v.p, v.r, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
  k_start<<<1, 1, 0, st>>>(scal, S_BB, prm->tol * prm->tol, (double)prm->max_iter);
  WK_CHECK_LAUNCH();
  int iters = 0, flag = 0;
  WK_TRY(run_until_done(gr, scal, st, &iters, &flag));
  WK_TRY(launch_residual(e, x, b, v.r, pp, rg, scal + S_RR64, st));  // true residual of the result
  WK_CUDA(cudaEventRecord(t1, st));
  double h[2];
  WK_CUDA(cudaMemcpyAsync(&h[0], scal + S_RR64, 8, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaMemcpyAsync(&h[1], scal + S_BB, 8, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  const double bb = h[1] > 0 ? h[1] : 1.0;
  prm->iters = iters;
  prm->outer = 0;
  prm->relres = std::sqrt(h[0] / bb);
  prm->seconds = ms * 1e-3;
  if (prm->relres <= prm->tol) return WK_OK;
  return set_error(WK_ERR_NOTCONV, "CG stopped after %d iterations at relative residual %.3e", iters, prm->relres);
}

extern "C" wk_status wk_ir_cg(wk_engine *e64, wk_engine *lo, const double *b, double *x, wk_cg_params *prm,
                              void *stream) {
  if (!e64 || !lo || !b || !x || !prm) return set_error(WK_ERR_INVALID, "NULL argument");
  WK_TRY(require_interleaved(e64->layout, "wk_ir_cg"));
  WK_TRY(require_interleaved(lo->layout, "wk_ir_cg"));
  if (e64->dtype != WK_F64) return set_error(WK_ERR_INVALID, "wk_ir_cg: the residual engine must be WK_F64");
  if (lo->dtype != WK_F32 && lo->dtype != WK_BF16 && lo->dtype != WK_F16S)
    return set_error(WK_ERR_INVALID, "wk_ir_cg: the inner engine must be WK_F32, WK_BF16 or WK_F16S");
  WK_TRY(check_square(e64));
  if (lo->layout->info.nrows != e64->layout->info.nrows || lo->ncols != e64->ncols)
    return set_error(WK_ERR_INVALID, "wk_ir_cg: engines of different sizes");
  if (prm->max_iter <= 0) return set_error(WK_ERR_INVALID, "max_iter must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t n = e64->layout->info.nrows;
  const int max_inner = prm->max_inner > 0 ? prm->max_inner : 1000;
  const double inner_tol = prm->inner_tol > 0 ? prm->inner_tol : 1e-4;
  const unsigned rg = residual_grid(e64->layout);
  DevBuf r64b, r32b, db, pb, qb, sb, part;
  WK_TRY(r64b.alloc((size_t)n * 8));
  WK_TRY(r32b.alloc((size_t)n * 4));
  WK_TRY(db.alloc((size_t)n * 4));
  WK_TRY(pb.alloc((size_t)n * 4));
  WK_TRY(qb.alloc((size_t)n * 4));
  WK_TRY(sb.alloc(S_COUNT * 8));
  WK_TRY(part.alloc(std::max(cg_partials(lo->layout, rg), cg_partials(e64->layout, rg)) * 8));
  DevBuf gs, gc;
  WK_TRY(gs.alloc((size_t)dot_groups(lo->layout) * 8));
  WK_TRY(gc.alloc((size_t)dot_groups(lo->layout) * 4));
  WK_CUDA(cudaMemsetAsync(gc.p, 0, (size_t)dot_groups(lo->layout) * 4, st));
  double *r64 = r64b.as<double>(), *scal = sb.as<double>(), *pp = part.as<double>();
  const CgScratch sc{pp, gs.as<double>(), gc.as<unsigned>()};
  CgVectors<float> v{db.as<float>(), r32b.as<float>(), pb.as<float>(), qb.as<float>()};
  const bool d64 = prm->inner_dots_fp32 == 0;
  IterGraph gr;
  WK_TRY(gr.build<float>(lo, v, scal, sc, batch_of(prm), d64));
  cudaEvent_t t0, t1;
  WK_CUDA(cudaEventCreate(&t0));
  WK_CUDA(cudaEventCreate(&t1));
  WK_CUDA(cudaEventRecord(t0, st));
  WK_TRY(dot_self<double>(b, n, pp, scal + S_BB, true, st));
  double bb = 0.0;
  WK_CUDA(cudaMemcpyAsync(&bb, scal + S_BB, 8, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  if (!(bb > 0)) bb = 1.0;
  const double tol2 = prm->tol * prm->tol * bb;
  int outer = 0, inner_total = 0;
  double rr64 = 0.0;
  for (;;) {
    // fp64: r = b - A x and ||r||^2
    WK_TRY(launch_residual(e64, x, b, r64, pp, rg, scal + S_RR64, st));
    WK_CUDA(cudaMemcpyAsync(&rr64, scal + S_RR64, 8, cudaMemcpyDeviceToHost, st));
    WK_CUDA(cudaStreamSynchronize(st));
    if (!(rr64 > tol2) || outer >= prm->max_iter) break;
    // fp32 inner CG: A d = r from d = 0 until ||r_inner|| <= inner_tol ||r||
    k_ir_prepare<<<VEC_GRID, VEC_BLOCK, 0, st>>>(r64, v.r, v.x, v.p, n);
    WK_TRY(dot_self<float>(v.r, n, pp, scal + S_RHO0, d64, st));
    k_start<<<1, 1, 0, st>>>(scal, S_RHO0, inner_tol * inner_tol, (double)max_inner);
    WK_CHECK_LAUNCH();
    int its = 0, flag = 0;
    WK_TRY(run_until_done(gr, scal, st, &its, &flag));
    inner_total += its;
    // fp64 update
    k_ir_correct<<<VEC_GRID, VEC_BLOCK, 0, st>>>(x, v.x, n);
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
  if (prm->relres <= prm->tol) return WK_OK;
  return set_error(WK_ERR_NOTCONV, "IR-CG stopped after %d outer / %d inner iterations at %.3e", outer, inner_total,
                   prm->relres);
}
