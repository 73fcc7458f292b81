// wk_batch.cu -- many WPK matrices, each with several right-hand sides, in
// one persistent launch.
//
// Work is split into items (matrix, range of layout warps) ordered by cost,
// largest first; every warp of a persistent grid (one wave of blocks) takes
// the next item from a global counter.  Which warp computes an item does not
// change its arithmetic, so results are deterministic.  For each stored slot
// the value and column are loaded once and reused for an RHS tile of TR
// right-hand sides, gathered with 16-byte loads from a blocked copy of X
// (see Blk) that each launch writes first.  The counter reset, the copy and
// the kernel are captured once in a CUDA graph and replayed.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "wk_internal.cuh"
#include "wk_spmv_core.cuh"

namespace wk {
namespace {

constexpr int WS = 32;
#ifndef WK_BATCH_BLOCK
#define WK_BATCH_BLOCK 256
#endif
constexpr int BATCH_BLOCK = WK_BATCH_BLOCK;
constexpr int BATCH_STAGES = 3;  // tiles in each warp's matrix-stream ring

// X is gathered from a blocked copy: right-hand sides BW*b .. BW*b+BW-1
// (BW = 16 bytes of T: 4 floats or 2 doubles) of every column form block b,
// an ncols x BW row-major array, zero-filled beyond the last right-hand side.
// A warp's gather of one block then reads 16 bytes per lane from rows of 16
// bytes: the 32 lanes, whose columns are neighbours in a finite-element
// matrix, touch about 512 contiguous bytes (4 L1 lines) per load instead of
// 32 rows of the caller's k-wide layout (up to 2 KB, 16 lines for k = 16;
// scalar loads when k is not a multiple of 4), which was the L1 wavefront
// limit of the kernel.  k_xblock writes the blocked copy at the start of
// every launch.
template <typename T>
struct Blk {
  static constexpr int BW = 16 / (int)sizeof(T);
  typedef typename std::conditional<sizeof(T) == 4, float4, double2>::type V;
};

template <typename T>
struct BatchMat {
  const int4 *desc;
  const T *vals;
  const int32_t *cols;
  const int32_t *row_map;
  const T *Xb;  // blocked X: block b at Xb + b * ncols * BW
  T *Y;         // caller's Y, nrows x k row-major
  uint32_t nzr, W, k, ncols;
};

// One item of the blocked copy: rows [r0, r1) of one matrix's X.
template <typename T>
struct XCopy {
  const T *X;
  T *Xb;
  uint32_t ncols, k, r0, r1;
};

__device__ __forceinline__ void set_vec(float (&g)[4], const float4 f) {
  g[0] = f.x; g[1] = f.y; g[2] = f.z; g[3] = f.w;
}
__device__ __forceinline__ void set_vec(double (&g)[2], const double2 f) {
  g[0] = f.x; g[1] = f.y;
}

// The blocked copy of X: one block of threads per item, thread i of a row
// range handles (row r0 + i / nb, block i % nb).
template <typename T>
__global__ void __launch_bounds__(256) k_xblock(const XCopy<T> *__restrict__ items, uint32_t nitems) {
  constexpr int BW = Blk<T>::BW;
  typedef typename Blk<T>::V V;
  for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x) {
    const XCopy<T> c = items[it];
    const uint32_t nb = (c.k + BW - 1) / BW;
    const size_t n = (size_t)(c.r1 - c.r0) * nb;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
      const uint32_t r = c.r0 + (uint32_t)(i / nb), b = (uint32_t)(i % nb);
      T q[BW];
#pragma unroll
      for (int t = 0; t < BW; t++) {
        const uint32_t j = (uint32_t)BW * b + (uint32_t)t;
        q[t] = j < c.k ? __ldg(c.X + (size_t)r * c.k + j) : T(0);
      }
      V v;
      if constexpr (BW == 4)
        v = make_float4(q[0], q[1], q[2], q[3]);
      else
        v = make_double2(q[0], q[1]);
      *reinterpret_cast<V *>(c.Xb + ((size_t)b * c.ncols + r) * BW) = v;
    }
  }
}

// One unit of the matrix stream: S steps, 32 bytes of values per lane.
template <typename T>
struct Unit {
  static constexpr int S = 32 / (int)sizeof(T);  // float: 8 steps, double: 4
};

template <typename T>
__device__ __forceinline__ T staged_val(const uint32_t *sv, int q);
template <>
__device__ __forceinline__ float staged_val<float>(const uint32_t *sv, int q) {
  return __uint_as_float(sv[q]);
}
template <>
__device__ __forceinline__ double staged_val<double>(const uint32_t *sv, int q) {
  return __hiloint2double((int)sv[2 * q + 1], (int)sv[2 * q]);
}

// Three resident blocks per SM: uncapped, the 16-RHS float kernel takes more
// than 100 registers (two blocks, 16 warps per SM); capped at 80 it runs
// with 8 bytes of spill.  fp64 with a 16-wide tile (32 registers of
// accumulators and 32 of gathered X) gets two blocks per SM.
template <typename T, int TR>
constexpr int batch_min_blocks() {
  return sizeof(T) == 8 && TR >= 16 ? 2 : 3;
}
// Layout warps [w0, w1) of one matrix for right-hand sides j0 .. j0 + jn - 1
// with TT accumulators per lane.  TT >= BW: TT / BW whole 16-byte groups
// per slot, unguarded (the blocked copy is zero past k, and only j < jn is
// stored; GUARD skips the groups past jn); TT < BW: the tile lies inside one
// group, gathered element-wise.  The matrix stream of each layout warp runs
// through a ring of BATCH_STAGES tiles of S steps in shared memory, filled
// by cp.async two units ahead (the partial last unit included, copied by
// the lanes that hold its slots) and read back in slot order, so lane l
// sums its own layout lane's slots in step order (fma from zero), which is
// the reference's order.  The next layout warp's descriptor is loaded while
// the current one streams.
template <typename T, int TT, bool GUARD = false>
__device__ __forceinline__ void batch_tile(const BatchMat<T> &M, uint32_t w0, uint32_t w1, uint32_t j0, int jn,
                                           uint32_t *sv, int32_t *sc, uint32_t lane, uint64_t pol) {
  using namespace core;
  constexpr int S = Unit<T>::S, BW = Blk<T>::BW, STAGES = BATCH_STAGES;
  constexpr int LV = S * (int)sizeof(T) / 4;  // value words per lane and unit
  constexpr int VW = LV * WS, CW = S * WS;    // words per value / column tile
  typedef typename Blk<T>::V V;
  const uint32_t bstride = M.ncols * (uint32_t)BW;
  const T *xt = M.Xb + (size_t)(j0 / BW) * bstride + (j0 % BW);
  auto gather = [&](uint32_t c, T(&g)[TT]) {
    const T *xc = xt + (size_t)c * BW;
    if constexpr (TT >= BW) {
#pragma unroll
      for (int j = 0; j < TT; j += BW) {
        T q[BW];
        if (!GUARD || j < jn)
          set_vec(q, __ldg(reinterpret_cast<const V *>(xc + (uint32_t)(j / BW) * bstride)));
        else
#pragma unroll
          for (int i = 0; i < BW; i++) q[i] = T(0);
#pragma unroll
        for (int i = 0; i < BW; i++) g[j + i] = q[i];
      }
    } else {
#pragma unroll
      for (int j = 0; j < TT; j++) g[j] = j < jn ? __ldg(xc + j) : T(0);
    }
  };
  int4 dn = w0 < w1 ? M.desc[w0] : make_int4(0, 0, 0, 0);
  for (uint32_t w = w0; w < w1; w++) {
    const int4 d = dn;
    if (w + 1 < w1) dn = M.desc[w + 1];
    const uint32_t T_ = (uint32_t)d.z, A = (uint32_t)d.y;
    const size_t o = (size_t)(uint32_t)d.x;
    const uint32_t full = A / S, rem = A % S, units = full + (rem != 0);
    // unit u: steps [u S, u S + S) of all lanes, S * 32 consecutive slots;
    // lane l copies slots [S l, S l + S) of it
    auto issue = [&](uint32_t u) {
      if (u < full || lane < rem * (WS / S)) {
        const size_t g = o + (size_t)u * S * WS + S * lane;
        uint32_t *dv = sv + (u % STAGES) * VW + LV * lane;
        const uint32_t *gv = reinterpret_cast<const uint32_t *>(M.vals + g);
#pragma unroll
        for (int q = 0; q < LV; q += 4) cp_async16(dv + q, gv + q, pol);
        int32_t *dc = sc + (u % STAGES) * CW + S * lane;
#pragma unroll
        for (int q = 0; q < S; q += 4) cp_async16(dc + q, M.cols + g + q, pol);
      }
    };
#pragma unroll
    for (int s0 = 0; s0 < STAGES - 1; s0++) {
      if ((uint32_t)s0 < units) issue((uint32_t)s0);
      cp_async_commit();
    }
    const uint32_t p = (uint32_t)d.w + lane / T_;
    const bool valid = p < M.nzr;
    const int32_t row = valid ? M.row_map[p] : 0;
    T acc[TT];
#pragma unroll
    for (int j = 0; j < TT; j++) acc[j] = T(0);
    for (uint32_t u = 0; u < units; u++) {
      if (u + STAGES - 1 < units) issue(u + STAGES - 1);
      cp_async_commit();
      cp_async_wait<STAGES - 1>();
      __syncwarp();
      const uint32_t *svs = sv + (u % STAGES) * VW;
      const int32_t *scs = sc + (u % STAGES) * CW;
      auto step = [&](int st) {
        const int q = st * WS + (int)lane;
        const T v = staged_val<T>(svs, q);
        T g[TT];
        gather((uint32_t)scs[q], g);
#pragma unroll
        for (int j = 0; j < TT; j++) acc[j] = fma(v, g[j], acc[j]);
      };
      if (u < full) {
#pragma unroll
        for (int st = 0; st < S; st++) step(st);
      } else {
        for (int st = 0; st < (int)rem; st++) step(st);
      }
      __syncwarp();  // this tile is refilled STAGES - 1 units later
    }
#pragma unroll
    for (int j = 0; j < TT; j++)
      for (uint32_t s2 = 1; s2 < T_; s2 <<= 1) acc[j] += __shfl_down_sync(0xffffffffu, acc[j], s2);
    if (valid && (lane & (T_ - 1)) == 0) {
      T *yr = M.Y + (size_t)row * M.k + j0;
#pragma unroll
      for (int j = 0; j < TT; j++)
        if (j < jn) __stcs(yr + j, acc[j]);  // streaming: keeps X in L2 (1.5 % faster)
    }
  }
}

// NG = TR / BW 16-byte groups at most; a tile of jn right-hand sides runs
// the instance with ceil(jn / BW) groups.
template <typename T, int TR, int G = 1>
__device__ __forceinline__ void batch_tile_groups(int ng, const BatchMat<T> &M, uint32_t w0, uint32_t w1, uint32_t j0,
                                                  int jn, uint32_t *sv, int32_t *sc, uint32_t lane, uint64_t pol) {
  constexpr int BW = Blk<T>::BW;
  if constexpr (G * BW <= TR) {
    if (ng == G)
      batch_tile<T, G * BW, (G * BW == TR)>(M, w0, w1, j0, jn, sv, sc, lane, pol);
    else
      batch_tile_groups<T, TR, G + 1>(ng, M, w0, w1, j0, jn, sv, sc, lane, pol);
  }
}

template <typename T, int TR>
__global__ void __launch_bounds__(BATCH_BLOCK, (batch_min_blocks<T, TR>())) k_batch(const BatchMat<T> *__restrict__ mats,
                                                        const int4 *__restrict__ items, uint32_t nitems,
                                                        unsigned *__restrict__ counter) {
  constexpr int S = Unit<T>::S, BW = Blk<T>::BW;
  constexpr int NSV = S * WS * (int)sizeof(T) / 4;  // value words per tile
  __shared__ __align__(16) uint32_t s_val[BATCH_BLOCK / WS][BATCH_STAGES * NSV];
  __shared__ __align__(16) int32_t s_col[BATCH_BLOCK / WS][BATCH_STAGES * S * WS];
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x / WS;
  uint32_t *sv = s_val[wib];
  int32_t *sc = s_col[wib];
  const uint64_t pol = core::policy_evict_first();
  for (;;) {
    unsigned it = 0;
    if (lane == 0) it = atomicAdd(counter, 1u);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= nitems) break;
    const int4 item = items[it];
    const BatchMat<T> M = mats[item.x];
    for (uint32_t j0 = 0; j0 < M.k; j0 += TR) {
      const int jn = (int)min((uint32_t)TR, M.k - j0);
      if constexpr (TR >= BW)
        batch_tile_groups<T, TR>((jn + BW - 1) / BW, M, (uint32_t)item.y, (uint32_t)item.z, j0, jn, sv, sc, lane, pol);
      else
        batch_tile<T, TR>(M, (uint32_t)item.y, (uint32_t)item.z, j0, jn, sv, sc, lane, pol);
    }
  }
}

}  // namespace
}  // namespace wk

struct wk_batch {
  int dtype = WK_F32;
  int rhs_tile = 8;
  int chunk = 16;
  std::vector<wk_engine *> engines;
  std::vector<uint32_t> nrhs;
  std::vector<uint32_t> nrows, ncols;
  wk::DevBuf mats, items, counter;
  wk::DevBuf xb, xcopy;  // blocked X of every matrix, and the copy items
  uint32_t nitems = 0, ncopy = 0;
  unsigned grid = 0;
  bool vectors_set = false;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;
  ~wk_batch() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

namespace wk {
namespace {

template <typename T>
wk_status launch_batch_t(wk_batch *b, cudaStream_t st) {
  const BatchMat<T> *mats = b->mats.as<BatchMat<T>>();
  const int4 *items = b->items.as<int4>();
  unsigned *ctr = b->counter.as<unsigned>();
  switch (b->rhs_tile) {
    case 1: k_batch<T, 1><<<b->grid, BATCH_BLOCK, 0, st>>>(mats, items, b->nitems, ctr); break;
    case 2: k_batch<T, 2><<<b->grid, BATCH_BLOCK, 0, st>>>(mats, items, b->nitems, ctr); break;
    case 4: k_batch<T, 4><<<b->grid, BATCH_BLOCK, 0, st>>>(mats, items, b->nitems, ctr); break;
    case 8: k_batch<T, 8><<<b->grid, BATCH_BLOCK, 0, st>>>(mats, items, b->nitems, ctr); break;
    case 16: k_batch<T, 16><<<b->grid, BATCH_BLOCK, 0, st>>>(mats, items, b->nitems, ctr); break;
    default: return set_error(WK_ERR_INVALID, "rhs tile %d not in {1,2,4,8,16}", b->rhs_tile);
  }
  WK_CHECK_LAUNCH();
  return WK_OK;
}

wk_status launch_batch(wk_batch *b, cudaStream_t st) {
  WK_CUDA(cudaMemsetAsync(b->counter.p, 0, sizeof(unsigned), st));
  if (b->ncopy) {
    const unsigned g = std::min<unsigned>(b->ncopy, 152u * 8u);
    if (b->dtype == WK_F64)
      k_xblock<double><<<g, 256, 0, st>>>(b->xcopy.as<XCopy<double>>(), b->ncopy);
    else
      k_xblock<float><<<g, 256, 0, st>>>(b->xcopy.as<XCopy<float>>(), b->ncopy);
    WK_CHECK_LAUNCH();
  }
  return b->dtype == WK_F64 ? launch_batch_t<double>(b, st) : launch_batch_t<float>(b, st);
}

// The blocked X buffer (one region per matrix, 16-byte aligned) and the copy
// items (rows of one matrix, XCOPY_ROWS at a time), for the caller's X.
constexpr uint32_t XCOPY_ROWS = 2048;
template <typename T>
wk_status setup_blocked_x(wk_batch *b, const void *const *X, std::vector<size_t> &off) {
  constexpr int BW = Blk<T>::BW;
  const size_t n = b->engines.size();
  off.assign(n, 0);
  size_t total = 0;
  std::vector<XCopy<T>> items;
  for (size_t m = 0; m < n; m++) {
    const size_t nb = (b->nrhs[m] + BW - 1) / BW;
    if (nb * (size_t)b->ncols[m] * BW >= ((size_t)1 << 32))
      return set_error(WK_ERR_INVALID, "matrix %zu: ncols x right-hand sides (%u x %u) too large for a batch", m,
                       b->ncols[m], b->nrhs[m]);
    off[m] = total;
    total += nb * (size_t)b->ncols[m] * BW;  // elements; a multiple of BW (16 bytes)
  }
  WK_TRY(b->xb.alloc(total * sizeof(T)));
  T *base = b->xb.as<T>();
  for (size_t m = 0; m < n; m++)
    for (uint32_t r0 = 0; r0 < b->ncols[m]; r0 += XCOPY_ROWS)
      items.push_back({(const T *)X[m], base + off[m], b->ncols[m], b->nrhs[m], r0,
                       std::min(b->ncols[m], r0 + XCOPY_ROWS)});
  WK_TRY(b->xcopy.alloc(items.size() * sizeof(XCopy<T>)));
  if (!items.empty())
    WK_CUDA(cudaMemcpy(b->xcopy.p, items.data(), items.size() * sizeof(XCopy<T>), cudaMemcpyHostToDevice));
  b->ncopy = (uint32_t)items.size();
  return WK_OK;
}

template <typename T>
int occupancy_blocks(int tile) {
  int nb = 0;
  switch (tile) {
    case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<T, 1>, BATCH_BLOCK, 0); break;
    case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<T, 2>, BATCH_BLOCK, 0); break;
    case 4: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<T, 4>, BATCH_BLOCK, 0); break;
    case 8: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<T, 8>, BATCH_BLOCK, 0); break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<T, 16>, BATCH_BLOCK, 0); break;
  }
  return nb > 0 ? nb : 1;
}

// Items: (matrix, [w0, w1)) chunks of `chunk` layout warps, largest cost first
// (cost = stored slots of the chunk x right-hand sides).
wk_status build_items(wk_batch *b) {
  struct It {
    int m, w0, w1;
    double cost;
  };
  std::vector<It> v;
  for (size_t m = 0; m < b->engines.size(); m++) {
    const wk_layout *l = b->engines[m]->layout;
    const uint32_t W = l->info.nwarps;
    if (!W) continue;
    std::vector<int4> desc(W);
    WK_CUDA(cudaMemcpy(desc.data(), l->d.warp_desc, (size_t)W * sizeof(int4), cudaMemcpyDeviceToHost));
    for (uint32_t w0 = 0; w0 < W; w0 += (uint32_t)b->chunk) {
      const uint32_t w1 = std::min(W, w0 + (uint32_t)b->chunk);
      double slots = 0;
      for (uint32_t w = w0; w < w1; w++) slots += (double)desc[w].y;
      v.push_back({(int)m, (int)w0, (int)w1, slots * (double)b->nrhs[m]});
    }
  }
  std::stable_sort(v.begin(), v.end(), [](const It &a, const It &c) { return a.cost > c.cost; });
  std::vector<int4> h(v.size());
  for (size_t i = 0; i < v.size(); i++) h[i] = make_int4(v[i].m, v[i].w0, v[i].w1, 0);
  WK_TRY(b->items.alloc(h.size() * sizeof(int4)));
  if (!h.empty()) WK_CUDA(cudaMemcpy(b->items.p, h.data(), h.size() * sizeof(int4), cudaMemcpyHostToDevice));
  b->nitems = (uint32_t)h.size();
  return WK_OK;
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

wk_status set_grid(wk_batch *b) {
  const int nb = b->dtype == WK_F64 ? occupancy_blocks<double>(b->rhs_tile) : occupancy_blocks<float>(b->rhs_tile);
  b->grid = (unsigned)(sm_count() * nb);  // one persistent wave
  return WK_OK;
}

void drop_graph(wk_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
}

}  // namespace
}  // namespace wk

using namespace wk;

extern "C" wk_status wk_batch_create(wk_engine *const *engines, const uint32_t *nrhs, int count, int rhs_tile,
                                     int chunk, wk_batch **out) {
  if (!out) return set_error(WK_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!engines || !nrhs || count <= 0) return set_error(WK_ERR_INVALID, "empty batch");
  for (int m = 0; m < count; m++)
    if (engines[m]) WK_TRY(require_interleaved(engines[m]->layout, "wk_batch_create"));
  wk_batch *b = new (std::nothrow) wk_batch();
  if (!b) return set_error(WK_ERR_ALLOC, "host allocation failed");
  b->dtype = engines[0]->dtype;
  b->rhs_tile = rhs_tile > 0 ? rhs_tile : 8;
  b->chunk = chunk > 0 ? chunk : 16;
  for (int m = 0; m < count; m++) {
    wk_engine *e = engines[m];
    if (!e || e->dtype != b->dtype || (b->dtype != WK_F32 && b->dtype != WK_F64)) {
      delete b;
      return set_error(WK_ERR_INVALID, "engine %d: all engines must be WK_F32 or all WK_F64", m);
    }
    if (nrhs[m] == 0) {
      delete b;
      return set_error(WK_ERR_INVALID, "matrix %d has no right-hand side", m);
    }
    b->engines.push_back(e);
    b->nrhs.push_back(nrhs[m]);
    b->nrows.push_back(e->layout->info.nrows);
    b->ncols.push_back(e->ncols);
  }
  wk_status s = build_items(b);
  if (s == WK_OK) s = b->counter.alloc(16);
  if (s == WK_OK) s = b->mats.alloc((size_t)count * std::max(sizeof(BatchMat<float>), sizeof(BatchMat<double>)));
  if (s == WK_OK) s = set_grid(b);
  if (s != WK_OK) {
    delete b;
    return s;
  }
  *out = b;
  return WK_OK;
}

// X[m]: device, ncols_m x nrhs_m row-major; Y[m]: device, nrows_m x nrhs_m.
extern "C" wk_status wk_batch_set_vectors(wk_batch *b, const void *const *X, void *const *Y) {
  if (!b || !X || !Y) return set_error(WK_ERR_INVALID, "NULL argument");
  const size_t n = b->engines.size();
  for (size_t m = 0; m < n; m++)
    if (!X[m] || !Y[m]) return set_error(WK_ERR_INVALID, "matrix %zu: NULL X or Y", m);
  drop_graph(b);
  std::vector<size_t> off;
  if (b->dtype == WK_F64) {
    WK_TRY(setup_blocked_x<double>(b, X, off));
    std::vector<BatchMat<double>> h(n);
    for (size_t m = 0; m < n; m++) {
      const wk_engine *e = b->engines[m];
      h[m] = {e->layout->d.warp_desc, e->vals.as<double>(), e->cols.as<int32_t>(), e->layout->d.row_map,
              b->xb.as<double>() + off[m], (double *)Y[m], e->layout->info.nznrows, e->layout->info.nwarps,
              b->nrhs[m], b->ncols[m]};
    }
    WK_CUDA(cudaMemcpy(b->mats.p, h.data(), n * sizeof(h[0]), cudaMemcpyHostToDevice));
  } else {
    WK_TRY(setup_blocked_x<float>(b, X, off));
    std::vector<BatchMat<float>> h(n);
    for (size_t m = 0; m < n; m++) {
      const wk_engine *e = b->engines[m];
      h[m] = {e->layout->d.warp_desc, e->vals.as<float>(), e->cols.as<int32_t>(), e->layout->d.row_map,
              b->xb.as<float>() + off[m], (float *)Y[m], e->layout->info.nznrows, e->layout->info.nwarps,
              b->nrhs[m], b->ncols[m]};
    }
    WK_CUDA(cudaMemcpy(b->mats.p, h.data(), n * sizeof(h[0]), cudaMemcpyHostToDevice));
  }
  b->vectors_set = true;
  return WK_OK;
}

extern "C" wk_status wk_batch_set_tile(wk_batch *b, int rhs_tile) {
  if (!b) return set_error(WK_ERR_INVALID, "batch is NULL");
  if (rhs_tile != 1 && rhs_tile != 2 && rhs_tile != 4 && rhs_tile != 8 && rhs_tile != 16)
    return set_error(WK_ERR_INVALID, "rhs tile %d not in {1,2,4,8,16}", rhs_tile);
  b->rhs_tile = rhs_tile;
  drop_graph(b);
  return set_grid(b);
}

// One persistent launch (replays the captured graph when there is one).
// seconds (optional): device time of the launch, synchronous.
extern "C" wk_status wk_batch_run(wk_batch *b, void *stream, float *seconds) {
  if (!b) return set_error(WK_ERR_INVALID, "batch is NULL");
  if (!b->vectors_set) return set_error(WK_ERR_STATE, "wk_batch_set_vectors has not been called");
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (seconds) {
    WK_CUDA(cudaEventCreate(&t0));
    WK_CUDA(cudaEventCreate(&t1));
    WK_CUDA(cudaEventRecord(t0, st));
  }
  wk_status s = WK_OK;
  if (b->graph) {
    cudaError_t e = cudaGraphLaunch(b->graph, st);
    if (e != cudaSuccess) s = set_error(WK_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e));
  } else {
    s = launch_batch(b, st);
  }
  if (seconds) {
    cudaEventRecord(t1, st);
    cudaError_t e = cudaEventSynchronize(t1);
    float ms = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (s == WK_OK && e != cudaSuccess) s = set_error(WK_ERR_CUDA, "batch run: %s", cudaGetErrorString(e));
    *seconds = ms * 1e-3f;
  }
  return s;
}

// Captures the counter reset and the persistent kernel into a CUDA graph
// that wk_batch_run replays (vectors and tile are baked in: call again after
// changing them).
extern "C" wk_status wk_batch_capture(wk_batch *b) {
  if (!b) return set_error(WK_ERR_INVALID, "batch is NULL");
  if (!b->vectors_set) return set_error(WK_ERR_STATE, "wk_batch_set_vectors has not been called");
  drop_graph(b);
  cudaStream_t cap;
  WK_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  wk_status s = e == cudaSuccess ? launch_batch(b, cap) : set_error(WK_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(cap, &g);
  if (s == WK_OK && e != cudaSuccess) s = set_error(WK_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
  if (s == WK_OK) {
    e = cudaGraphInstantiate(&b->graph, g, 0);
    if (e != cudaSuccess) s = set_error(WK_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  }
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cap);
  return s;
}

extern "C" wk_status wk_batch_info(const wk_batch *b, uint32_t *nitems, uint32_t *grid, int *rhs_tile) {
  if (!b) return set_error(WK_ERR_INVALID, "batch is NULL");
  if (nitems) *nitems = b->nitems;
  if (grid) *grid = b->grid;
  if (rhs_tile) *rhs_tile = b->rhs_tile;
  return WK_OK;
}

extern "C" wk_status wk_batch_destroy(wk_batch *b) {
  delete b;
  return WK_OK;
}
