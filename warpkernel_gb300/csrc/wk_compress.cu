// wk_compress.cu -- 16-bit column storage for the mixed-precision paths.
//
// With fp32 values a stored slot costs 4 B of value + 4 B of column, so the
// column index is half of the traffic.  Finite-element rows of one layout
// warp (32 consecutive sorted rows, i.e. nearby nodes) reference a narrow
// band of columns; when a warp's real entries span fewer than 65,536 columns
// its indices are stored as uint16 offsets from a per-warp base.  Warps with
// a wider span keep int32 indices in a compact side array.  Padding slots
// store offset 0 (their value is 0).
#include <algorithm>
#include <vector>

#include "wk_internal.cuh"

namespace wk {
namespace {

constexpr int WS = 32;

__device__ __forceinline__ bool slot_valid(const int4 d, uint32_t lane, uint32_t i, const uint32_t *slen,
                                           uint32_t nzr) {
  const uint32_t tpr = (uint32_t)d.z;
  const uint32_t p = (uint32_t)d.w + lane / tpr;
  if (p >= nzr) return false;
  return i + (lane % tpr) * (uint32_t)d.y < slen[p];
}

// Per layout warp: mode (0: 16-bit, 1: 32-bit), base, and the 32-bit slot count.
__global__ void k_col_modes(const int4 *__restrict__ desc, uint32_t W, const uint32_t *__restrict__ slen,
                            uint32_t nzr, const int32_t *__restrict__ cols, int4 *__restrict__ cdesc,
                            unsigned long long *__restrict__ wide_slots) {
  const uint32_t lane = threadIdx.x & 31;
  for (size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS; w < W;
       w += (size_t)gridDim.x * blockDim.x / WS) {
    const int4 d = desc[w];
    int lo = 0x7fffffff, hi = -1;
    size_t slot = (size_t)(uint32_t)d.x + lane;
    for (uint32_t i = 0; i < (uint32_t)d.y; i++, slot += WS) {
      if (slot_valid(d, lane, i, slen, nzr)) {
        const int c = cols[slot];
        lo = min(lo, c);
        hi = max(hi, c);
      }
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lane == 0) {
      const bool narrow = hi < 0 || (long long)hi - lo < 65536;
      cdesc[w] = make_int4(hi < 0 ? 0 : lo, narrow ? 0 : 1, 0, 0);
      wide_slots[w] = narrow ? 0ull : (unsigned long long)WS * (uint32_t)d.y;
    }
  }
}

__global__ void k_col_fill(const int4 *__restrict__ desc, uint32_t W, const uint32_t *__restrict__ slen,
                           uint32_t nzr, const int32_t *__restrict__ cols,
                           const unsigned long long *__restrict__ wide_off, int4 *__restrict__ cdesc,
                           uint16_t *__restrict__ c16, int32_t *__restrict__ c32) {
  const uint32_t lane = threadIdx.x & 31;
  for (size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS; w < W;
       w += (size_t)gridDim.x * blockDim.x / WS) {
    const int4 d = desc[w];
    int4 cd = cdesc[w];
    const size_t o = (uint32_t)d.x;
    if (cd.y == 0) {
      size_t slot = o + lane;
      for (uint32_t i = 0; i < (uint32_t)d.y; i++, slot += WS)
        c16[slot] = slot_valid(d, lane, i, slen, nzr) ? (uint16_t)(cols[slot] - cd.x) : (uint16_t)0;
    } else {
      const size_t off = (size_t)wide_off[w];
      for (uint32_t k = lane; k < WS * (uint32_t)d.y; k += WS) {
        const uint32_t i = k / WS;
        c32[off + k] = slot_valid(d, lane, i, slen, nzr) ? cols[o + k] : 0;
        c16[o + k] = 0;
      }
      if (lane == 0) {
        cd.z = (int)off;
        cdesc[w] = cd;
      }
    }
  }
}

// ---- x windows -------------------------------------------------------------------
// A narrow layout warp of a finite-element matrix touches few distinct
// columns: on hex meshes with 3 dofs per node about 350 for 2,500 slots, in 9
// runs of consecutive columns (the nodes along a mesh line in three planes,
// three dofs each).  Such a warp gets an x window: its distinct columns in
// ascending order, described by chunks of at most 32 consecutive columns
// {first column, window position | length << 16}, and every slot stores its
// column's window position in 16 bits (w16).  The fast SpMV copies the
// window's x values into shared memory with one warp-wide load per chunk and
// gathers from there (wk_spmv_core.cuh, stage_window).  Warps with more than
// WIN_MAX distinct columns or WIN_CHUNKS chunks keep the plain 16-bit form.

constexpr int BM_WORDS = 2048;  // one bit per column of a narrow warp's span (< 65,536)
constexpr int WB = 256;         // threads of the window-building blocks
constexpr int WPT = BM_WORDS / WB;

// Block-wide exclusive scan of one value per thread (WB threads); *total =
// the sum.  sh: WB / 32 + 1 words.  All threads must call it.
__device__ uint32_t block_excl_scan(uint32_t v, uint32_t *sh, uint32_t *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) sh[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const uint32_t a = lane < WB / 32 ? sh[lane] : 0u;
    uint32_t ai = a;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, ai, o);
      if (lane >= o) ai += t;
    }
    if (lane < WB / 32) sh[lane] = ai - a;
    if (lane == 31) sh[WB / 32] = ai;
  }
  __syncthreads();
  const uint32_t r = sh[wid] + inc - v;
  *total = sh[WB / 32];
  __syncthreads();
  return r;
}

struct WinShared {
  uint32_t bm[BM_WORDS];  // distinct columns (offsets from the warp's base)
  uint32_t wp[BM_WORDS];  // distinct columns below each bitmap word
  uint32_t rs[WIN_CHUNKS], re[WIN_CHUNKS];  // first / last offset of each run
  uint32_t sh[WB / 32 + 1];
};

// Bitmap, word prefixes and runs of layout warp d's columns (offsets from
// base; the warp spans fewer than 65,536 columns).  Block-uniform call.
__device__ void window_scan(WinShared &S, const int4 d, int base, const uint32_t *__restrict__ slen, uint32_t nzr,
                            const int32_t *__restrict__ cols, uint32_t *distinct, uint32_t *runs) {
  for (int i = threadIdx.x; i < BM_WORDS; i += WB) S.bm[i] = 0u;
  __syncthreads();
  const size_t o = (uint32_t)d.x;
  for (uint32_t k = threadIdx.x; k < (uint32_t)WS * (uint32_t)d.y; k += WB) {
    if (slot_valid(d, k & 31u, k >> 5, slen, nzr)) {
      const uint32_t c = (uint32_t)(cols[o + k] - base);
      atomicOr(&S.bm[c >> 5], 1u << (c & 31u));
    }
  }
  __syncthreads();
  const int w0 = threadIdx.x * WPT;
  // a run may start in one thread's words and end in another's, so starts
  // and ends are numbered by separate scans
  uint32_t pop = 0, nst = 0, nen = 0;
  for (int j = 0; j < WPT; j++) {
    const int wi = w0 + j;
    const uint32_t wv = S.bm[wi];
    const uint32_t prev_top = wi ? S.bm[wi - 1] >> 31 : 0u;
    const uint32_t next_low = wi + 1 < BM_WORDS ? S.bm[wi + 1] & 1u : 0u;
    pop += __popc(wv);
    nst += __popc(wv & ~((wv << 1) | prev_top));
    nen += __popc(wv & ~((wv >> 1) | (next_low << 31)));
  }
  uint32_t tot_pop, tot_runs, tot_ends;
  const uint32_t pop_off = block_excl_scan(pop, S.sh, &tot_pop);
  const uint32_t run_off = block_excl_scan(nst, S.sh, &tot_runs);
  const uint32_t end_off = block_excl_scan(nen, S.sh, &tot_ends);
  uint32_t acc = pop_off, ra = run_off, ea = end_off;
  for (int j = 0; j < WPT; j++) {
    const int wi = w0 + j;
    const uint32_t wv = S.bm[wi];
    S.wp[wi] = acc;
    acc += __popc(wv);
    const uint32_t prev_top = wi ? S.bm[wi - 1] >> 31 : 0u;
    const uint32_t next_low = wi + 1 < BM_WORDS ? S.bm[wi + 1] & 1u : 0u;
    uint32_t st = wv & ~((wv << 1) | prev_top);
    uint32_t en = wv & ~((wv >> 1) | (next_low << 31));
    while (st) {
      const int b = __ffs(st) - 1;
      st &= st - 1;
      if (ra < (uint32_t)WIN_CHUNKS) S.rs[ra] = (uint32_t)(wi * 32 + b);
      ra++;
    }
    while (en) {
      const int b = __ffs(en) - 1;
      en &= en - 1;
      if (ea < (uint32_t)WIN_CHUNKS) S.re[ea] = (uint32_t)(wi * 32 + b);
      ea++;
    }
  }
  __syncthreads();
  *distinct = tot_pop;
  *runs = tot_runs;
}

// Chunks of layout warp w's window (0: the warp gets no window).
__global__ void __launch_bounds__(WB) k_win_count(const int4 *__restrict__ desc, uint32_t W,
                                                  const uint32_t *__restrict__ slen, uint32_t nzr,
                                                  const int32_t *__restrict__ cols, const int4 *__restrict__ cdesc,
                                                  unsigned long long *__restrict__ nch_out) {
  __shared__ WinShared S;
  for (size_t w = blockIdx.x; w < W; w += gridDim.x) {
    const int4 cd = cdesc[w], d = desc[w];
    uint32_t nch = 0;
    if (cd.y == 0 && d.y > 0) {
      uint32_t distinct, runs;
      window_scan(S, d, cd.x, slen, nzr, cols, &distinct, &runs);
      if (distinct > 0 && distinct <= (uint32_t)WIN_MAX && runs <= (uint32_t)WIN_CHUNKS) {
        const uint32_t c = threadIdx.x < runs ? (S.re[threadIdx.x] - S.rs[threadIdx.x] + 32u) / 32u : 0u;
        uint32_t tot;
        block_excl_scan(c, S.sh, &tot);
        nch = tot <= (uint32_t)WIN_CHUNKS ? tot : 0u;
      }
    }
    if (threadIdx.x == 0) nch_out[w] = nch;
    __syncthreads();
  }
}

// Writes the chunks, the window positions of the slots and wdesc = {first
// chunk, chunks, window size, 0} ({0, 0, 0, 0}: no window).
__global__ void __launch_bounds__(WB) k_win_fill(const int4 *__restrict__ desc, uint32_t W,
                                                 const uint32_t *__restrict__ slen, uint32_t nzr,
                                                 const int32_t *__restrict__ cols, const int4 *__restrict__ cdesc,
                                                 const unsigned long long *__restrict__ nch_in,
                                                 const unsigned long long *__restrict__ ch_off,
                                                 int4 *__restrict__ wdesc, int2 *__restrict__ chunks,
                                                 uint16_t *__restrict__ w16) {
  __shared__ WinShared S;
  for (size_t w = blockIdx.x; w < W; w += gridDim.x) {
    const uint32_t nch = (uint32_t)nch_in[w];
    if (nch == 0) {
      if (threadIdx.x == 0) wdesc[w] = make_int4(0, 0, 0, 0);
      continue;  // block-uniform
    }
    const int4 cd = cdesc[w], d = desc[w];
    const int base = cd.x;
    uint32_t distinct, runs;
    window_scan(S, d, base, slen, nzr, cols, &distinct, &runs);
    const uint32_t t = threadIdx.x;
    const uint32_t c = t < runs ? (S.re[t] - S.rs[t] + 32u) / 32u : 0u;
    uint32_t tot;
    const uint32_t co = block_excl_scan(c, S.sh, &tot);
    const size_t c0 = (size_t)ch_off[w];
    if (tot != nch || runs > (uint32_t)WIN_CHUNKS || distinct > (uint32_t)WIN_MAX) {
      // not the window the count pass saw: leave the warp without one
      if (t == 0) wdesc[w] = make_int4(0, 0, 0, 0);
      __syncthreads();
      continue;  // block-uniform
    }
    if (t < runs) {
      const uint32_t s0 = S.rs[t], len = S.re[t] - s0 + 1u;
      const uint32_t rank = S.wp[s0 >> 5] + __popc(S.bm[s0 >> 5] & ((1u << (s0 & 31u)) - 1u));
      for (uint32_t j = 0; j * 32u < len && co + j < nch; j++) {
        const uint32_t l = min(32u, len - 32u * j);
        chunks[c0 + co + j] = make_int2(base + (int)(s0 + 32u * j), (int)((rank + 32u * j) | (l << 16)));
      }
    }
    const size_t o = (uint32_t)d.x;
    for (uint32_t k = t; k < (uint32_t)WS * (uint32_t)d.y; k += WB) {
      uint16_t v = 0;
      if (slot_valid(d, k & 31u, k >> 5, slen, nzr)) {
        const uint32_t cc = (uint32_t)(cols[o + k] - base);
        v = (uint16_t)(S.wp[cc >> 5] + __popc(S.bm[cc >> 5] & ((1u << (cc & 31u)) - 1u)));
      }
      w16[o + k] = v;
    }
    if (t == 0) wdesc[w] = make_int4((int)c0, (int)nch, (int)distinct, 0);
    __syncthreads();
  }
}

unsigned grid_for_warps(uint32_t W) {
  size_t g = ((size_t)W * WS + 255) / 256;
  if (g < 1) g = 1;
  if (g > 152u * 64u) g = 152u * 64u;
  return (unsigned)g;
}

}  // namespace

// Builds the x windows of an engine with compact columns (see above).
// x windows of layout l over its padded columns `cols` (device), given the
// per-warp modes / bases of k_col_modes in `cdesc`: the slots' window
// positions (w16), the chunks and the per-warp window descriptors.
wk_status build_window_arrays(const wk_layout *l, const int32_t *cols, const int4 *cdesc, DevBuf &w16,
                              DevBuf &wchunks, DevBuf &wdesc, uint32_t *warps, cudaStream_t st) {
  const uint32_t W = l->info.nwarps;
  const size_t anz = l->info.allocate_nz;
  DevBuf tot;
  WK_TRY(tot.alloc(8));
  DevBuf nch, choff;
  WK_TRY(nch.alloc((size_t)W * 8));
  WK_TRY(choff.alloc((size_t)W * 8));
  if (W) {
    const unsigned g = (unsigned)std::min<size_t>(W, 152u * 8u);
    k_win_count<<<g, WB, 0, st>>>(l->d.warp_desc, W, l->d.slen, l->info.nznrows, cols, cdesc,
                                  nch.as<unsigned long long>());
    WK_CHECK_LAUNCH();
  }
  WK_TRY(scan_u64(nch.as<unsigned long long>(), choff.as<unsigned long long>(), W, tot.as<unsigned long long>(), st));
  unsigned long long nchunks = 0;
  WK_CUDA(cudaMemcpyAsync(&nchunks, tot.p, 8, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  WK_TRY(wchunks.alloc(nchunks * 8));
  WK_TRY(wdesc.alloc((size_t)W * sizeof(int4)));
  WK_TRY(w16.alloc(anz * 2));
  if (W) {
    const unsigned g = (unsigned)std::min<size_t>(W, 152u * 8u);
    k_win_fill<<<g, WB, 0, st>>>(l->d.warp_desc, W, l->d.slen, l->info.nznrows, cols, cdesc,
                                 nch.as<unsigned long long>(), choff.as<unsigned long long>(), wdesc.as<int4>(),
                                 wchunks.as<int2>(), w16.as<uint16_t>());
    WK_CHECK_LAUNCH();
  }
  WK_CUDA(cudaStreamSynchronize(st));
  std::vector<unsigned long long> h(W);
  if (W) WK_CUDA(cudaMemcpy(h.data(), nch.p, (size_t)W * 8, cudaMemcpyDeviceToHost));
  uint32_t c = 0;
  for (unsigned long long v : h) c += v != 0;
  *warps = c;
  return WK_OK;
}

wk_status build_windows(wk_engine *e, cudaStream_t st) {
  WK_TRY(build_window_arrays(e->layout, e->cols.as<int32_t>(), e->cdesc.as<int4>(), e->w16, e->wchunks, e->wdesc,
                             &e->window_warps, st));
  e->windows_built = true;
  return WK_OK;
}

wk_status build_window_set(const wk_layout *l, const int32_t *cols, WinSet &ws, cudaStream_t st) {
  const uint32_t W = l->info.nwarps;
  DevBuf wide;
  WK_TRY(ws.cdesc.alloc((size_t)W * sizeof(int4)));
  WK_TRY(wide.alloc((size_t)W * 8));
  if (W) {
    k_col_modes<<<grid_for_warps(W), 256, 0, st>>>(l->d.warp_desc, W, l->d.slen, l->info.nznrows, cols,
                                                   ws.cdesc.as<int4>(), wide.as<unsigned long long>());
    WK_CHECK_LAUNCH();
  }
  return build_window_arrays(l, cols, ws.cdesc.as<int4>(), ws.w16, ws.chunks, ws.wdesc, &ws.warps, st);
}

wk_status build_compressed_cols(wk_engine *e, cudaStream_t st, uint32_t *wide_warps) {
  const wk_layout *l = e->layout;
  const uint32_t W = l->info.nwarps;
  const size_t anz = l->info.allocate_nz;
  DevBuf wide, tot;
  WK_TRY(e->cdesc.alloc((size_t)W * sizeof(int4)));
  WK_TRY(e->c16.alloc(anz * 2));
  WK_TRY(wide.alloc((size_t)W * 8));
  WK_TRY(tot.alloc(8));
  if (W) {
    k_col_modes<<<grid_for_warps(W), 256, 0, st>>>(l->d.warp_desc, W, l->d.slen, l->info.nznrows,
                                                   e->cols.as<int32_t>(), e->cdesc.as<int4>(),
                                                   wide.as<unsigned long long>());
    WK_CHECK_LAUNCH();
  }
  WK_TRY(scan_u64(wide.as<unsigned long long>(), wide.as<unsigned long long>(), W, tot.as<unsigned long long>(), st));
  unsigned long long nwide = 0;
  WK_CUDA(cudaMemcpyAsync(&nwide, tot.p, 8, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  WK_TRY(e->c32.alloc(nwide * 4));
  if (W) {
    k_col_fill<<<grid_for_warps(W), 256, 0, st>>>(l->d.warp_desc, W, l->d.slen, l->info.nznrows,
                                                  e->cols.as<int32_t>(), wide.as<unsigned long long>(),
                                                  e->cdesc.as<int4>(), e->c16.as<uint16_t>(), e->c32.as<int32_t>());
    WK_CHECK_LAUNCH();
  }
  e->windows_built = false;
  if (e->use_windows) WK_TRY(build_windows(e, st));
  e->compressed = true;
  if (wide_warps) {
    // count warps in 32-bit mode: slots / (32 * steps) is not uniform, so count descriptors
    std::vector<int4> h(W);
    if (W) WK_CUDA(cudaMemcpy(h.data(), e->cdesc.p, (size_t)W * sizeof(int4), cudaMemcpyDeviceToHost));
    uint32_t c = 0;
    for (const int4 &v : h) c += v.y != 0;
    *wide_warps = c;
  }
  return WK_OK;
}

}  // namespace wk

using namespace wk;

extern "C" wk_status wk_engine_set_windows(wk_engine *e, int on, uint32_t *window_warps) {
  if (!e) return set_error(WK_ERR_INVALID, "engine is NULL");
  if (on && !e->compressed)
    return set_error(WK_ERR_STATE, "x windows need the compact columns: call wk_engine_compress_cols first");
  if (on && !e->windows_built) {
    e->use_windows = true;
    WK_TRY(build_windows(e, nullptr));
  }
  e->use_windows = on != 0;
  if (window_warps) *window_warps = e->windows_built ? e->window_warps : 0u;
  return WK_OK;
}

extern "C" wk_status wk_engine_compress_cols(wk_engine *e, void *stream, uint32_t *wide_warps) {
  if (!e) return set_error(WK_ERR_INVALID, "engine is NULL");
  WK_TRY(require_interleaved(e->layout, "wk_engine_compress_cols"));
  return build_compressed_cols(e, (cudaStream_t)stream, wide_warps);
}
