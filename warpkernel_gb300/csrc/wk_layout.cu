// wk_layout.cu -- WPK1/WPK2 layout built on the GPU.
//
// The reference builds the layout on the host (warpkernel.hpp:215-771):
// std::sort of (row, length) pairs, per-warp maxima, prefix sums, and for WPK2
// a sequential warp-splitting loop that inserts into std::vectors.  Here every
// step is a data-parallel kernel and the arrays come out bit-identical:
//
//  1. row lengths + CSR validation + max length / non-empty count;
//  2. stable LSD radix sort of key (maxlen - len) with row ids as values --
//     the reference's strict order "longer first, then lower row" (222-225);
//  3. row_map / row_map_inv / sorted lengths;
//  4. per original warp of 32 sorted rows, the split decision of 633-691 is a
//     pure function of (warp max, rows in warp, threshold), so it becomes a
//     per-warp map followed by two exclusive scans (output warp index and
//     slot offset) and an expansion;
//  5. reorder_rows (352-364, 719-735) computed per sorted row.
// process() (380-398) is a gather over padded slots with coalesced writes.
#include "wk_internal.cuh"

namespace wk {
namespace {

constexpr int WS = 32;

// ---------------------------------------------------------------------------
// Exclusive scan (uint32 / uint64), three passes, deterministic.
// ---------------------------------------------------------------------------
constexpr int SCAN_NT = 512;
constexpr int SCAN_IPT = 8;
constexpr int SCAN_TILE = SCAN_NT * SCAN_IPT;

template <typename T>
__device__ T block_excl_scan(T v, T *total) {
  __shared__ T warp_tot[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T incl = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += t;
  }
  __syncthreads();  // warp_tot may still be read by a previous call
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    T w = lane < nw ? warp_tot[lane] : T(0);
    T wi = w;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      T t = __shfl_up_sync(0xffffffffu, wi, off);
      if (lane >= off) wi += t;
    }
    if (lane < nw) warp_tot[lane] = wi - w;
    if (lane == nw - 1) warp_tot[31] = wi;  // nw <= 31 here (blockDim <= 992) or lane 31 itself
  }
  __syncthreads();
  T res = warp_tot[wid] + incl - v;
  if (total) *total = warp_tot[31];
  return res;
}

template <typename T>
__global__ void k_scan_reduce(const T *__restrict__ in, size_t n, T *__restrict__ part) {
  size_t base = (size_t)blockIdx.x * SCAN_TILE;
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    size_t i = base + (size_t)k * SCAN_NT + threadIdx.x;
    if (i < n) s += in[i];
  }
  T tot;
  block_excl_scan<T>(s, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

template <typename T>
__global__ void k_scan_partials(T *part, size_t nb, T *total) {
  T carry = 0;
  for (size_t c = 0; c < nb; c += blockDim.x) {
    size_t i = c + threadIdx.x;
    T v = i < nb ? part[i] : T(0);
    T tot;
    T ex = block_excl_scan<T>(v, &tot);
    if (i < nb) part[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

template <typename T>
__global__ void k_scan_apply(const T *in, T *out, size_t n, const T *__restrict__ part) {
  size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_IPT;
  T v[SCAN_IPT];
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    v[k] = base + k < n ? in[base + k] : T(0);
    s += v[k];
  }
  T run = part[blockIdx.x] + block_excl_scan<T>(s, (T *)nullptr);
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

// out[i] = sum(in[0..i)), *d_total = sum(in) (device).  out may alias in.
template <typename T>
wk_status exclusive_scan(const T *in, T *out, size_t n, T *d_total, cudaStream_t st) {
  size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb == 0) nb = 1;
  DevBuf part;
  WK_TRY(part.alloc(nb * sizeof(T)));
  if (n == 0) {
    WK_CUDA(cudaMemsetAsync(part.p, 0, sizeof(T), st));
  } else {
    k_scan_reduce<T><<<(unsigned)nb, SCAN_NT, 0, st>>>(in, n, part.as<T>());
  }
  k_scan_partials<T><<<1, 992, 0, st>>>(part.as<T>(), nb, d_total);
  if (n) k_scan_apply<T><<<(unsigned)nb, SCAN_NT, 0, st>>>(in, out, n, part.as<T>());
  WK_CHECK_LAUNCH();
  WK_CUDA(cudaStreamSynchronize(st));  // `part` is freed on return
  return WK_OK;
}

// ---------------------------------------------------------------------------
// Row lengths and CSR checks.
// stats[0] = max length, [1] = non-empty rows, [2] = 1 if some length < 0,
// [3] = rowptr[0], [4] = rowptr[n].
// ---------------------------------------------------------------------------
__global__ void k_rowlen(const int32_t *__restrict__ rowptr, uint32_t n, uint32_t *__restrict__ len,
                         unsigned *stats) {
  unsigned mx = 0, cnt = 0, bad = 0;
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (size_t)gridDim.x * blockDim.x) {
    int32_t l = rowptr[r + 1] - rowptr[r];
    if (l < 0) { bad = 1; l = 0; }
    len[r] = (uint32_t)l;
    mx = max(mx, (unsigned)l);
    cnt += l > 0;
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    bad |= __shfl_xor_sync(0xffffffffu, bad, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&stats[0], mx);
    atomicAdd(&stats[1], cnt);
    if (bad) atomicOr(&stats[2], 1u);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    stats[3] = (unsigned)rowptr[0];
    stats[4] = (unsigned)rowptr[n];
  }
}

// Sort keys: length descending (maxlen - len), or for the unsorted ablation
// layout only "empty rows last" (len == 0), so rows keep their CSR order.
__global__ void k_init_keys(const uint32_t *__restrict__ len, uint32_t n, uint32_t maxlen,
                            uint32_t *__restrict__ keys, uint32_t *__restrict__ vals, int nosort) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (size_t)gridDim.x * blockDim.x) {
    keys[r] = nosort ? (uint32_t)(len[r] == 0) : maxlen - len[r];
    vals[r] = (uint32_t)r;
  }
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.  A tile of RS_TILE keys belongs to one
// warp; ranks inside a 32-key chunk come from __match_any_sync, and chunks are
// taken in order, so equal digits keep their input order.
// ---------------------------------------------------------------------------
constexpr int RS_WARPS = 8;
constexpr int RS_CHUNKS = 16;
constexpr int RS_TILE = 32 * RS_CHUNKS;

__global__ void __launch_bounds__(RS_WARPS * 32)
    k_radix_up(const uint32_t *__restrict__ keys, uint32_t n, int shift, uint32_t *__restrict__ hist,
               uint32_t ntiles) {
  __shared__ uint32_t cnt[RS_WARPS][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t t = blockIdx.x * RS_WARPS + w;
  for (int d = lane; d < 256; d += 32) cnt[w][d] = 0;
  __syncwarp();
  if (t >= ntiles) return;
  for (int c = 0; c < RS_CHUNKS; c++) {
    size_t i = (size_t)t * RS_TILE + c * 32 + lane;
    if (i < n) atomicAdd(&cnt[w][(keys[i] >> shift) & 255u], 1u);
  }
  __syncwarp();
  for (int d = lane; d < 256; d += 32) hist[(size_t)d * ntiles + t] = cnt[w][d];
}

__global__ void __launch_bounds__(RS_WARPS * 32)
    k_radix_down(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                 uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, uint32_t n, int shift,
                 const uint32_t *__restrict__ hist, uint32_t ntiles) {
  __shared__ uint32_t base[RS_WARPS][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t t = blockIdx.x * RS_WARPS + w;
  if (t >= ntiles) return;
  for (int d = lane; d < 256; d += 32) base[w][d] = hist[(size_t)d * ntiles + t];
  __syncwarp();
  const unsigned lt = (1u << lane) - 1u;
  for (int c = 0; c < RS_CHUNKS; c++) {
    size_t i = (size_t)t * RS_TILE + c * 32 + lane;
    bool valid = i < n;
    uint32_t k = valid ? kin[i] : 0u, v = valid ? vin[i] : 0u;
    uint32_t d = valid ? ((k >> shift) & 255u) : 256u;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned rank = __popc(peers & lt);
    uint32_t pos = valid ? base[w][d] + rank : 0u;
    __syncwarp();
    if (valid && rank == 0) base[w][d] += __popc(peers);
    __syncwarp();
    if (valid) {
      kout[pos] = k;
      vout[pos] = v;
    }
  }
}

// row_map[p] (already in `vals`), slen[p], row_map_inv[row_map[p]] = p.
__global__ void k_finish_sort(const uint32_t *__restrict__ vals, const uint32_t *__restrict__ len, uint32_t n,
                              int32_t *__restrict__ row_map, int32_t *__restrict__ row_map_inv,
                              uint32_t *__restrict__ slen) {
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (size_t)gridDim.x * blockDim.x) {
    uint32_t r = vals[p];
    row_map[p] = (int32_t)r;
    row_map_inv[r] = (int32_t)p;
    slen[p] = len[r];
  }
}

// ---------------------------------------------------------------------------
// Warp tables.
// ---------------------------------------------------------------------------
struct WarpSplit {
  uint32_t tpr;    // threads per row (1 if not split)
  uint32_t steps;  // max_nz_rows of each output warp
  uint32_t full;   // 1: i output warps of 32/i rows; 0: one output warp
  uint32_t rows;   // rows_w of each output warp
};

// The split rule of warpkernel.hpp:645-688 for one warp with maximum row
// length A and `cnt` rows, restated as a function.  The reference compares
// unsigned values (uint A_w vs uint threshold) and multiplies int by int;
// unsigned wrapping arithmetic gives the same results wherever the
// reference's is defined.
__device__ __forceinline__ WarpSplit split_rule(uint32_t A, uint32_t cnt, uint32_t th, bool wpk2) {
  WarpSplit s{1u, A, 0u, cnt};
  if (!wpk2 || !(A > th)) return s;
  int32_t npw = (int32_t)th;
  if (A > th * 32u) npw = (int32_t)((A + 31u) / 32u);
  for (uint32_t i = 2; i <= 32; i *= 2) {
    if (A <= (uint32_t)npw * i) {
      s.tpr = i;
      s.steps = (A + i - 1) / i;
      if (cnt * i < 32u) {
        s.full = 0;  // partial last warp: real row count kept
      } else {
        s.full = 1;
        s.rows = 32u / i;
      }
      return s;
    }
  }
  return s;  // unreachable: i = 32 always satisfies A <= npw * 32
}

__global__ void k_warp_split(const uint32_t *__restrict__ slen, uint32_t nzr, uint32_t W0,
                             uint32_t th, int wpk2, int nosort, WarpSplit *__restrict__ ws,
                             unsigned long long *__restrict__ count,
                             unsigned long long *__restrict__ slots) {
  for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < W0;
       w += (size_t)gridDim.x * blockDim.x) {
    uint32_t A = slen[w * WS];  // sorted descending: the warp's first row is its longest
    uint32_t cnt = min((uint32_t)WS, nzr - (uint32_t)w * WS);
    if (nosort)
      for (uint32_t q = 1; q < cnt; q++) A = max(A, slen[w * WS + q]);
    WarpSplit s = split_rule(A, cnt, th, wpk2 != 0);
    ws[w] = s;
    unsigned long long c = s.full ? s.tpr : 1u;
    count[w] = c;
    slots[w] = c * WS * (unsigned long long)s.steps;
  }
}

__global__ void k_warp_expand(const WarpSplit *__restrict__ ws, uint32_t W0,
                              const unsigned long long *__restrict__ ostart,
                              const unsigned long long *__restrict__ soff, int wpk2,
                              int32_t *__restrict__ warp_offsets, uint32_t *__restrict__ max_nz_rows,
                              uint32_t *__restrict__ tpr_out, uint32_t *__restrict__ row_off,
                              int4 *__restrict__ desc) {
  for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < W0;
       w += (size_t)gridDim.x * blockDim.x) {
    WarpSplit s = ws[w];
    uint32_t c = s.full ? s.tpr : 1u;
    for (uint32_t j = 0; j < c; j++) {
      size_t o = ostart[w] + j;
      unsigned long long off = soff[w] + (unsigned long long)j * WS * s.steps;
      uint32_t first_row = (uint32_t)w * WS + j * s.rows;
      warp_offsets[o] = (int32_t)off;
      max_nz_rows[o] = s.steps;
      if (wpk2) {
        tpr_out[o] = s.tpr;
        row_off[o] = first_row;
      }
      desc[o] = make_int4((int)off, (int)s.steps, (int)s.tpr, (int)first_row);
    }
  }
}

__global__ void k_warp_tail(int32_t *warp_offsets, uint32_t *row_off, uint32_t W, uint32_t nrows,
                            const unsigned long long *total_slots, int wpk2) {
  warp_offsets[W] = (int32_t)*total_slots;
  if (wpk2) row_off[W] = nrows;
}

// m[0] += sum A_w^2, m[1] += sum A_w, m[2] = max A_w (exact, any order).
__global__ void k_step_moments(const uint32_t *__restrict__ steps, uint32_t W, unsigned long long *__restrict__ m) {
  unsigned long long a2 = 0, a1 = 0, am = 0;
  for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < W; w += (size_t)gridDim.x * blockDim.x) {
    const unsigned long long a = steps[w];
    a2 += a * a;
    a1 += a;
    am = a > am ? a : am;
  }
  for (int o = 16; o; o >>= 1) {
    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    const unsigned long long b = __shfl_xor_sync(0xffffffffu, am, o);
    am = b > am ? b : am;
  }
  if ((threadIdx.x & 31) == 0 && a1) {
    atomicAdd(m, a2);
    atomicAdd(m + 1, a1);
    atomicMax(m + 2, am);
  }
}

// reorder_rows[rowptr[row] + e] for every entry e of sorted row p.
__global__ void k_reorder_rows(const WarpSplit *__restrict__ ws,
                               const unsigned long long *__restrict__ soff,
                               const int32_t *__restrict__ row_map, const uint32_t *__restrict__ slen,
                               const int32_t *__restrict__ rowptr, uint32_t nzr,
                               uint32_t *__restrict__ reorder_rows, int nocoal) {
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < nzr;
       p += (size_t)gridDim.x * blockDim.x) {
    size_t w = p / WS;
    uint32_t q = (uint32_t)(p % WS);
    WarpSplit s = ws[w];
    uint32_t j = 0, r = q;
    if (s.full) {
      j = q / s.rows;
      r = q % s.rows;
    }
    uint32_t base = (uint32_t)(soff[w] + (unsigned long long)j * WS * s.steps);
    uint32_t len = slen[p];
    uint32_t k0 = (uint32_t)rowptr[row_map[p]];
    if (nocoal) {  // WPK1 lane r holds its row's entries contiguously
      for (uint32_t e = 0; e < len; e++) reorder_rows[k0 + e] = base + r * s.steps + e;
      continue;
    }
    uint32_t lane0 = base + r * s.tpr;
    for (uint32_t e = 0; e < len; e++)
      reorder_rows[k0 + e] = lane0 + e / s.steps + WS * (e % s.steps);
  }
}

// ---------------------------------------------------------------------------
// process(): padded values / column indices, one warp per layout warp.
// ---------------------------------------------------------------------------
template <typename E>
__global__ void k_process(const int4 *__restrict__ desc, uint32_t W, const int32_t *__restrict__ row_map,
                          const int32_t *__restrict__ row_map_inv, const uint32_t *__restrict__ slen,
                          const int32_t *__restrict__ rowptr, uint32_t nzr, const E *__restrict__ vals,
                          const int32_t *__restrict__ cols, E *__restrict__ pv, int32_t *__restrict__ pc,
                          int renumber, int nocoal) {
  const int lane = threadIdx.x & 31;
  for (size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS; w < W;
       w += (size_t)gridDim.x * blockDim.x / WS) {
    int4 d = desc[w];
    uint32_t tpr = (uint32_t)d.z;
    uint32_t q = lane / tpr, t = lane % tpr;
    uint32_t p = (uint32_t)d.w + q;
    bool valid = p < nzr;
    uint32_t len = 0, k0 = 0;
    if (valid) {
      len = slen[p];
      k0 = (uint32_t)rowptr[row_map[p]];
    }
    const uint32_t A = (uint32_t)d.y;
    // interleaved: slot o + lane + 32 i; non-interleaved ablation: o + lane * A + i
    size_t slot = (size_t)(uint32_t)d.x + (nocoal ? (size_t)lane * A : (size_t)lane);
    const size_t stride = nocoal ? 1 : WS;
    for (uint32_t i = 0; i < A; i++, slot += stride) {
      uint32_t e = i + t * A;
      E v = E(0);
      int32_t c = 0;
      if (valid && e < len) {
        if (vals) v = vals[k0 + e];
        if (cols) {
          c = cols[k0 + e];
          if (renumber) c = row_map_inv[c];
        }
      }
      if (pv) pv[slot] = v;
      if (pc) pc[slot] = c;
    }
  }
}

__global__ void k_reorder_columns(const int32_t *__restrict__ cols, size_t nz,
                                  const int32_t *__restrict__ row_map_inv, int32_t *__restrict__ out) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nz;
       k += (size_t)gridDim.x * blockDim.x)
    out[k] = row_map_inv[cols[k]];
}

template <typename E>
__global__ void k_reorder_x(const E *__restrict__ x, const int32_t *__restrict__ row_map, uint32_t n,
                            E *__restrict__ out) {
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (size_t)gridDim.x * blockDim.x)
    out[p] = x[row_map[p]];
}

__global__ void k_check_cols(const int32_t *__restrict__ cols, size_t n, uint32_t ncols, int *bad) {
  int b = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    b += (uint32_t)cols[k] >= ncols;
  b = __reduce_add_sync(0xffffffffu, b);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(bad, b);
}

unsigned grid_for(size_t n, int bs) {
  size_t g = (n + bs - 1) / bs;
  if (g < 1) g = 1;
  if (g > 152u * 64u) g = 152u * 64u;  // grid-stride beyond 64 blocks per SM
  return (unsigned)g;
}

}  // namespace

// ---------------------------------------------------------------------------
// Stable sort of n (key, value) pairs by the low `bits` bits of the key;
// buffers 0 hold the input, *out = index (0/1) of the buffers with the result.
wk_status radix_sort_pairs(uint32_t *k0, uint32_t *k1, uint32_t *v0, uint32_t *v1, uint32_t n, int bits,
                           cudaStream_t st, int *out) {
  uint32_t *kb[2] = {k0, k1}, *vb[2] = {v0, v1};
  const uint32_t ntiles = (n + RS_TILE - 1) / RS_TILE;
  int cur = 0;
  if (n > 0 && bits > 0) {
    DevBuf hist;
    WK_TRY(hist.alloc((size_t)256 * ntiles * 4));
    const unsigned nblk = (ntiles + RS_WARPS - 1) / RS_WARPS;
    for (int shift = 0; shift < bits; shift += 8) {
      k_radix_up<<<nblk, RS_WARPS * 32, 0, st>>>(kb[cur], n, shift, hist.as<uint32_t>(), ntiles);
      WK_CHECK_LAUNCH();
      WK_TRY(exclusive_scan<uint32_t>(hist.as<uint32_t>(), hist.as<uint32_t>(), (size_t)256 * ntiles, nullptr, st));
      k_radix_down<<<nblk, RS_WARPS * 32, 0, st>>>(kb[cur], vb[cur], kb[cur ^ 1], vb[cur ^ 1], n, shift,
                                                   hist.as<uint32_t>(), ntiles);
      WK_CHECK_LAUNCH();
      cur ^= 1;
    }
  }
  *out = cur;
  return WK_OK;
}

wk_status scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *d_total, cudaStream_t st) {
  return exclusive_scan<uint32_t>(in, out, n, d_total, st);
}

wk_status build_layout(wk_layout *l, const int32_t *d_rowptr, int kind, int32_t threshold,
                       cudaStream_t st, int variant) {
  const uint32_t n = l->info.nrows, nz = l->info.nz;
  const bool wpk2 = kind == WK_WPK2;
  if (wpk2 && variant) return set_error(WK_ERR_INVALID, "the ablation layouts are WPK1 layouts");
  const int nosort = (variant & WK_ABL_NOSORT) ? 1 : 0, nocoal = (variant & WK_ABL_NOCOALESCE) ? 1 : 0;
  l->info.kind = kind;
  l->info.variant = (uint32_t)variant;
  l->info.nmax_per_thread = wpk2 ? (uint32_t)threshold : 0u;

  // 1. lengths, checks
  DevBuf len, stats;
  WK_TRY(len.alloc((size_t)n * 4));
  WK_TRY(stats.alloc(8 * sizeof(unsigned)));
  WK_CUDA(cudaMemsetAsync(stats.p, 0, 8 * sizeof(unsigned), st));
  k_rowlen<<<grid_for(n, 256), 256, 0, st>>>(d_rowptr, n, len.as<uint32_t>(), stats.as<unsigned>());
  WK_CHECK_LAUNCH();
  unsigned hs[8];
  WK_CUDA(cudaMemcpyAsync(hs, stats.p, sizeof hs, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  if (hs[3] != 0) return set_error(WK_ERR_INVALID, "rowptr[0] = %d, expected 0", (int)hs[3]);
  if (hs[2]) return set_error(WK_ERR_INVALID, "rowptr is not monotone");
  if (hs[4] != nz)
    return set_error(WK_ERR_INVALID, "rowptr[nrows] = %u does not equal nz = %u", hs[4], nz);
  const uint32_t maxlen = hs[0], nzr = hs[1];
  l->info.nznrows = nzr;

  // 2-3. sort, maps
  DevBuf kb[2], vb[2];
  for (int i = 0; i < 2; i++) {
    WK_TRY(kb[i].alloc((size_t)n * 4));
    WK_TRY(vb[i].alloc((size_t)n * 4));
  }
  k_init_keys<<<grid_for(n, 256), 256, 0, st>>>(len.as<uint32_t>(), n, maxlen, kb[0].as<uint32_t>(),
                                                vb[0].as<uint32_t>(), nosort);
  WK_CHECK_LAUNCH();
  int bits = 0;
  while (bits < 32 && (maxlen >> bits)) bits++;
  if (nosort) bits = 1;
  int cur = 0;
  WK_TRY(radix_sort_pairs(kb[0].as<uint32_t>(), kb[1].as<uint32_t>(), vb[0].as<uint32_t>(), vb[1].as<uint32_t>(), n,
                          bits, st, &cur));
  LayoutDev &d = l->d;
  WK_TRY(l->bufs[0].alloc((size_t)n * 4));
  WK_TRY(l->bufs[1].alloc((size_t)n * 4));
  WK_TRY(l->bufs[8].alloc((size_t)n * 4));
  d.row_map = l->bufs[0].as<int32_t>();
  d.row_map_inv = l->bufs[1].as<int32_t>();
  d.slen = l->bufs[8].as<uint32_t>();
  d.rowptr = const_cast<int32_t *>(d_rowptr);
  k_finish_sort<<<grid_for(n, 256), 256, 0, st>>>(vb[cur].as<uint32_t>(), len.as<uint32_t>(), n, d.row_map,
                                                  d.row_map_inv, d.slen);
  WK_CHECK_LAUNCH();

  // 4. warp tables
  const uint32_t W0 = (nzr + WS - 1) / WS;
  DevBuf wsb, cnt, slots, tot;
  WK_TRY(wsb.alloc((size_t)W0 * sizeof(WarpSplit)));
  WK_TRY(cnt.alloc((size_t)W0 * 8));
  WK_TRY(slots.alloc((size_t)W0 * 8));
  WK_TRY(tot.alloc(3 * 8));
  auto *totals = tot.as<unsigned long long>();
  if (W0) {
    k_warp_split<<<grid_for(W0, 256), 256, 0, st>>>(d.slen, nzr, W0, (uint32_t)threshold, wpk2, nosort,
                                                    wsb.as<WarpSplit>(), cnt.as<unsigned long long>(),
                                                    slots.as<unsigned long long>());
    WK_CHECK_LAUNCH();
  }
  WK_TRY(exclusive_scan<unsigned long long>(cnt.as<unsigned long long>(), cnt.as<unsigned long long>(),
                                            W0, totals, st));
  WK_TRY(exclusive_scan<unsigned long long>(slots.as<unsigned long long>(),
                                            slots.as<unsigned long long>(), W0, totals + 1, st));
  unsigned long long ht[2];
  WK_CUDA(cudaMemcpyAsync(ht, totals, sizeof ht, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  if (ht[1] > 0x7fffffffULL)
    return set_error(WK_ERR_OVERFLOW,
                     "allocate_nz = %llu exceeds the int32 warp_offsets of the layout", ht[1]);
  const uint32_t W = (uint32_t)ht[0];
  l->info.nwarps = W;
  l->info.allocate_nz = (uint32_t)ht[1];
  if (wpk2) {
    // min/max over non-empty rows: sorted descending
    uint32_t mm[2] = {n, 0};
    if (nzr) {
      WK_CUDA(cudaMemcpyAsync(&mm[0], d.slen + (nzr - 1), 4, cudaMemcpyDeviceToHost, st));
      WK_CUDA(cudaMemcpyAsync(&mm[1], d.slen, 4, cudaMemcpyDeviceToHost, st));
      WK_CUDA(cudaStreamSynchronize(st));
    }
    l->info.min_nz = mm[0];
    l->info.max_nz = mm[1];
  }
  WK_TRY(l->bufs[3].alloc((size_t)(W + 1) * 4));
  WK_TRY(l->bufs[4].alloc((size_t)W * 4));
  WK_TRY(l->bufs[9].alloc((size_t)W * sizeof(int4)));
  d.warp_offsets = l->bufs[3].as<int32_t>();
  d.max_nz_rows = l->bufs[4].as<uint32_t>();
  d.warp_desc = l->bufs[9].as<int4>();
  if (wpk2) {
    WK_TRY(l->bufs[5].alloc((size_t)W * 4));
    WK_TRY(l->bufs[6].alloc((size_t)(W + 1) * 4));
    d.threads_per_row = l->bufs[5].as<uint32_t>();
    d.row_offset_warp = l->bufs[6].as<uint32_t>();
  }
  if (W0) {
    k_warp_expand<<<grid_for(W0, 256), 256, 0, st>>>(wsb.as<WarpSplit>(), W0, cnt.as<unsigned long long>(),
                                                     slots.as<unsigned long long>(), wpk2, d.warp_offsets,
                                                     d.max_nz_rows, d.threads_per_row, d.row_offset_warp,
                                                     d.warp_desc);
    WK_CHECK_LAUNCH();
  }
  k_warp_tail<<<1, 1, 0, st>>>(d.warp_offsets, d.row_offset_warp, W, n, totals + 1, wpk2);
  WK_CHECK_LAUNCH();
  if (W) {  // sum A_w^2, sum A_w and max A_w (exact integers, any order)
    WK_CUDA(cudaMemsetAsync(tot.p, 0, 24, st));
    k_step_moments<<<grid_for(W, 256), 256, 0, st>>>(d.max_nz_rows, W, totals);
    WK_CHECK_LAUNCH();
    unsigned long long hm[3];
    WK_CUDA(cudaMemcpyAsync(hm, totals, sizeof hm, cudaMemcpyDeviceToHost, st));
    WK_CUDA(cudaStreamSynchronize(st));
    l->mean_steps = hm[1] ? (double)hm[0] / (double)hm[1] : 0.0;
    l->sum_steps = (double)hm[1];
    l->max_steps = (double)hm[2];
  }

  // 5. reorder_rows
  WK_TRY(l->bufs[2].alloc((size_t)nz * 4));
  d.reorder_rows = l->bufs[2].as<uint32_t>();
  if (nzr) {
    k_reorder_rows<<<grid_for(nzr, 256), 256, 0, st>>>(wsb.as<WarpSplit>(), slots.as<unsigned long long>(),
                                                       d.row_map, d.slen, d_rowptr, nzr, d.reorder_rows, nocoal);
    WK_CHECK_LAUNCH();
  }
  WK_CUDA(cudaStreamSynchronize(st));  // temporaries are freed on return
  return WK_OK;
}

wk_status launch_process(const wk_layout *l, const void *vals, int elem_bytes, const int32_t *cols,
                         void *pvals, int32_t *pcols, bool renumber, cudaStream_t st) {
  const uint32_t W = l->info.nwarps;
  if (W == 0) return WK_OK;
  const LayoutDev &d = l->d;
  unsigned grid = grid_for((size_t)W * WS, 256);
#define WK_PROCESS(E)                                                                          \
  k_process<E><<<grid, 256, 0, st>>>(d.warp_desc, W, d.row_map, d.row_map_inv, d.slen, d.rowptr, \
                                     l->info.nznrows, (const E *)vals, cols, (E *)pvals, pcols,   \
                                     renumber ? 1 : 0, (l->info.variant & WK_ABL_NOCOALESCE) ? 1 : 0)
  switch (elem_bytes) {
    case 8: WK_PROCESS(unsigned long long); break;
    case 4: WK_PROCESS(uint32_t); break;
    case 2: WK_PROCESS(unsigned short); break;
    default: return set_error(WK_ERR_INVALID, "unsupported element size %d", elem_bytes);
  }
#undef WK_PROCESS
  WK_CHECK_LAUNCH();
  return WK_OK;
}

wk_status launch_reorder_columns(const wk_layout *l, const int32_t *cols, int32_t *out,
                                 cudaStream_t st) {
  size_t nz = l->info.nz;
  if (!nz) return WK_OK;
  k_reorder_columns<<<grid_for(nz, 256), 256, 0, st>>>(cols, nz, l->d.row_map_inv, out);
  WK_CHECK_LAUNCH();
  return WK_OK;
}

wk_status launch_reorder_x(const wk_layout *l, const void *x, void *xout, int eb, cudaStream_t st) {
  uint32_t n = l->info.nrows;
  if (!n) return WK_OK;
  unsigned g = grid_for(n, 256);
  switch (eb) {
    case 8: k_reorder_x<unsigned long long><<<g, 256, 0, st>>>((const unsigned long long *)x, l->d.row_map, n, (unsigned long long *)xout); break;
    case 4: k_reorder_x<uint32_t><<<g, 256, 0, st>>>((const uint32_t *)x, l->d.row_map, n, (uint32_t *)xout); break;
    case 2: k_reorder_x<unsigned short><<<g, 256, 0, st>>>((const unsigned short *)x, l->d.row_map, n, (unsigned short *)xout); break;
    default: return set_error(WK_ERR_INVALID, "unsupported element size %d", eb);
  }
  WK_CHECK_LAUNCH();
  return WK_OK;
}

wk_status launch_check_cols(const int32_t *cols, size_t n, uint32_t ncols, int *d_bad, cudaStream_t st) {
  if (!n) return WK_OK;
  k_check_cols<<<grid_for(n, 256), 256, 0, st>>>(cols, n, ncols, d_bad);
  WK_CHECK_LAUNCH();
  return WK_OK;
}

wk_status scan_u64(const unsigned long long *in, unsigned long long *out, size_t n, unsigned long long *d_total,
                   cudaStream_t st) {
  return exclusive_scan<unsigned long long>(in, out, n, d_total, st);
}

}  // namespace wk
