// wk_adjoint.cu -- adjoint of the WPK SpMV: dx = A^T dy through a transposed
// WPK layout built on the device, and dvals[k] = dy[row(k)] * x[col(k)] over
// the stored pattern (CSR order).  Deterministic: no atomics on values.
//
// Build: the CSR entries of A (recovered from the forward engine through
// reorder_rows) are stably sorted by column on the device, which gives the
// CSR of A^T with rows in ascending order and the permutation perm[k'] = k
// (entry k' of A^T is entry k of A).  A^T's layout and engine then come from
// the same device scan and process as A's.
//
// Structurally symmetric matrices (every finite-element matrix) with sorted
// rows give A^T the same row offsets and columns as A, so with the same
// kind/threshold the two layouts coincide slot for slot and the transposed
// engine's padded values are the mirror values A[c][r] at A's slot (r, c).
// One fused pass over A's layout then reads mirror value + column per slot,
// accumulates dx[r] = sum_c A[c][r] dy[c] and writes dvals for the same slot.
#include <algorithm>

#include "wk_internal.cuh"
#include "wk_spmv_core.cuh"

struct wk_adjoint {
  wk_engine *fwd = nullptr;  // not owned: must outlive the adjoint
  wk_layout *tl = nullptr;   // transposed layout (reference held)
  wk_engine *te = nullptr;   // transposed engine (owned)
  wk::DevBuf perm;           // [nz] A^T CSR entry -> A CSR index
  wk::DevBuf tmp;            // [nz] value staging for refreshes
  wk::DevBuf xdy;            // [nrows] interleaved (x, dy) of the fused pass
  wk::WinSet win;            // x windows of the forward layout (fused slot-order pass, fp32)
  bool win_built = false;
  bool symmetric = false;
  int kind = 1;
  int32_t threshold = 0;
};

namespace wk {
namespace {

constexpr int WS = 32;

unsigned grid_for(size_t n, int bs) {
  size_t g = (n + bs - 1) / bs;
  if (g < 1) g = 1;
  if (g > 152u * 64u) g = 152u * 64u;
  return (unsigned)g;
}

// CSR-order columns and the identity (sort keys / values), from A's padded arrays.
__global__ void k_csr_cols(const int32_t *__restrict__ pcols, const uint32_t *__restrict__ reorder_rows, uint32_t nz,
                           uint32_t *__restrict__ keys, uint32_t *__restrict__ idx) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nz; k += (size_t)gridDim.x * blockDim.x) {
    keys[k] = (uint32_t)pcols[reorder_rows[k]];
    idx[k] = (uint32_t)k;
  }
}

template <typename E>
__global__ void k_gather_padded(const E *__restrict__ pv, const uint32_t *__restrict__ reorder_rows, uint32_t nz,
                                E *__restrict__ out) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nz; k += (size_t)gridDim.x * blockDim.x)
    out[k] = pv[reorder_rows[k]];
}

template <typename E>
__global__ void k_permute(const E *__restrict__ in, const uint32_t *__restrict__ perm, uint32_t nz, E *__restrict__ out) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nz; k += (size_t)gridDim.x * blockDim.x)
    out[k] = in[perm[k]];
}

__global__ void k_count(const uint32_t *__restrict__ keys, uint32_t nz, uint32_t *__restrict__ counts) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nz; k += (size_t)gridDim.x * blockDim.x)
    atomicAdd(&counts[keys[k]], 1u);  // integer counts: order-independent
}

__global__ void k_row_of(const int32_t *__restrict__ rowptr, uint32_t n, uint32_t *__restrict__ row_of) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x)
    for (int32_t k = rowptr[r]; k < rowptr[r + 1]; k++) row_of[k] = (uint32_t)r;
}

__global__ void k_count_diff(const uint32_t *__restrict__ a, const uint32_t *__restrict__ b, size_t n,
                             unsigned *__restrict__ diff) {
  unsigned c = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    c += a[k] != b[k];
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(diff, c);
}

// x and dy interleaved, so a slot needs one 8- (fp32) or 16-byte (fp64) gather.
template <typename T>
struct Pair;
template <>
struct Pair<float> {
  typedef float2 type;
};
template <>
struct Pair<double> {
  typedef double2 type;
};

template <typename T>
__global__ void k_interleave(const T *__restrict__ x, const T *__restrict__ dy, uint32_t n,
                             typename Pair<T>::type *__restrict__ xdy) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    typename Pair<T>::type v;
    v.x = x[i];
    v.y = dy[i];
    xdy[i] = v;
  }
}

// dvals for the slots of A's layout, indexed by padded slot (padding gets 0),
// for a general pattern: one warp per layout warp, one coalesced streaming
// store per step (evict-first: the gradient must not displace x in L2; 2-3 %
// faster, hex 64^3 with 1 % of the entries dropped).
template <typename T>
__global__ void k_dvals_slots(const int4 *__restrict__ desc, uint32_t W, const int32_t *__restrict__ row_map,
                              const uint32_t *__restrict__ slen, uint32_t nzr, const int32_t *__restrict__ pc,
                              const T *__restrict__ x, const T *__restrict__ dy, T *__restrict__ dvals) {
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w >= W) return;
  const int4 d = desc[w];
  const uint32_t T_ = (uint32_t)d.z, A = (uint32_t)d.y, t = lane % T_;
  const uint32_t p = (uint32_t)d.w + lane / T_;
  const bool valid = p < nzr;
  uint32_t len = 0;
  T dyr = T(0);
  if (valid) {
    len = slen[p];
    dyr = dy[row_map[p]];
  }
  size_t slot = (size_t)(uint32_t)d.x + lane;
#pragma unroll 4
  for (uint32_t i = 0; i < A; i++, slot += WS) {
    const bool real = valid && i + t * A < len;
    __stcs(dvals + slot, real ? dyr * __ldg(x + __ldcs(pc + slot)) : T(0));
  }
}

// Fused adjoint for the coinciding layouts of a structurally symmetric A:
// dx[r] = sum over row r's slots of mirror value * dy[c], and dvals for each
// slot, with one gather of the interleaved (x, dy) pair per slot.  The
// streaming pattern is the fast SpMV's with S slots per lane (8 for fp32, 4
// for fp64: 256-bit loads and stores; measured faster than 4 fp32 slots with
// 128-bit accesses despite the lower occupancy).  dvals go to the same slots
// with one vector store per lane, or (CSR order) through shared memory, which
// measured 11 % faster (fp32) than the 4-slot kernel it replaced.  It serves
// fp64; the fp32 gradient runs k_adjoint_sym_staged (slot order, 0.105
// against 0.1415 ms at hex 64^3) or k_adjoint_sym_staged_csr (CSR order,
// 0.1584 against 0.207 ms).  For fp64 this kernel stayed
// ahead of a register-staged form of that kernel (0.262 against 0.264 ms,
// 0.289 with x windows).
template <typename T>
struct AdjSlots {
  static constexpr int value = core::SlotsPerLane<T>::value;
};
#define kAdjS (AdjSlots<T>::value)
// dvals are written once and not read again by the kernel: evict-first in L2
// (and streaming stores in the tail and the CSR flush), so they do not
// displace the gathered (x, dy) pairs -- 5 % faster in slot order, 8 % with
// 16-bit columns, fp32 hex 64^3.
__device__ __forceinline__ void st_words(void *p, const uint32_t (&w)[8], uint64_t pol) {
  asm volatile("st.global.L1::no_allocate.L2::cache_hint.v8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8}, %9;" ::"l"(p),
               "r"(w[0]), "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7]), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void put_word(uint32_t *w, int k, float v) { w[k] = __float_as_uint(v); }
__device__ __forceinline__ void put_word(uint32_t *w, int k, double v) {
  w[2 * k] = (uint32_t)__double2loint(v);
  w[2 * k + 1] = (uint32_t)__double2hiint(v);
}

// One layout warp of the slot-order adjoint; columns as int32 (C = int32_t)
// or as 16-bit offsets from `base` (C = uint16_t).  Returns layout lane
// `lane`'s sum of mirror value * dy[c].
// CSR: dvals in CSR order.  The gradients of a chunk of steps are staged in
// `stg` as [layout lane][step] and written row segment by row segment: the
// entries of one layout lane in one chunk are contiguous in CSR order
// (skb[l] + step), so one warp store writes 32 consecutive values of one row
// (fp32: 32-step chunks, 6 % faster than 16) or a half-warp 16 (fp64: 16-step
// chunks keep a block's static shared memory under 48 KB).
template <typename T>
struct CsrChunk {
  static constexpr int value = sizeof(T) == 4 ? 32 : 16;
};
#define ADJ_CSR_CHUNK (CsrChunk<T>::value)
template <typename T>
__device__ __forceinline__ void flush_csr_chunk(T *__restrict__ dvals, const T (*stg)[ADJ_CSR_CHUNK + 1],
                                                const int *__restrict__ skb, const int *__restrict__ sel,
                                                uint32_t c0, uint32_t nst, uint32_t lane) {
  __syncwarp();
  const uint32_t jj = lane % ADJ_CSR_CHUNK;
#pragma unroll 4
  for (uint32_t sg = 0; sg < 32; sg += 32 / ADJ_CSR_CHUNK) {
    const uint32_t l = sg + lane / ADJ_CSR_CHUNK;
    const uint32_t e = c0 + jj;
    if (jj < nst && (int)e < sel[l]) __stcs(dvals + (size_t)skb[l] + e, stg[l][jj]);
  }
  __syncwarp();
}

// The same for the staged kernel's 32-step chunks: each lane computes its
// own row's store limit and CSR offset for the chunk once, and the loop over
// rows takes them by shuffle (two shuffles, one compare and one store per
// row segment).
__device__ __forceinline__ void flush_csr_chunk32(float *__restrict__ dvals, const float (*stg)[33],
                                                  const int *__restrict__ skb, const int *__restrict__ sel,
                                                  uint32_t c0, uint32_t nst, uint32_t lane) {
  __syncwarp();
  const int lim_me = min((int)nst, sel[lane] - (int)c0);  // entries of this lane's row in the chunk
  const int off_me = skb[lane] + (int)c0;
#pragma unroll 8
  for (int l = 0; l < 32; l++) {
    const int lim = __shfl_sync(0xffffffffu, lim_me, l);
    const int off = __shfl_sync(0xffffffffu, off_me, l);
    if ((int)lane < lim) __stcs(dvals + (uint32_t)(off + (int)lane), stg[l][lane]);
  }
  __syncwarp();
}

// dvals in CSR order for a general pattern.  Lane l's entries of one step
// belong to different rows, so storing them directly scatters 32 single
// values per warp store; instead a chunk of steps is staged in shared memory
// as [layout lane][step] and written row segment by row segment
// (flush_csr_chunk): 32 (fp32) or 16 (fp64) consecutive entries of one row
// per warp store.
template <typename T>
__global__ void __launch_bounds__(256) k_dvals_csr(const int4 *__restrict__ desc, uint32_t W,
                                                   const int32_t *__restrict__ row_map,
                                                   const uint32_t *__restrict__ slen,
                                                   const int32_t *__restrict__ rowptr, uint32_t nzr,
                                                   const int32_t *__restrict__ pc, const T *__restrict__ x,
                                                   const T *__restrict__ dy, T *__restrict__ dvals) {
  __shared__ int s_el[8][32];
  __shared__ int s_kb[8][32];
  __shared__ T s_stage[8][32][ADJ_CSR_CHUNK + 1];
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w >= W) return;  // warp-uniform: the staging below is per warp
  const int4 d = desc[w];
  const uint32_t T_ = (uint32_t)d.z, A = (uint32_t)d.y, t = lane % T_;
  const uint32_t p = (uint32_t)d.w + lane / T_;
  int el = 0, kb = 0;
  T dyr = T(0);
  if (p < nzr) {
    const int32_t row = row_map[p];
    el = max(0, min((int)A, (int)slen[p] - (int)(t * A)));
    kb = rowptr[row] + (int)(t * A);
    dyr = dy[row];
  }
  const uint32_t wib = threadIdx.x / WS;
  int *sel = s_el[wib], *skb = s_kb[wib];
  T(*stg)[ADJ_CSR_CHUNK + 1] = s_stage[wib];
  sel[lane] = el;
  skb[lane] = kb;
  size_t slot = (size_t)(uint32_t)d.x + lane;
  for (uint32_t i = 0; i < A; i++, slot += WS) {
    stg[lane][i % ADJ_CSR_CHUNK] = (int)i < el ? dyr * __ldg(x + __ldcs(pc + slot)) : T(0);
    if ((i + 1) % ADJ_CSR_CHUNK == 0) flush_csr_chunk(dvals, stg, skb, sel, i + 1 - ADJ_CSR_CHUNK, ADJ_CSR_CHUNK, lane);
  }
  const uint32_t c0 = (A / ADJ_CSR_CHUNK) * ADJ_CSR_CHUNK;
  if (A > c0) flush_csr_chunk(dvals, stg, skb, sel, c0, A - c0, lane);
}

template <typename T, typename C, bool CSR, int DEPTH>
__device__ __forceinline__ T adjoint_warp_slots(const int4 d, const C *__restrict__ cp0, int base,
                                                const T *__restrict__ tv, const typename Pair<T>::type *__restrict__ xdy,
                                                T *__restrict__ dvals, const T *__restrict__ sdy,
                                                const int *__restrict__ sel, const int *__restrict__ skb,
                                                T (*stg)[ADJ_CSR_CHUNK + 1], T dyr, int el,
                                                uint32_t lane, uint64_t pol) {
  using namespace core;
  typedef typename Pair<T>::type P;
  constexpr int S = kAdjS, R = 32 / S;
  const uint32_t A = (uint32_t)d.y;
  const size_t o = (size_t)(uint32_t)d.x;
  T acc[S];
#pragma unroll
  for (int m = 0; m < S; m++) acc[m] = T(0);
  const uint32_t units = A / S, rem = A % S, sl = lane / R;
  const T *vp = tv + o + S * lane;
  const C *cp = cp0 + S * lane;
  T *dp = dvals + o + S * lane;
  constexpr int NV = S * sizeof(T) / 4, NC = S * sizeof(C) / 4;
  // the values and columns of units u .. u+DEPTH-1 in flight while unit u is
  // consumed
  uint32_t wv[DEPTH][NV], wc[DEPTH][NC];
#pragma unroll
  for (int s = 0; s < DEPTH; s++)
    if ((uint32_t)s < units) {
      ld_words(vp + s * S * WS, wv[s], pol);
      ld_words(cp + s * S * WS, wc[s], pol);
    }
#pragma unroll 1
  for (uint32_t u = 0; u < units; u++) {
    uint32_t nv[NV], nc[NC], wd[NV];
    if (u + DEPTH < units) {
      ld_words(vp + DEPTH * S * WS, nv, pol);
      ld_words(cp + DEPTH * S * WS, nc, pol);
    }
    const int step = (int)(u * S + sl);
#pragma unroll
    for (int m = 0; m < S; m++) {
      const P g = __ldg(xdy + word_col<C>(wc[0], m, base));
      acc[m] = fma(word_val<T>(wv[0], m), g.y, acc[m]);
      const int q = S * (int)(lane % R) + m;
      const T dv = step < sel[q] ? sdy[q] * g.x : T(0);
      if constexpr (CSR)
        stg[q][step % ADJ_CSR_CHUNK] = dv;
      else
        put_word(wd, m, dv);
    }
    if constexpr (CSR) {
      if (((u + 1) * S) % ADJ_CSR_CHUNK == 0)
        flush_csr_chunk(dvals, stg, skb, sel, (u + 1) * S - ADJ_CSR_CHUNK, ADJ_CSR_CHUNK, lane);
    } else {
      st_words(dp, wd, pol);
    }
#pragma unroll
    for (int s = 0; s + 1 < DEPTH; s++) {
#pragma unroll
      for (int q = 0; q < NV; q++) wv[s][q] = wv[s + 1][q];
#pragma unroll
      for (int q = 0; q < NC; q++) wc[s][q] = wc[s + 1][q];
    }
#pragma unroll
    for (int q = 0; q < NV; q++) wv[DEPTH - 1][q] = nv[q];
#pragma unroll
    for (int q = 0; q < NC; q++) wc[DEPTH - 1][q] = nc[q];
    vp += S * WS;
    cp += S * WS;
    dp += S * WS;
  }
  T tail = T(0);
  const size_t ut = (size_t)units * S * WS + lane;
  for (uint32_t i = 0; i < rem; i++) {
    const size_t k = ut + (size_t)i * WS;
    const P g = __ldg(xdy + ld_col1(cp0 + k, base, pol));
    tail = fma(__ldcs(tv + o + k), g.y, tail);
    const T dv = (int)(units * S + i) < el ? dyr * g.x : T(0);
    if constexpr (CSR)
      stg[lane][(units * S + i) % ADJ_CSR_CHUNK] = dv;
    else
      __stcs(dvals + o + k, dv);
  }
  if constexpr (CSR) {  // the last, partial chunk
    const uint32_t c0 = (units * S / ADJ_CSR_CHUNK) * ADJ_CSR_CHUNK;
    if (A > c0) flush_csr_chunk(dvals, stg, skb, sel, c0, A - c0, lane);
  }
  return combine_lanes<S>(acc, lane) + tail;
}

// Launch shape per value type and dvals order: units of loads in flight per
// lane (DEPTH), warps per block and the blocks per SM the registers are
// capped for.  fp32: two units in flight, five blocks of 4 warps (96
// registers), 5 % faster in slot order than one unit with three blocks of 8
// warps (80 registers) at hex 64^3; the rows' dy / slot counts are read from
// shared memory instead of held in 16 registers per lane.  fp64 in slot
// order runs 4 % faster with four blocks of 8 warps (64 registers) than with
// three; a ring of load sets unrolled over the loop (no register moves)
// measured slower for fp32 and fp64 slot order.
template <typename T, bool CSR>
struct AdjCfg {
  static constexpr int depth = sizeof(T) == 4 ? 2 : 1;
  static constexpr int warps = sizeof(T) == 4 ? 4 : 8;
  static constexpr int min_blocks = sizeof(T) == 4 ? 5 : (CSR ? 3 : 4);
};

// CSR: dvals in CSR order (rowptr gives each row's first entry), staged in
// shared memory per chunk of steps.
template <typename T, bool COMP, bool CSR>
__global__ void __launch_bounds__(AdjCfg<T, CSR>::warps * 32, AdjCfg<T, CSR>::min_blocks) k_adjoint_sym_slots(
    const int4 *__restrict__ desc, uint32_t W, const int32_t *__restrict__ row_map, const uint32_t *__restrict__ slen,
    const int32_t *__restrict__ rowptr, uint32_t nzr, uint32_t nrows, const int32_t *__restrict__ pc,
    const uint16_t *__restrict__ c16, const int32_t *__restrict__ c32, const int4 *__restrict__ cdesc,
    const T *__restrict__ tv, const typename Pair<T>::type *__restrict__ xdy, T *__restrict__ dx,
    T *__restrict__ dvals) {
  using namespace core;
  constexpr int NW = AdjCfg<T, CSR>::warps, DEPTH = AdjCfg<T, CSR>::depth;
  __shared__ T s_dy[NW][32];
  __shared__ int s_el[NW][32];
  __shared__ int s_kb[CSR ? NW : 1][32];
  __shared__ T s_stage[CSR ? NW : 1][32][ADJ_CSR_CHUNK + 1];
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w < W) {
    const uint64_t pol = policy_evict_first();
    const int4 d = desc[w];
    const uint32_t T_ = (uint32_t)d.z, A = (uint32_t)d.y, t = lane % T_;
    const uint32_t p = (uint32_t)d.w + lane / T_;
    const bool valid = p < nzr;
    int32_t row = 0;
    int el = 0, kb = 0;
    T dyr = T(0);
    if (valid) {
      row = row_map[p];
      el = max(0, min((int)A, (int)slen[p] - (int)(t * A)));
      dyr = xdy[row].y;
      if (CSR) kb = rowptr[row] + (int)(t * A);
    }
    // the warp's 32 row gradients and slot counts (and CSR offsets), read by
    // the lanes that store those rows' slots
    const uint32_t wib = threadIdx.x / WS;
    T *sdy = s_dy[wib];
    int *sel = s_el[wib];
    int *skb = s_kb[CSR ? wib : 0];
    T(*stg)[ADJ_CSR_CHUNK + 1] = s_stage[CSR ? wib : 0];
    sdy[lane] = dyr;
    sel[lane] = el;
    if (CSR) skb[lane] = kb;
    __syncwarp();
    T total;
    if constexpr (COMP) {
      const int4 cd = cdesc[w];
      if (cd.y == 0)
        total = adjoint_warp_slots<T, uint16_t, CSR, DEPTH>(d, c16 + (uint32_t)d.x, cd.x, tv, xdy, dvals, sdy, sel, skb, stg,
                                                     dyr, el, lane, pol);
      else
        total = adjoint_warp_slots<T, int32_t, CSR, DEPTH>(d, c32 + (uint32_t)cd.z, 0, tv, xdy, dvals, sdy, sel, skb, stg,
                                                    dyr, el, lane, pol);
    } else {
      total = adjoint_warp_slots<T, int32_t, CSR, DEPTH>(d, pc + (uint32_t)d.x, 0, tv, xdy, dvals, sdy, sel, skb, stg, dyr,
                                                  el, lane, pol);
    }
    for (uint32_t k = 1; k < T_; k <<= 1) total += __shfl_down_sync(0xffffffffu, total, k);
    if (valid && (lane & (T_ - 1)) == 0) dx[row] = total;
  }
  for (size_t q = (size_t)nzr + (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nrows;
       q += (size_t)gridDim.x * blockDim.x)
    dx[row_map[q]] = T(0);
}

// Fused slot-order adjoint with the matrix stream copied into shared memory
// (fp32).  Each unit of S steps of mirror values and columns is copied by
// cp.async (16 bytes per lane and instruction, L2 evict-first) into a ring
// of STAGES tiles, STAGES - 1 units ahead, and read back step by step, so
// lane l handles its own layout lane: dx accumulates in one register in step
// order (no cross-lane combine), the row's dy and slot count stay in
// registers, and each step's 32 gradients leave in one coalesced 128-byte
// streaming store.  A warp with an x window (WinSet) copies its (x, dy)
// pairs into shared memory with the first unit's copies (so their L2
// latency overlaps the stream's), streams 16-bit window positions instead of
// 32-bit columns, and gathers from shared memory; a warp without one gathers
// x and dy from their vectors.  Full units run an unguarded step loop (a
// guard per step for the partial last unit cost 21 % more instructions and
// 7 % of the time).  Measured at hex 64^3 (fp32, three of 25,747 layout warps
// without a window): 0.105 ms with four stages and four blocks per SM,
// against 0.1415 for k_adjoint_sym_slots; three stages 0.106, two 0.109.
// A persistent form (each warp walking layout warps gw, gw +
// NW, ... with the ring and a double-buffered window running on across
// them, so that no layout warp's descriptor and window latency is exposed)
// measured 0.123-0.129 ms: the second window buffer costs a block per SM.
constexpr int ADJ_SW = 4;  // warps per block

// One layout warp.  Units of S steps; the last unit may be partial (the
// remainder steps ride in the same ring, copied by the lanes that hold
// them).  The first STAGES - 1 units are issued as soon as the descriptors
// are known, before the row data and the window, which join the first
// group.  WIN: the warp has an x window (its (x, dy) pairs staged in `wp`,
// the stream carries 16-bit window positions); otherwise the stream carries
// 32-bit columns and x, dy are gathered from their vectors.  DX = false:
// the value gradient alone (no mirror values streamed, no dx; the window
// holds x only).  CSR: dvals in CSR order (`cs`: the warp's staging of
// ADJ_CSR_STAGED-step chunks as [layout lane][step], flushed row segment by
// row segment).
constexpr int ADJ_CSR_STAGED = 32;  // 16-step chunks (half-warp row segments) measured slower
struct CsrStage {
  float (*stg)[ADJ_CSR_STAGED + 1];
  int *skb, *sel;
  const int32_t *rowptr;
};
template <int STAGES, bool WIN, bool DX = true, bool CSR = false>
__device__ __forceinline__ float adjoint_warp_pipe(const int4 d, const int4 wd, const int2 *__restrict__ wch,
                                                   const int32_t *__restrict__ pc, const uint16_t *__restrict__ w16,
                                                   const float *__restrict__ tv, const float *__restrict__ x,
                                                   const float *__restrict__ dy, const int32_t *__restrict__ row_map,
                                                   const uint32_t *__restrict__ slen, uint32_t nzr, float2 *wp,
                                                   float *__restrict__ dvals, uint32_t *sv, uint32_t *sc,
                                                   uint32_t lane, uint64_t pol, int32_t &row, bool &valid,
                                                   const CsrStage cs = CsrStage{}) {
  using namespace core;
  constexpr int S = 8;                 // steps per unit (32 bytes of fp32 per lane)
  constexpr int NC = WIN ? S / 2 : S;  // column words per lane and unit
  constexpr int VSTAGE = S * WS, CSTAGE = NC * WS;  // words per tile
  const size_t o = (size_t)(uint32_t)d.x;
  const uint32_t A = (uint32_t)d.y, full = A / S, rem = A % S, units = full + (rem != 0);
  // unit u covers steps [u S, u S + S) of all lanes: S * 32 consecutive
  // slots, of which lane l copies S (and NC column words) from S l on; in a
  // partial unit only the lanes below 4 rem hold slots
  auto issue = [&](uint32_t u) {
    if (u < full || lane < 4 * rem) {
      const size_t g = o + (size_t)u * S * WS + S * lane;
      if constexpr (DX) {
        uint32_t *dv = sv + (u % STAGES) * VSTAGE + S * lane;
#pragma unroll
        for (int q = 0; q < S; q += 4) cp_async16(dv + q, tv + g + q, pol);
      }
      uint32_t *dc = sc + (u % STAGES) * CSTAGE + NC * lane;
      const uint32_t *gc =
          WIN ? reinterpret_cast<const uint32_t *>(w16 + g) : reinterpret_cast<const uint32_t *>(pc + g);
#pragma unroll
      for (int q = 0; q < NC; q += 4) cp_async16(dc + q, gc + q, pol);
    }
  };
#pragma unroll
  for (int s = 0; s < STAGES - 1; s++)
    if ((uint32_t)s < units) issue((uint32_t)s);
  // the lane's row: its dy and slot count
  const uint32_t T_ = (uint32_t)d.z, t = lane % T_;
  const uint32_t p = (uint32_t)d.w + lane / T_;
  valid = p < nzr;
  row = 0;
  int el = 0;
  float dyr = 0.f;
  if (valid) {
    row = row_map[p];
    el = max(0, min((int)A, (int)slen[p] - (int)(t * A)));
    dyr = dy[row];
  }
  if constexpr (CSR) {  // the lane's first CSR entry and entry count, for the flushes
    cs.skb[lane] = valid ? cs.rowptr[row] + (int)(t * A) : 0;
    cs.sel[lane] = el;
  }
  if constexpr (WIN) {
    // chunk q = {first column, window position | length << 16}, <= 32 columns
    const int nch = wd.y;
    const int2 mine = lane < (uint32_t)nch ? wch[wd.x + lane] : make_int2(0, 0);
    for (int q = 0; q < nch; q++) {
      const int c0 = __shfl_sync(0xffffffffu, mine.x, q);
      const int pl = __shfl_sync(0xffffffffu, mine.y, q);
      const int pos = (pl & 0xffff) + (int)lane;
      if (lane < (uint32_t)(pl >> 16) && pos < WIN_MAX) {
        cp_async_ca<4>(&wp[pos].x, x + c0 + (int)lane);
        if constexpr (DX) cp_async_ca<4>(&wp[pos].y, dy + c0 + (int)lane);
      }
    }
  }
  // group 0: units 0 .. STAGES - 2 and the window; groups 1 .. STAGES - 2
  // are empty, so that group u is complete once STAGES - 1 later ones are
  // committed
#pragma unroll
  for (int s = 0; s < STAGES - 1; s++) cp_async_commit();
  float acc = 0.f;
  for (uint32_t u = 0; u < units; u++) {
    if (u + STAGES - 1 < units) issue(u + STAGES - 1);
    cp_async_commit();
    cp_async_wait<STAGES - 1>();
    __syncwarp();
    const uint32_t *svs = sv + (u % STAGES) * VSTAGE;
    const uint32_t *scs = sc + (u % STAGES) * CSTAGE;
    float *dp = dvals + o + (size_t)u * S * WS + lane;
    auto step = [&](int st) {
      const int q = st * WS + (int)lane;
      float2 g;
      if constexpr (WIN) {
        g = wp[reinterpret_cast<const uint16_t *>(scs)[q]];
      } else {
        const int c = (int)scs[q];
        g = make_float2(__ldg(x + c), DX ? __ldg(dy + c) : 0.f);
      }
      if constexpr (DX) acc = fmaf(__uint_as_float(svs[q]), g.y, acc);
      const float gv = (int)(u * S + st) < el ? dyr * g.x : 0.f;
      if constexpr (CSR)
        cs.stg[lane][(u * S + st) % ADJ_CSR_STAGED] = gv;
      else
        __stcs(dp + st * WS, gv);
    };
    if (u < full) {  // a full unit: no guards, so the tile reads can be batched
#pragma unroll
      for (int st = 0; st < S; st++) step(st);
      if constexpr (CSR)
        if (((u + 1) * S) % ADJ_CSR_STAGED == 0)
          flush_csr_chunk32(dvals, cs.stg, cs.skb, cs.sel, (u + 1) * S - ADJ_CSR_STAGED, ADJ_CSR_STAGED, lane);
    } else {
      for (int st = 0; st < (int)rem; st++) step(st);
    }
    __syncwarp();  // this tile is refilled STAGES - 1 units later
  }
  cp_async_wait<0>();
  if constexpr (CSR) {  // the last, partial chunk
    const uint32_t c0 = A / ADJ_CSR_STAGED * ADJ_CSR_STAGED;
    if (A > c0) flush_csr_chunk32(dvals, cs.stg, cs.skb, cs.sel, c0, A - c0, lane);
  }
  return acc;
}

// STAGES tiles in the ring, BLOCKS blocks per SM.  ALLWIN: every warp has
// an x window, so the column tiles hold 16-bit positions only.  DX = false:
// dvals alone (any pattern: no mirror values, dx untouched).
template <int STAGES, int BLOCKS, bool ALLWIN, bool DX = true>
__global__ void __launch_bounds__(ADJ_SW * 32, BLOCKS) k_adjoint_sym_staged(
    const int4 *__restrict__ desc, uint32_t W, const int32_t *__restrict__ row_map, const uint32_t *__restrict__ slen,
    uint32_t nzr, uint32_t nrows, const int32_t *__restrict__ pc, const uint16_t *__restrict__ w16,
    const int2 *__restrict__ wch, const int4 *__restrict__ wdesc, const float *__restrict__ tv,
    const float *__restrict__ x, const float *__restrict__ dy, float *__restrict__ dx, float *__restrict__ dvals) {
  using namespace core;
  constexpr int S = 8;
  constexpr int NCW = ALLWIN ? S / 2 : S;  // column words per lane and unit
  __shared__ __align__(16) uint32_t s_val[ADJ_SW][DX ? STAGES * S * WS : 4];
  __shared__ __align__(16) uint32_t s_col[ADJ_SW][STAGES * NCW * WS];
  __shared__ __align__(16) float2 s_win[ADJ_SW][WIN_MAX];
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x / WS;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w < W) {
    const uint64_t pol = policy_evict_first();
    const int4 d = desc[w], wd = wdesc[w];  // independent loads, in flight together
    int32_t row;
    bool valid;
    float acc = 0.f;
    if (ALLWIN || wd.y != 0) {
      acc = adjoint_warp_pipe<STAGES, true, DX>(d, wd, wch, pc, w16, tv, x, dy, row_map, slen, nzr, s_win[wib],
                                                dvals, s_val[wib], s_col[wib], lane, pol, row, valid);
    } else {
      if constexpr (!ALLWIN)
        acc = adjoint_warp_pipe<STAGES, false, DX>(d, wd, wch, pc, w16, tv, x, dy, row_map, slen, nzr, nullptr,
                                                   dvals, s_val[wib], s_col[wib], lane, pol, row, valid);
    }
    if constexpr (DX) {
      const uint32_t T_ = (uint32_t)d.z;
      for (uint32_t k = 1; k < T_; k <<= 1) acc += __shfl_down_sync(0xffffffffu, acc, k);
      if (valid && (lane & (T_ - 1)) == 0) dx[row] = acc;
    }
  }
  if constexpr (DX)
    for (size_t q = (size_t)nzr + (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nrows;
         q += (size_t)gridDim.x * blockDim.x)
      dx[row_map[q]] = 0.f;
}

// The fused adjoint with dvals in CSR order: the staged kernel's pipe with
// each warp's 32-step chunks of gradients staged as [layout lane][step] and
// written row segment by row segment.  Shared memory per warp (dynamic):
// STAGES value and column tiles, the x window, the staging and the lanes'
// CSR offsets and entry counts.
template <int STAGES, bool ALLWIN>
struct AdjCsrCfg {
  static constexpr int S = 8, NCW = ALLWIN ? S / 2 : S;
  static constexpr int V_WORDS = STAGES * S * WS, C_WORDS = STAGES * NCW * WS, WIN_WORDS = WIN_MAX * 2;
  static constexpr int STG_WORDS = (32 * (ADJ_CSR_STAGED + 1) + 3) / 4 * 4;
  static constexpr int WARP_WORDS = V_WORDS + C_WORDS + WIN_WORDS + STG_WORDS + 64;
  static constexpr size_t SMEM = (size_t)ADJ_SW * WARP_WORDS * 4;
};

template <int STAGES, bool ALLWIN>
__global__ void __launch_bounds__(ADJ_SW * 32) k_adjoint_sym_staged_csr(
    const int4 *__restrict__ desc, uint32_t W, const int32_t *__restrict__ row_map, const uint32_t *__restrict__ slen,
    const int32_t *__restrict__ rowptr, uint32_t nzr, uint32_t nrows, const int32_t *__restrict__ pc,
    const uint16_t *__restrict__ w16, const int2 *__restrict__ wch, const int4 *__restrict__ wdesc,
    const float *__restrict__ tv, const float *__restrict__ x, const float *__restrict__ dy, float *__restrict__ dx,
    float *__restrict__ dvals) {
  using namespace core;
  using C = AdjCsrCfg<STAGES, ALLWIN>;
  extern __shared__ __align__(16) uint32_t adj_csr_smem[];
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x / WS;
  uint32_t *base = adj_csr_smem + wib * C::WARP_WORDS;
  uint32_t *sv = base, *sc = base + C::V_WORDS;
  float2 *wp = reinterpret_cast<float2 *>(sc + C::C_WORDS);
  float(*stg)[ADJ_CSR_STAGED + 1] = reinterpret_cast<float(*)[ADJ_CSR_STAGED + 1]>(sc + C::C_WORDS + C::WIN_WORDS);
  int *skb = reinterpret_cast<int *>(sc + C::C_WORDS + C::WIN_WORDS + C::STG_WORDS);
  const CsrStage cs{stg, skb, skb + 32, rowptr};
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w < W) {
    const uint64_t pol = policy_evict_first();
    const int4 d = desc[w], wd = wdesc[w];
    int32_t row;
    bool valid;
    float acc = 0.f;
    if (ALLWIN || wd.y != 0) {
      acc = adjoint_warp_pipe<STAGES, true, true, true>(d, wd, wch, pc, w16, tv, x, dy, row_map, slen, nzr, wp,
                                                        dvals, sv, sc, lane, pol, row, valid, cs);
    } else {
      if constexpr (!ALLWIN)
        acc = adjoint_warp_pipe<STAGES, false, true, true>(d, wd, wch, pc, w16, tv, x, dy, row_map, slen, nzr,
                                                           nullptr, dvals, sv, sc, lane, pol, row, valid, cs);
    }
    const uint32_t T_ = (uint32_t)d.z;
    for (uint32_t k = 1; k < T_; k <<= 1) acc += __shfl_down_sync(0xffffffffu, acc, k);
    if (valid && (lane & (T_ - 1)) == 0) dx[row] = acc;
  }
  for (size_t q = (size_t)nzr + (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nrows;
       q += (size_t)gridDim.x * blockDim.x)
    dx[row_map[q]] = 0.f;
}

wk_status refresh_transposed(wk_adjoint *a, const void *vals_csr, cudaStream_t st) {
  const wk_engine *f = a->fwd;
  const uint32_t nz = f->layout->info.nz;
  const size_t eb = dtype_size(f->dtype);
  const void *src = vals_csr;
  if (!src) {  // from the forward engine's padded values
    if (eb == 8)
      k_gather_padded<unsigned long long><<<grid_for(nz, 256), 256, 0, st>>>(
          f->vals.as<unsigned long long>(), f->layout->d.reorder_rows, nz, a->tmp.as<unsigned long long>());
    else
      k_gather_padded<uint32_t><<<grid_for(nz, 256), 256, 0, st>>>(f->vals.as<uint32_t>(), f->layout->d.reorder_rows,
                                                                   nz, a->tmp.as<uint32_t>());
    WK_CHECK_LAUNCH();
    src = a->tmp.p;
  }
  // tmp2 = vals[perm]: reuse the transposed engine's scratch as the CSR-order staging
  DevBuf stage;
  WK_TRY(stage.alloc((size_t)nz * eb));
  if (eb == 8)
    k_permute<unsigned long long><<<grid_for(nz, 256), 256, 0, st>>>((const unsigned long long *)src,
                                                                     a->perm.as<uint32_t>(), nz,
                                                                     stage.as<unsigned long long>());
  else
    k_permute<uint32_t><<<grid_for(nz, 256), 256, 0, st>>>((const uint32_t *)src, a->perm.as<uint32_t>(), nz,
                                                           stage.as<uint32_t>());
  WK_CHECK_LAUNCH();
  WK_TRY(launch_process(a->tl, stage.p, (int)eb, nullptr, a->te->vals.p, nullptr, false, st));
  WK_CUDA(cudaStreamSynchronize(st));
  return WK_OK;
}

}  // namespace
}  // namespace wk

using namespace wk;

extern "C" wk_status wk_adjoint_create(wk_engine *fwd, int kind, int32_t threshold, void *stream, wk_adjoint **out) {
  if (!out) return set_error(WK_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!fwd) return set_error(WK_ERR_INVALID, "engine is NULL");
  WK_TRY(require_interleaved(fwd->layout, "wk_adjoint_create"));
  if (fwd->dtype != WK_F64 && fwd->dtype != WK_F32)
    return set_error(WK_ERR_INVALID, "the adjoint supports WK_F64 and WK_F32 engines");
  if (kind != WK_WPK1 && kind != WK_WPK2) return set_error(WK_ERR_INVALID, "kind must be WK_WPK1 or WK_WPK2");
  cudaStream_t st = (cudaStream_t)stream;
  const wk_layout *L = fwd->layout;
  const uint32_t n = L->info.nrows, m = fwd->ncols, nz = L->info.nz;
  if (m > 0x7fffffffu) return set_error(WK_ERR_INVALID, "ncols too large");
  const size_t eb = dtype_size(fwd->dtype);
  wk_adjoint *a = new (std::nothrow) wk_adjoint();
  if (!a) return set_error(WK_ERR_ALLOC, "host allocation failed");
  a->fwd = fwd;
  a->kind = kind;
  a->threshold = threshold;
  auto fail = [&](wk_status s) {
    if (a->te) wk_engine_destroy(a->te);
    if (a->tl) wk_layout_destroy(a->tl);
    delete a;
    return s;
  };
  DevBuf k0, k1, v0, v1, counts, rowptrT, valsc, colsT, rowof, diff, csrcols;
  wk_status s = WK_OK;
  if (s == WK_OK) s = k0.alloc((size_t)nz * 4);
  if (s == WK_OK) s = k1.alloc((size_t)nz * 4);
  if (s == WK_OK) s = v0.alloc((size_t)nz * 4);
  if (s == WK_OK) s = v1.alloc((size_t)nz * 4);
  if (s == WK_OK) s = csrcols.alloc((size_t)nz * 4);
  if (s == WK_OK) s = counts.alloc(((size_t)m + 1) * 4);
  if (s == WK_OK) s = rowptrT.alloc(((size_t)m + 1) * 4);
  if (s == WK_OK) s = a->tmp.alloc((size_t)nz * eb);
  if (s == WK_OK) s = colsT.alloc((size_t)nz * 4);
  if (s == WK_OK) s = rowof.alloc((size_t)nz * 4);
  if (s == WK_OK) s = diff.alloc(16);
  if (s != WK_OK) return fail(s);
  // CSR columns of A, then a stable sort by column: perm and A^T's columns
  k_csr_cols<<<grid_for(nz, 256), 256, 0, st>>>(fwd->cols.as<int32_t>(), L->d.reorder_rows, nz, k0.as<uint32_t>(),
                                                v0.as<uint32_t>());
  if (cudaMemcpyAsync(csrcols.p, k0.p, (size_t)nz * 4, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return fail(set_error(WK_ERR_CUDA, "copy failed"));
  if (cudaMemsetAsync(counts.p, 0, ((size_t)m + 1) * 4, st) != cudaSuccess)
    return fail(set_error(WK_ERR_CUDA, "memset failed"));
  k_count<<<grid_for(nz, 256), 256, 0, st>>>(k0.as<uint32_t>(), nz, counts.as<uint32_t>());
  if (cudaGetLastError() != cudaSuccess) return fail(set_error(WK_ERR_CUDA, "kernel launch failed"));
  s = scan_u32(counts.as<uint32_t>(), rowptrT.as<uint32_t>(), (size_t)m + 1, nullptr, st);
  if (s != WK_OK) return fail(s);
  int bits = 0;
  while (bits < 32 && (((uint64_t)m > 0 ? (uint64_t)m - 1 : 0) >> bits)) bits++;
  int cur = 0;
  s = radix_sort_pairs(k0.as<uint32_t>(), k1.as<uint32_t>(), v0.as<uint32_t>(), v1.as<uint32_t>(), nz, bits, st, &cur);
  if (s != WK_OK) return fail(s);
  s = a->perm.alloc((size_t)nz * 4);
  if (s != WK_OK) return fail(s);
  const uint32_t *perm = cur ? v1.as<uint32_t>() : v0.as<uint32_t>();
  if (cudaMemcpyAsync(a->perm.p, perm, (size_t)nz * 4, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return fail(set_error(WK_ERR_CUDA, "copy failed"));
  k_row_of<<<grid_for(n, 256), 256, 0, st>>>(L->d.rowptr, n, rowof.as<uint32_t>());
  k_permute<uint32_t><<<grid_for(nz, 256), 256, 0, st>>>(rowof.as<uint32_t>(), a->perm.as<uint32_t>(), nz,
                                                         colsT.as<uint32_t>());
  if (cudaGetLastError() != cudaSuccess) return fail(set_error(WK_ERR_CUDA, "kernel launch failed"));
  // A^T's layout and engine (values in A^T's CSR order = A's values permuted)
  // a WPK1 adjoint keeps the forward layout's row order (sorted or CSR order)
  s = make_layout(rowptrT.as<int32_t>(), m, nz, kind, threshold, st, &a->tl,
                  kind == WK_WPK1 ? (int)L->info.variant : 0);
  if (s != WK_OK) return fail(s);
  if (eb == 8)
    k_gather_padded<unsigned long long><<<grid_for(nz, 256), 256, 0, st>>>(
        fwd->vals.as<unsigned long long>(), L->d.reorder_rows, nz, a->tmp.as<unsigned long long>());
  else
    k_gather_padded<uint32_t><<<grid_for(nz, 256), 256, 0, st>>>(fwd->vals.as<uint32_t>(), L->d.reorder_rows, nz,
                                                                 a->tmp.as<uint32_t>());
  s = valsc.alloc((size_t)nz * eb);
  if (s != WK_OK) return fail(s);
  if (eb == 8)
    k_permute<unsigned long long><<<grid_for(nz, 256), 256, 0, st>>>(a->tmp.as<unsigned long long>(),
                                                                     a->perm.as<uint32_t>(), nz,
                                                                     valsc.as<unsigned long long>());
  else
    k_permute<uint32_t><<<grid_for(nz, 256), 256, 0, st>>>(a->tmp.as<uint32_t>(), a->perm.as<uint32_t>(), nz,
                                                           valsc.as<uint32_t>());
  s = make_engine(a->tl, fwd->dtype, valsc.p, colsT.as<int32_t>(), n, st, &a->te);
  if (s != WK_OK) return fail(s);
  // structurally symmetric with sorted rows: same row offsets and columns
  if (m == n && kind == L->info.kind && a->tl->info.variant == L->info.variant &&
      (kind == WK_WPK1 || (uint32_t)threshold == L->info.nmax_per_thread)) {
    if (cudaMemsetAsync(diff.p, 0, 4, st) != cudaSuccess) return fail(set_error(WK_ERR_CUDA, "memset failed"));
    k_count_diff<<<grid_for((size_t)n + 1, 256), 256, 0, st>>>(rowptrT.as<uint32_t>(), (const uint32_t *)L->d.rowptr,
                                                               (size_t)n + 1, diff.as<unsigned>());
    k_count_diff<<<grid_for(nz, 256), 256, 0, st>>>(colsT.as<uint32_t>(), csrcols.as<uint32_t>(), nz,
                                                    diff.as<unsigned>());
    unsigned h = 1;
    if (cudaMemcpyAsync(&h, diff.p, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return fail(set_error(WK_ERR_CUDA, "symmetry check failed"));
    a->symmetric = h == 0;
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(set_error(WK_ERR_CUDA, "adjoint build failed"));
  *out = a;
  return WK_OK;
}

extern "C" wk_status wk_adjoint_refresh(wk_adjoint *a, const void *vals_csr, void *stream) {
  if (!a) return set_error(WK_ERR_INVALID, "adjoint is NULL");
  cudaStream_t st = (cudaStream_t)stream;
  if (vals_csr) {
    WK_TRY(wk_engine_set_values(a->fwd, vals_csr, stream));
    DevView v;
    WK_TRY(v.from(vals_csr, (size_t)a->fwd->layout->info.nz * dtype_size(a->fwd->dtype), st));
    return refresh_transposed(a, v.dptr, st);
  }
  return refresh_transposed(a, nullptr, st);
}

extern "C" wk_status wk_adjoint_run(wk_adjoint *a, const void *x, const void *dy, void *dx, void *dvals,
                                   int dvals_order, void *stream) {
  if (!a || !dy) return set_error(WK_ERR_INVALID, "NULL argument");
  if (dvals && !x) return set_error(WK_ERR_INVALID, "dvals needs x");
  if (dvals_order != WK_DVALS_CSR && dvals_order != WK_DVALS_SLOTS)
    return set_error(WK_ERR_INVALID, "unknown dvals order %d", dvals_order);
  cudaStream_t st = (cudaStream_t)stream;
  const wk_engine *f = a->fwd;
  const wk_layout *L = f->layout;
  const uint32_t W = L->info.nwarps, n = L->info.nrows;
  const bool f64 = f->dtype == WK_F64;
  const bool slots = dvals_order == WK_DVALS_SLOTS;
  if (a->symmetric && dx && dvals) {
    const size_t pb = (size_t)n * (f64 ? 16 : 8);
    if (slots && ((uintptr_t)dvals & 31u))
      return set_error(WK_ERR_INVALID, "slot-order dvals must be 32-byte aligned");
    const unsigned gi = grid_for(n, 256);
    // fp32 gradient in slot order: the staged kernel, with the x windows of
    // the forward layout's int32 columns (built on the first such call; the
    // forward engine's own 16-bit columns, if any, are not used here)
    if (!f64 && slots) {
      if (!a->win_built) {
        WK_TRY(build_window_set(L, f->cols.as<int32_t>(), a->win, st));
        a->win_built = true;
      }
      const unsigned g = (unsigned)std::max<size_t>(1, ((size_t)W + ADJ_SW - 1) / ADJ_SW);
#define WK_ADJ_ST(ST, BL, AW)                                                                                      \
  k_adjoint_sym_staged<ST, BL, AW><<<g, ADJ_SW * 32, 0, st>>>(                                                     \
      L->d.warp_desc, W, L->d.row_map, L->d.slen, L->info.nznrows, n, f->cols.as<int32_t>(),                      \
      a->win.w16.as<uint16_t>(), a->win.chunks.as<int2>(), a->win.wdesc.as<int4>(), a->te->vals.as<float>(),      \
      (const float *)x, (const float *)dy, (float *)dx, (float *)dvals)
      if (a->win.warps == W)
        WK_ADJ_ST(4, 5, true);  // 16-bit positions only: 40 KB per block
      else
        WK_ADJ_ST(4, 4, false);
#undef WK_ADJ_ST
      WK_CHECK_LAUNCH();
      return WK_OK;
    }
    // fp32 gradient in CSR order: the same pipe, gradients staged per warp
    // and written row segment by row segment; two stages leave four blocks
    // per SM (hex 64^3: 0.1584 ms, three stages 0.1582, k_adjoint_sym_slots
    // 0.207)
    if (!f64) {
      if (!a->win_built) {
        WK_TRY(build_window_set(L, f->cols.as<int32_t>(), a->win, st));
        a->win_built = true;
      }
      const unsigned g = (unsigned)std::max<size_t>(1, ((size_t)W + ADJ_SW - 1) / ADJ_SW);
#define WK_ADJ_CSR(ST, AW)                                                                                         \
  do {                                                                                                             \
    const size_t sm = AdjCsrCfg<ST, AW>::SMEM;                                                                     \
    WK_CUDA(cudaFuncSetAttribute(k_adjoint_sym_staged_csr<ST, AW>, cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                                 (int)sm));                                                                        \
    k_adjoint_sym_staged_csr<ST, AW><<<g, ADJ_SW * 32, sm, st>>>(                                                  \
        L->d.warp_desc, W, L->d.row_map, L->d.slen, L->d.rowptr, L->info.nznrows, n, f->cols.as<int32_t>(),        \
        a->win.w16.as<uint16_t>(), a->win.chunks.as<int2>(), a->win.wdesc.as<int4>(), a->te->vals.as<float>(),    \
        (const float *)x, (const float *)dy, (float *)dx, (float *)dvals);                                         \
  } while (0)
      if (a->win.warps == W)
        WK_ADJ_CSR(2, true);
      else
        WK_ADJ_CSR(2, false);
#undef WK_ADJ_CSR
      WK_CHECK_LAUNCH();
      return WK_OK;
    }
    if (a->xdy.bytes < pb) WK_TRY(a->xdy.alloc(pb));
#define WK_ADJ_SLOTS1(T, COMP, CSR)                                                                                 \
  k_adjoint_sym_slots<T, COMP, CSR><<<(unsigned)std::max<size_t>(1, ((size_t)W + AdjCfg<T, CSR>::warps - 1) /      \
                                                          AdjCfg<T, CSR>::warps),                                  \
                                      AdjCfg<T, CSR>::warps * 32, 0, st>>>(                                        \
      L->d.warp_desc, W, L->d.row_map, L->d.slen, L->d.rowptr, L->info.nznrows, n, f->cols.as<int32_t>(),           \
      f->c16.as<uint16_t>(), f->c32.as<int32_t>(), f->cdesc.as<int4>(), a->te->vals.as<T>(),                        \
      a->xdy.as<typename Pair<T>::type>(), (T *)dx, (T *)dvals)
#define WK_ADJ_SLOTS(T)                                                                                             \
  do {                                                                                                              \
    if (f->compressed) {                                                                                            \
      if (slots) WK_ADJ_SLOTS1(T, true, false); else WK_ADJ_SLOTS1(T, true, true);                                  \
    } else {                                                                                                        \
      if (slots) WK_ADJ_SLOTS1(T, false, false); else WK_ADJ_SLOTS1(T, false, true);                                \
    }                                                                                                               \
  } while (0)
    if (f64) {
      k_interleave<double><<<gi, 256, 0, st>>>((const double *)x, (const double *)dy, n, a->xdy.as<double2>());
      WK_ADJ_SLOTS(double);
    } else {
      k_interleave<float><<<gi, 256, 0, st>>>((const float *)x, (const float *)dy, n, a->xdy.as<float2>());
      WK_ADJ_SLOTS(float);
    }
#undef WK_ADJ_SLOTS1
#undef WK_ADJ_SLOTS
    WK_CHECK_LAUNCH();
    return WK_OK;
  }
  if (dx) {
    const size_t yb = (size_t)a->te->layout->info.nrows * dtype_size(f->dtype);
    if (a->te->layout->info.nznrows < a->te->layout->info.nrows) WK_CUDA(cudaMemsetAsync(dx, 0, yb, st));
    RunArgs ra{a->te, 0, 0, 1, WK_ORDER_FAST, true, dy, dx, st};
    WK_TRY(launch_spmv(ra));
  }
  if (dvals && W && !f64 && slots) {
    // fp32 gradient in slot order: the staged kernel without mirror values or
    // dx, gathering x from the layout warps' windows
    if (!a->win_built) {
      WK_TRY(build_window_set(L, f->cols.as<int32_t>(), a->win, st));
      a->win_built = true;
    }
    const unsigned g = (unsigned)std::max<size_t>(1, ((size_t)W + ADJ_SW - 1) / ADJ_SW);
#define WK_ADJ_DV(AW)                                                                                              \
  k_adjoint_sym_staged<4, 6, AW, false><<<g, ADJ_SW * 32, 0, st>>>(                                                \
      L->d.warp_desc, W, L->d.row_map, L->d.slen, L->info.nznrows, n, f->cols.as<int32_t>(),                      \
      a->win.w16.as<uint16_t>(), a->win.chunks.as<int2>(), a->win.wdesc.as<int4>(), nullptr, (const float *)x,    \
      (const float *)dy, nullptr, (float *)dvals)
    if (a->win.warps == W)
      WK_ADJ_DV(true);
    else
      WK_ADJ_DV(false);
#undef WK_ADJ_DV
    WK_CHECK_LAUNCH();
  } else if (dvals && W) {
    const unsigned g = (unsigned)std::max<size_t>(1, ((size_t)W * WS + 255) / 256);
#define WK_DV(T)                                                                                                       \
  do {                                                                                                                 \
    if (slots)                                                                                                         \
      k_dvals_slots<T><<<g, 256, 0, st>>>(L->d.warp_desc, W, L->d.row_map, L->d.slen, L->info.nznrows,               \
                                          f->cols.as<int32_t>(), (const T *)x, (const T *)dy, (T *)dvals);             \
    else                                                                                                               \
      k_dvals_csr<T><<<g, 256, 0, st>>>(L->d.warp_desc, W, L->d.row_map, L->d.slen, L->d.rowptr, L->info.nznrows,    \
                                        f->cols.as<int32_t>(), (const T *)x, (const T *)dy, (T *)dvals);               \
  } while (0)
    if (f64)
      WK_DV(double);
    else
      WK_DV(float);
#undef WK_DV
    WK_CHECK_LAUNCH();
  }
  return WK_OK;
}

// Values in slot order (allocate_nz, padding ignored): copied into the forward
// engine, then A^T's values are re-derived from it.
extern "C" wk_status wk_adjoint_refresh_slots(wk_adjoint *a, const void *vals_slots, void *stream) {
  if (!a || !vals_slots) return set_error(WK_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = (size_t)a->fwd->layout->info.allocate_nz * dtype_size(a->fwd->dtype);
  if (bytes) WK_CUDA(cudaMemcpyAsync(a->fwd->vals.p, vals_slots, bytes, cudaMemcpyDefault, st));
  return refresh_transposed(a, nullptr, st);
}

extern "C" wk_status wk_adjoint_info(const wk_adjoint *a, int *symmetric, wk_layout_info *tinfo) {
  if (!a) return set_error(WK_ERR_INVALID, "adjoint is NULL");
  if (symmetric) *symmetric = a->symmetric ? 1 : 0;
  if (tinfo) *tinfo = a->tl->info;
  return WK_OK;
}

extern "C" wk_status wk_adjoint_transposed_layout(const wk_adjoint *a, wk_layout **tl) {
  if (!a || !tl) return set_error(WK_ERR_INVALID, "NULL argument");
  a->tl->refs.fetch_add(1);
  *tl = a->tl;
  return WK_OK;
}

extern "C" wk_status wk_adjoint_destroy(wk_adjoint *a) {
  if (!a) return WK_OK;
  if (a->te) wk_engine_destroy(a->te);
  if (a->tl) wk_layout_destroy(a->tl);
  delete a;
  return WK_OK;
}
