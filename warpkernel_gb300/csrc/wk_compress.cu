// wk_compress.cu -- 16-bit column storage for the mixed-precision paths.
//
// With fp32 values a stored slot costs 4 B of value + 4 B of column, so the
// column index is half of the traffic.  Finite-element rows of one layout
// warp (32 consecutive sorted rows, i.e. nearby nodes) reference a narrow
// band of columns; when a warp's real entries span fewer than 65,536 columns
// its indices are stored as uint16 offsets from a per-warp base.  Warps with
// a wider span keep int32 indices in a compact side array.  Padding slots
// store offset 0 (their value is 0).
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

unsigned grid_for_warps(uint32_t W) {
  size_t g = ((size_t)W * WS + 255) / 256;
  if (g < 1) g = 1;
  if (g > 152u * 64u) g = 152u * 64u;
  return (unsigned)g;
}

}  // namespace

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
  WK_CUDA(cudaStreamSynchronize(st));
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

extern "C" wk_status wk_engine_compress_cols(wk_engine *e, void *stream, uint32_t *wide_warps) {
  if (!e) return set_error(WK_ERR_INVALID, "engine is NULL");
  WK_TRY(require_interleaved(e->layout, "wk_engine_compress_cols"));
  return build_compressed_cols(e, (cudaStream_t)stream, wide_warps);
}
