// wk_f16s.cu -- value storage of WK_F16S engines: FP16 relative to a
// power-of-two scale per layout warp.
//
// A layout warp's values share one scale 2^e chosen from the warp's largest
// finite magnitude m (m = f * 2^k, f in [0.5, 1), e = k - 15), so m / 2^e lies in
// [2^14, 2^15) below FP16's largest finite value and values up to 2^29 times
// smaller stay normal.  Dividing by 2^e is exact; the only rounding is FP16's
// (11-bit significand).  The SpMV kernels sum h * x in FP32 and multiply the
// row total by 2^e, which is exact too (barring FP32 overflow or underflow).
#include <cuda_fp16.h>

#include "wk_internal.cuh"

namespace wk {
namespace {

constexpr int WS = 32;

unsigned warp_grid(uint32_t W) {
  size_t g = ((size_t)W * WS + 255) / 256;
  if (g < 1) g = 1;
  if (g > 152u * 64u) g = 152u * 64u;
  return (unsigned)g;
}

// One warp per layout warp over its 32 * A slots.
__global__ void k_f16s_encode(const int4 *__restrict__ desc, uint32_t W, const float *__restrict__ v32,
                              __half *__restrict__ v16, float *__restrict__ scale) {
  const uint32_t lane = threadIdx.x & 31;
  for (size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS; w < W;
       w += (size_t)gridDim.x * blockDim.x / WS) {
    const int4 d = desc[w];
    const size_t o = (size_t)(uint32_t)d.x, end = o + (size_t)WS * (uint32_t)d.y;
    float m = 0.f;  // largest finite magnitude: inf / nan entries encode as themselves
    for (size_t k = o + lane; k < end; k += WS) {
      const float a = fabsf(v32[k]);
      if (isfinite(a)) m = fmaxf(m, a);
    }
    for (int s = 16; s > 0; s >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, s));
    int e = 0;
    if (m > 0.f && isfinite(m)) {
      frexpf(m, &e);   // m = f * 2^e, f in [0.5, 1)
      e = max(e - 15, -126);  // keep the scale a normal FP32 number
    }
    const float sc = ldexpf(1.f, e), inv = ldexpf(1.f, -e);
    if (lane == 0) scale[w] = sc;
    for (size_t k = o + lane; k < end; k += WS) v16[k] = __float2half_rn(v32[k] * inv);
  }
}

__global__ void k_f16s_decode(const int4 *__restrict__ desc, uint32_t W, const __half *__restrict__ v16,
                              const float *__restrict__ scale, float *__restrict__ out) {
  const uint32_t lane = threadIdx.x & 31;
  for (size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS; w < W;
       w += (size_t)gridDim.x * blockDim.x / WS) {
    const int4 d = desc[w];
    const size_t o = (size_t)(uint32_t)d.x, end = o + (size_t)WS * (uint32_t)d.y;
    const float sc = scale[w];
    for (size_t k = o + lane; k < end; k += WS) out[k] = __half2float(v16[k]) * sc;
  }
}

}  // namespace

wk_status load_values(wk_engine *e, const void *d_vals, cudaStream_t st) {
  const wk_layout *l = e->layout;
  if (e->dtype != WK_F16S)
    return launch_process(l, d_vals, (int)dtype_size(e->dtype), nullptr, e->vals.p, nullptr, false, st);
  const uint32_t W = l->info.nwarps;
  DevBuf tmp;
  WK_TRY(tmp.alloc((size_t)l->info.allocate_nz * 4));
  WK_TRY(launch_process(l, d_vals, 4, nullptr, tmp.p, nullptr, false, st));
  if (W) {
    k_f16s_encode<<<warp_grid(W), 256, 0, st>>>(l->d.warp_desc, W, tmp.as<float>(), e->vals.as<__half>(),
                                                  e->scale.as<float>());
    WK_CHECK_LAUNCH();
  }
  WK_CUDA(cudaStreamSynchronize(st));  // tmp is freed on return
  return WK_OK;
}

wk_status launch_f16s_decode(const wk_engine *e, float *out, cudaStream_t st) {
  const wk_layout *l = e->layout;
  const uint32_t W = l->info.nwarps;
  if (!W) return WK_OK;
  k_f16s_decode<<<warp_grid(W), 256, 0, st>>>(l->d.warp_desc, W, e->vals.as<__half>(), e->scale.as<float>(), out);
  WK_CHECK_LAUNCH();
  return WK_OK;
}

}  // namespace wk
