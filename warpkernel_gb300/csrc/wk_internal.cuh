// wk_internal.cuh -- shared definitions of libwarpkernel_gb300 (not installed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/wk_capi.h"

namespace wk {

// x windows (wk_compress.cu): at most WIN_MAX distinct columns in at most
// WIN_CHUNKS chunks of <= 32 consecutive columns per layout warp.
constexpr int WIN_MAX = 512;
constexpr int WIN_CHUNKS = 32;

// ---- errors ------------------------------------------------------------------
wk_status set_error(wk_status code, const char *fmt, ...);
const std::string &last_error();

#define WK_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return ::wk::set_error(e_ == cudaErrorMemoryAllocation ? WK_ERR_ALLOC : WK_ERR_CUDA, \
                             "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                             __FILE__, __LINE__);                                  \
  } while (0)

#define WK_TRY(call)                  \
  do {                                \
    wk_status s_ = (call);            \
    if (s_ != WK_OK) return s_;       \
  } while (0)

#define WK_CHECK_LAUNCH() WK_CUDA(cudaGetLastError())

// ---- device memory -------------------------------------------------------------
// Fault injection for the error paths: when positive, the countdown is
// decremented by every device allocation and the one that brings it to zero
// fails with WK_ERR_ALLOC instead of calling cudaMalloc (wk_debug_fail_alloc).
extern std::atomic<int> g_alloc_fail_countdown;

// Owning device buffer (cudaMalloc / cudaFree).
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) { release(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  wk_status alloc(size_t n) {
    release();
    if (n == 0) n = 16;  // keep a valid pointer for empty arrays
    if (g_alloc_fail_countdown.load() > 0 && g_alloc_fail_countdown.fetch_sub(1) == 1)
      return set_error(WK_ERR_ALLOC, "injected allocation failure (%zu bytes)", n);
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();
      return set_error(e == cudaErrorMemoryAllocation ? WK_ERR_ALLOC : WK_ERR_CUDA,
                       "cudaMalloc(%zu bytes) failed: %s", n, cudaGetErrorString(e));
    }
    bytes = n;
    return WK_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T *as() const { return static_cast<T *>(p); }
};

// true if `ptr` is device (or managed) memory usable by kernels.
bool is_device_ptr(const void *ptr);

// A device view of a caller array: uses it in place if it is device memory,
// otherwise uploads `bytes` into a temporary buffer on `stream`.
struct DevView {
  const void *dptr = nullptr;
  DevBuf tmp;
  wk_status from(const void *src, size_t bytes, cudaStream_t stream);
};

// Copies `bytes` from device `src` to caller memory `dst` (host or device).
wk_status copy_out(void *dst, const void *src, size_t bytes, cudaStream_t stream);

// Bytes per element of the values a caller passes and of x (WK_F16S: FP32).
size_t dtype_size(int dtype);
// Bytes per stored padded value (WK_F16S: 2).
size_t stored_size(int dtype);

// ---- handles ---------------------------------------------------------------------
struct LayoutDev {
  // Reference fields (bit-identical to warpkernel.hpp's host scan).
  int32_t *row_map = nullptr;          // [nrows]
  int32_t *row_map_inv = nullptr;      // [nrows]
  uint32_t *reorder_rows = nullptr;    // [nz]
  int32_t *warp_offsets = nullptr;     // [nwarps+1]
  uint32_t *max_nz_rows = nullptr;     // [nwarps]
  uint32_t *threads_per_row = nullptr; // [nwarps]   (WPK2)
  uint32_t *row_offset_warp = nullptr; // [nwarps+1] (WPK2)
  // Working arrays of this implementation.
  int32_t *rowptr = nullptr;           // [nrows+1] device copy of the CSR row offsets
  uint32_t *slen = nullptr;            // [nrows]   row length in sorted order
  int4 *warp_desc = nullptr;           // [nwarps]  {offset, steps, threads_per_row, first row}
};

}  // namespace wk

struct wk_layout {
  std::atomic<int> refs{1};
  int device = 0;
  wk_layout_info info{};
  wk::LayoutDev d;
  wk::DevBuf bufs[10];
  // Slot-weighted mean of the warps' step counts (sum A_w^2 / sum A_w): the
  // fast order runs the one-slot-per-step kernel when it is small.
  double mean_steps = 0.0;
  double sum_steps = 0.0, max_steps = 0.0;  // sum and max of A_w over the warps
};

struct wk_engine {
  wk_layout *layout = nullptr;
  int dtype = WK_F64;
  uint32_t ncols = 0;
  wk::DevBuf vals;   // allocate_nz values (padding 0)
  wk::DevBuf cols;   // allocate_nz int32 column indices (padding 0)
  wk::DevBuf status; // device status word for kernels that can report errors
  wk::DevBuf xbuf, ybuf;  // staging vectors of wk_run_host (allocated on first use)
  wk::DevBuf xbuf2, ybuf2;  // second staging pair of wk_run_host_stream (double buffering)
  wk::DevBuf scratch;     // per-block partial sums of the solver kernels (grown on demand)
  // compressed columns (wk_engine_compress_cols): 16-bit offsets per slot,
  // compact 32-bit indices of the warps whose span needs them, per-warp descriptor
  bool compressed = false;
  wk::DevBuf c16, c32, cdesc;
  // x windows of the narrow warps (built with the compact columns): per slot
  // the window position of its column, the chunks of each window, and per
  // warp {first chunk, chunks (0: no window), window size, 0}
  wk::DevBuf w16, wchunks, wdesc;
  uint32_t window_warps = 0;
  bool windows_built = false;
  bool use_windows = false;  // wk_engine_set_windows; wk_engine_create turns it on for FP32 and scaled FP16
  wk::DevBuf scale;  // WK_F16S: float power-of-two scale per layout warp
  // device address of wk_residual_static's static scratch array, looked up
  // on the engine's first wk_residual_static call (an engine lives in one
  // context, so the address stays valid for the engine's lifetime)
  double *static_partials = nullptr;
};

namespace wk {

// ---- launchers (stream-ordered) ----------------------------------------------------
// Builds all layout arrays from a device CSR row-pointer array (kind 1/2).
wk_status build_layout(wk_layout *l, const int32_t *d_rowptr, int kind, int32_t threshold,
                       cudaStream_t stream, int variant = 0);
// Padded gather of values (elem bytes 8/4/2) and column indices; cols are
// optionally renumbered through row_map_inv.  Either output may be null.
wk_status launch_process(const wk_layout *l, const void *vals, int elem_bytes,
                         const int32_t *cols, void *pvals, int32_t *pcols, bool renumber,
                         cudaStream_t stream);
wk_status launch_reorder_columns(const wk_layout *l, const int32_t *cols, int32_t *out,
                                 cudaStream_t stream);
wk_status launch_reorder_x(const wk_layout *l, const void *x, void *xout, int elem_bytes,
                           cudaStream_t stream);
// Counts column indices outside [0, ncols) into *d_bad (device int).
wk_status launch_check_cols(const int32_t *cols, size_t n, uint32_t ncols, int *d_bad,
                            cudaStream_t stream);

// Exclusive scan of n uint64 values (out may alias in); *d_total = the sum.
// Synchronises `stream`.
wk_status scan_u64(const unsigned long long *in, unsigned long long *out, size_t n,
                   unsigned long long *d_total, cudaStream_t stream);
wk_status scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *d_total, cudaStream_t stream);
// Stable LSD radix sort of n (key, value) pairs by the low `bits` key bits;
// input in buffers 0, *out = which buffer pair holds the result.
wk_status radix_sort_pairs(uint32_t *k0, uint32_t *k1, uint32_t *v0, uint32_t *v1, uint32_t n, int bits,
                           cudaStream_t stream, int *out);
// Allocates a layout and builds it on the device from a device copy of the
// CSR row offsets (the layout keeps its own copy).
wk_status make_layout(const int32_t *d_rowptr, uint32_t nrows, uint32_t nz, int kind, int32_t threshold,
                      cudaStream_t stream, wk_layout **out, int variant = 0);
// WK_ERR_INVALID for layouts whose slots are not interleaved (WK_ABL_NOCOALESCE),
// which only the plain SpMV and data-movement calls accept; `op` names the call.
wk_status require_interleaved(const wk_layout *l, const char *op);
// Allocates an engine over layout l (takes a layout reference) from device
// CSR-ordered values (elem bytes 8/4/2) and column indices.
wk_status make_engine(wk_layout *l, int dtype, const void *d_vals, const int32_t *d_cols, uint32_t ncols,
                      cudaStream_t stream, wk_engine **out);
// Places CSR-ordered device values (the engine's input type) into the padded
// value array; WK_F16S values are scaled per warp and rounded to FP16.
wk_status load_values(wk_engine *e, const void *d_vals, cudaStream_t stream);
// WK_F16S: decodes the padded values to FP32 (allocate_nz floats, device).
wk_status launch_f16s_decode(const wk_engine *e, float *out, cudaStream_t stream);
// x windows of a layout over padded device columns, owned by the caller
// (the adjoint's): per-warp modes / bases, slot window positions, chunks and
// window descriptors (see wk_compress.cu).
struct WinSet {
  DevBuf cdesc, w16, chunks, wdesc;
  uint32_t warps = 0;
};
wk_status build_window_set(const wk_layout *l, const int32_t *cols, WinSet &ws, cudaStream_t stream);
// Builds / refreshes the engine's 16-bit column storage from its int32 columns.
wk_status build_compressed_cols(wk_engine *e, cudaStream_t stream, uint32_t *wide_warps);

// fp64 residual r = b - A x with block partials of ||r||^2 (wk_solve.cu);
// norm2 (device, optional) receives their fixed-order sum.
unsigned residual_grid(const wk_layout *l);
wk_status launch_residual(const wk_engine *e, const double *x, const double *b, double *r, double *partials,
                          unsigned grid, double *norm2, cudaStream_t stream);

struct RunArgs {
  const wk_engine *e;
  int nblocks, blocksize, cache, order;
  bool mapped;
  const void *x;
  void *y;
  cudaStream_t stream;
};
wk_status launch_spmv(const RunArgs &a);
// True if the layout's warps are short for `dtype`: the one-slot-per-step
// loop then beats the vector path.  Crossovers of the slot-weighted mean step
// count measured on hex meshes (1-3 dof, WPK2 thresholds giving 6-81 steps):
// fp64 between 27 and 41 steps (vector / exact time 0.97-1.09 at 27, 0.97 at
// 41), fp32 and bf16 near 21, scaled FP16 near 10.  One value per type keeps
// the 16-bit column form's sums bit-identical to the 32-bit form's.
inline double short_steps(int dtype) {
  switch (dtype) {
    case WK_F64: return 32.0;
    case WK_F32:
    case WK_BF16: return 20.0;
    default: return 16.0;
  }
}
inline bool short_layout(const wk_layout *l, int dtype) { return l->mean_steps < short_steps(dtype); }
// True if the longest warp alone outlasts the rest of the work: its steps
// times the warps the GPU keeps resident (152 SMs x 32) exceed all warps'
// steps together (a WPK1 layout of a power-law matrix: a few hundred warps of
// 2,000 steps).  Each such warp's own loads in flight then set the time.
inline bool long_warps(const wk_layout *l) { return l->max_steps * (152.0 * 32.0) > l->sum_steps; }
// Grid / block of a one-warp-per-layout-warp launch (nblocks/blocksize <= 0: automatic).
wk_status launch_shape(uint32_t W, int nblocks, int blocksize, unsigned *grid, unsigned *block);

wk_status launch_fe_fill(int dim, int ex, int ey, int ez, int dof, int value_mode, uint64_t seed,
                         int32_t *rowptr, int32_t *cols, double *vals, cudaStream_t stream);
wk_status launch_uniform(uint64_t seed, uint64_t stream_id, double *x, int64_t n,
                         cudaStream_t stream);
wk_status launch_convert(const void *src, int sdt, void *dst, int ddt, int64_t n,
                         cudaStream_t stream);

}  // namespace wk
