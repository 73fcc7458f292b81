// wk_capi.cu -- the C ABI (include/wk_capi.h): argument checks, handle
// lifetime, host/device classification of caller pointers, verify.
#include <cmath>
#include <cstring>
#include <vector>

#include "wk_internal.cuh"

namespace wk {

namespace {
thread_local std::string g_err;
}

std::atomic<int> g_alloc_fail_countdown{0};

wk_status set_error(wk_status code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

const std::string &last_error() { return g_err; }

bool is_device_ptr(const void *ptr) {
  if (!ptr) return false;
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, ptr);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

wk_status DevView::from(const void *src, size_t bytes, cudaStream_t st) {
  if (is_device_ptr(src)) {
    dptr = src;
    return WK_OK;
  }
  WK_TRY(tmp.alloc(bytes));
  if (bytes) WK_CUDA(cudaMemcpyAsync(tmp.p, src, bytes, cudaMemcpyHostToDevice, st));
  dptr = tmp.p;
  return WK_OK;
}

wk_status copy_out(void *dst, const void *src, size_t bytes, cudaStream_t st) {
  if (!bytes) return WK_OK;
  WK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, st));
  return WK_OK;
}

size_t dtype_size(int dtype) {
  switch (dtype) {
    case WK_F64: return 8;
    case WK_F32: return 4;
    case WK_BF16: return 2;
    case WK_F16S: return 4;
  }
  return 0;
}

size_t stored_size(int dtype) { return dtype == WK_F16S ? 2 : dtype_size(dtype); }

}  // namespace wk

using namespace wk;

namespace {

cudaStream_t S(void *stream) { return (cudaStream_t)stream; }

void layout_release(wk_layout *l) {
  if (l && l->refs.fetch_sub(1) == 1) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(l->device);
    delete l;  // DevBufs free on the layout's device
    cudaSetDevice(prev);
  }
}

// Renumbering through row_map_inv needs every column index in [0, nrows).
wk_status check_square_cols(const wk_layout *l, const int32_t *dcols, cudaStream_t st) {
  DevBuf bad;
  WK_TRY(bad.alloc(sizeof(int)));
  WK_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
  WK_TRY(launch_check_cols(dcols, l->info.nz, l->info.nrows, bad.as<int>(), st));
  int h = 0;
  WK_CUDA(cudaMemcpyAsync(&h, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  if (h) return set_error(WK_ERR_INVALID, "%d column indices lie outside [0, nrows = %u)", h, l->info.nrows);
  return WK_OK;
}

wk_status scan_common(const int32_t *rowptr, uint32_t nrows, uint32_t nz, int kind, int32_t th,
                      void *stream, wk_layout **out, int variant = 0) {
  if (!out) return set_error(WK_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!rowptr) return set_error(WK_ERR_INVALID, "rowptr is NULL");
  if (nrows > 0x7fffffffu) return set_error(WK_ERR_INVALID, "nrows %u exceeds INT32_MAX", nrows);
  if (nz > 0x7fffffffu) return set_error(WK_ERR_INVALID, "nz %u exceeds INT32_MAX", nz);
  if (!is_device_ptr(rowptr)) {  // host input: reject malformed CSR before any device work
    if (rowptr[0] != 0) return set_error(WK_ERR_INVALID, "rowptr[0] = %d, expected 0", rowptr[0]);
    for (uint32_t r = 0; r < nrows; r++)
      if (rowptr[r + 1] < rowptr[r]) return set_error(WK_ERR_INVALID, "rowptr is not monotone at row %u", r);
    if ((uint32_t)rowptr[nrows] != nz)
      return set_error(WK_ERR_INVALID, "rowptr[nrows] = %d does not equal nz = %u", rowptr[nrows], nz);
  }
  wk_layout *l = new (std::nothrow) wk_layout();
  if (!l) return set_error(WK_ERR_ALLOC, "host allocation failed");
  cudaGetDevice(&l->device);
  l->info.nrows = nrows;
  l->info.nz = nz;
  cudaStream_t st = S(stream);
  wk_status s = l->bufs[7].alloc(((size_t)nrows + 1) * 4);
  if (s == WK_OK) {
    cudaError_t e = cudaMemcpyAsync(l->bufs[7].p, rowptr, ((size_t)nrows + 1) * 4, cudaMemcpyDefault, st);
    if (e != cudaSuccess) s = set_error(WK_ERR_CUDA, "rowptr copy failed: %s", cudaGetErrorString(e));
  }
  if (s == WK_OK) s = build_layout(l, l->bufs[7].as<int32_t>(), kind, th, st, variant);
  if (s != WK_OK) {
    delete l;
    return s;
  }
  *out = l;
  return WK_OK;
}

}  // namespace

namespace wk {
wk_status make_layout(const int32_t *d_rowptr, uint32_t nrows, uint32_t nz, int kind, int32_t threshold,
                      cudaStream_t stream, wk_layout **out, int variant) {
  return scan_common(d_rowptr, nrows, nz, kind, threshold, stream, out, variant);
}

wk_status require_interleaved(const wk_layout *l, const char *op) {
  if (l && (l->info.variant & WK_ABL_NOCOALESCE))
    return set_error(WK_ERR_INVALID, "%s does not accept a non-interleaved (WK_ABL_NOCOALESCE) layout", op);
  return WK_OK;
}
}  // namespace wk

extern "C" {

size_t wk_last_error(char *buf, size_t cap) {
  const std::string &e = last_error();
  if (buf && cap) {
    size_t n = e.size() < cap - 1 ? e.size() : cap - 1;
    memcpy(buf, e.data(), n);
    buf[n] = 0;
  }
  return e.size();
}

const char *wk_version(void) { return "warpkernel_gb300 0.1 (sm_103a)"; }

void wk_debug_fail_alloc(int nth) { g_alloc_fail_countdown.store(nth > 0 ? nth : 0); }

wk_status wk_scan1(const int32_t *rowptr, uint32_t nrows, uint32_t nz, void *stream, wk_layout **out) {
  return scan_common(rowptr, nrows, nz, WK_WPK1, 0, stream, out);
}

wk_status wk_scan2(const int32_t *rowptr, uint32_t nrows, uint32_t nz, int32_t threshold, void *stream,
                   wk_layout **out) {
  return scan_common(rowptr, nrows, nz, WK_WPK2, threshold, stream, out);
}

wk_status wk_scan1_ablation(const int32_t *rowptr, uint32_t nrows, uint32_t nz, int flags, void *stream,
                            wk_layout **out) {
  if (flags & ~(WK_ABL_NOSORT | WK_ABL_NOCOALESCE)) {
    if (out) *out = nullptr;
    return set_error(WK_ERR_INVALID, "unknown ablation flags %d", flags);
  }
  return scan_common(rowptr, nrows, nz, WK_WPK1, 0, stream, out, flags);
}

wk_status wk_layout_info_get(const wk_layout *l, wk_layout_info *info) {
  if (!l || !info) return set_error(WK_ERR_INVALID, "NULL argument");
  *info = l->info;
  return WK_OK;
}

wk_status wk_layout_get(const wk_layout *l, int field, void *dst, size_t cap, size_t *count) {
  if (!l) return set_error(WK_ERR_INVALID, "layout is NULL");
  const wk_layout_info &I = l->info;
  const void *src = nullptr;
  size_t n = 0;
  const bool k2 = I.kind == WK_WPK2;
  switch (field) {
    case WK_FIELD_ROW_MAP: src = l->d.row_map; n = I.nrows; break;
    case WK_FIELD_ROW_MAP_INV: src = l->d.row_map_inv; n = I.nrows; break;
    case WK_FIELD_REORDER_ROWS: src = l->d.reorder_rows; n = I.nz; break;
    case WK_FIELD_WARP_OFFSETS: src = l->d.warp_offsets; n = (size_t)I.nwarps + 1; break;
    case WK_FIELD_MAX_NZ_ROWS: src = l->d.max_nz_rows; n = I.nwarps; break;
    case WK_FIELD_THREADS_PER_ROW: src = l->d.threads_per_row; n = k2 ? I.nwarps : 0; break;
    case WK_FIELD_ROW_OFFSET_WARP: src = l->d.row_offset_warp; n = k2 ? (size_t)I.nwarps + 1 : 0; break;
    default: return set_error(WK_ERR_INVALID, "unknown field %d", field);
  }
  if (count) *count = n;
  if (!dst) return WK_OK;
  if (cap < n) return set_error(WK_ERR_INVALID, "capacity %zu < %zu elements", cap, n);
  if (n) {
    WK_CUDA(cudaMemcpy(dst, src, n * 4, cudaMemcpyDefault));
  }
  return WK_OK;
}

wk_status wk_layout_destroy(wk_layout *l) {
  layout_release(l);
  return WK_OK;
}

wk_status wk_reorder_columns_coalesced(const wk_layout *l, const int32_t *cols, int32_t *out, void *stream) {
  if (!l || !cols || !out) return set_error(WK_ERR_INVALID, "NULL argument");
  cudaStream_t st = S(stream);
  DevView c;
  WK_TRY(c.from(cols, (size_t)l->info.nz * 4, st));
  WK_TRY(check_square_cols(l, (const int32_t *)c.dptr, st));
  bool dev_out = is_device_ptr(out);
  DevBuf tmp;
  int32_t *dout = out;
  if (!dev_out) {
    WK_TRY(tmp.alloc((size_t)l->info.allocate_nz * 4));
    dout = tmp.as<int32_t>();
  }
  if (l->info.allocate_nz && l->info.nwarps == 0)
    return set_error(WK_ERR_STATE, "inconsistent layout");
  WK_TRY(launch_process(l, nullptr, 8, (const int32_t *)c.dptr, nullptr, dout, true, st));
  if (!dev_out) WK_TRY(copy_out(out, dout, (size_t)l->info.allocate_nz * 4, st));
  WK_CUDA(cudaStreamSynchronize(st));
  return WK_OK;
}

wk_status wk_reorder_columns(const wk_layout *l, const int32_t *cols, int32_t *out, void *stream) {
  if (!l || !cols || !out) return set_error(WK_ERR_INVALID, "NULL argument");
  cudaStream_t st = S(stream);
  DevView c;
  WK_TRY(c.from(cols, (size_t)l->info.nz * 4, st));
  WK_TRY(check_square_cols(l, (const int32_t *)c.dptr, st));
  bool dev_out = is_device_ptr(out);
  DevBuf tmp;
  int32_t *dout = out;
  if (!dev_out) {
    WK_TRY(tmp.alloc((size_t)l->info.nz * 4));
    dout = tmp.as<int32_t>();
  }
  WK_TRY(launch_reorder_columns(l, (const int32_t *)c.dptr, dout, st));
  if (!dev_out) WK_TRY(copy_out(out, dout, (size_t)l->info.nz * 4, st));
  WK_CUDA(cudaStreamSynchronize(st));
  return WK_OK;
}

wk_status wk_reorder_x(const wk_layout *l, int dtype, const void *x, void *x_out, void *stream) {
  if (!l || !x || !x_out) return set_error(WK_ERR_INVALID, "NULL argument");
  size_t eb = dtype_size(dtype);
  if (!eb) return set_error(WK_ERR_INVALID, "unknown dtype %d", dtype);
  cudaStream_t st = S(stream);
  size_t bytes = (size_t)l->info.nrows * eb;
  DevView xv;
  WK_TRY(xv.from(x, bytes, st));
  bool dev_out = is_device_ptr(x_out);
  DevBuf tmp;
  void *dout = x_out;
  if (!dev_out) {
    WK_TRY(tmp.alloc(bytes));
    dout = tmp.p;
  }
  WK_TRY(launch_reorder_x(l, xv.dptr, dout, (int)eb, st));
  if (!dev_out) {
    WK_TRY(copy_out(x_out, dout, bytes, st));
    WK_CUDA(cudaStreamSynchronize(st));
  } else if (xv.tmp.p) {
    WK_CUDA(cudaStreamSynchronize(st));
  }
  return WK_OK;
}

wk_status wk_engine_create(wk_layout *l, int dtype, const void *vals, const int32_t *cols, uint32_t ncols,
                           void *stream, wk_engine **out) {
  if (!out) return set_error(WK_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!l || !vals || !cols) return set_error(WK_ERR_INVALID, "NULL argument");
  size_t eb = dtype_size(dtype);
  if (!eb) return set_error(WK_ERR_INVALID, "unknown dtype %d", dtype);
  if (ncols == 0 && l->info.nz) return set_error(WK_ERR_INVALID, "ncols is 0 but the matrix has entries");
  cudaStream_t st = S(stream);
  wk_engine *e = new (std::nothrow) wk_engine();
  if (!e) return set_error(WK_ERR_ALLOC, "host allocation failed");
  e->dtype = dtype;
  e->ncols = ncols;
  // x windows with the compact columns: on for 4-byte x (FP32, scaled FP16),
  // where the asynchronous window copy made them the faster form; off for
  // BF16, whose 2-byte x is staged by loads and stores (measured slower)
  e->use_windows = dtype == WK_F32 || dtype == WK_F16S;
  const size_t anz = l->info.allocate_nz, nz = l->info.nz;
  wk_status s = WK_OK;
  DevView v, c;
  if (s == WK_OK) s = v.from(vals, nz * eb, st);
  if (s == WK_OK) s = c.from(cols, nz * 4, st);
  if (s == WK_OK) s = e->vals.alloc(anz * stored_size(dtype));
  if (s == WK_OK) s = e->cols.alloc(anz * 4);
  if (s == WK_OK) s = e->status.alloc(64);
  if (s == WK_OK && dtype == WK_F16S) s = e->scale.alloc((size_t)l->info.nwarps * 4);
  int bad = 0;
  if (s == WK_OK) {
    cudaMemsetAsync(e->status.p, 0, 64, st);
    s = launch_check_cols((const int32_t *)c.dptr, nz, ncols, e->status.as<int>(), st);
  }
  e->layout = l;  // not yet referenced: cleared again on failure
  if (s == WK_OK) s = launch_process(l, nullptr, (int)eb, (const int32_t *)c.dptr, nullptr,
                                     e->cols.as<int32_t>(), false, st);
  if (s == WK_OK) s = load_values(e, v.dptr, st);
  if (s == WK_OK) {
    cudaError_t ce = cudaMemcpyAsync(&bad, e->status.p, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) s = set_error(WK_ERR_CUDA, "engine creation: %s", cudaGetErrorString(ce));
  }
  if (s == WK_OK && bad)
    s = set_error(WK_ERR_INVALID, "%d column indices lie outside [0, %u)", bad, ncols);
  if (s != WK_OK) {
    e->layout = nullptr;
    delete e;
    return s;
  }
  l->refs.fetch_add(1);
  *out = e;
  return WK_OK;
}

wk_status wk_engine_set_colinds(wk_engine *e, const int32_t *padded_cols, void *stream) {
  if (!e || !padded_cols) return set_error(WK_ERR_INVALID, "NULL argument");
  cudaStream_t st = S(stream);
  const size_t anz = e->layout->info.allocate_nz;
  DevView c;
  WK_TRY(c.from(padded_cols, anz * 4, st));
  WK_CUDA(cudaMemsetAsync(e->status.p, 0, sizeof(int), st));
  WK_TRY(launch_check_cols((const int32_t *)c.dptr, anz, e->ncols, e->status.as<int>(), st));
  int bad = 0;
  WK_CUDA(cudaMemcpyAsync(&bad, e->status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  if (bad) return set_error(WK_ERR_INVALID, "%d column indices lie outside [0, %u)", bad, e->ncols);
  if (anz) WK_CUDA(cudaMemcpyAsync(e->cols.p, c.dptr, anz * 4, cudaMemcpyDeviceToDevice, st));
  WK_CUDA(cudaStreamSynchronize(st));
  if (e->compressed) WK_TRY(build_compressed_cols(e, st, nullptr));
  return WK_OK;
}

wk_status wk_engine_set_values(wk_engine *e, const void *vals, void *stream) {
  if (!e || !vals) return set_error(WK_ERR_INVALID, "NULL argument");
  cudaStream_t st = S(stream);
  const size_t eb = dtype_size(e->dtype);
  DevView v;
  WK_TRY(v.from(vals, (size_t)e->layout->info.nz * eb, st));
  WK_TRY(load_values(e, v.dptr, st));
  if (v.tmp.p) WK_CUDA(cudaStreamSynchronize(st));
  return WK_OK;
}

wk_status wk_engine_get_values(const wk_engine *e, void *dst, size_t cap) {
  if (!e || !dst) return set_error(WK_ERR_INVALID, "NULL argument");
  size_t n = e->layout->info.allocate_nz;
  if (cap < n) return set_error(WK_ERR_INVALID, "capacity %zu < %zu", cap, n);
  if (n && e->dtype == WK_F16S) {  // the values the SpMV multiplies with, as FP32
    DevBuf t;
    WK_TRY(t.alloc(n * 4));
    WK_TRY(launch_f16s_decode(e, t.as<float>(), nullptr));
    WK_CUDA(cudaMemcpy(dst, t.p, n * 4, cudaMemcpyDefault));
    return WK_OK;
  }
  if (n) WK_CUDA(cudaMemcpy(dst, e->vals.p, n * dtype_size(e->dtype), cudaMemcpyDefault));
  return WK_OK;
}

wk_status wk_engine_get_colinds(const wk_engine *e, int32_t *dst, size_t cap) {
  if (!e || !dst) return set_error(WK_ERR_INVALID, "NULL argument");
  size_t n = e->layout->info.allocate_nz;
  if (cap < n) return set_error(WK_ERR_INVALID, "capacity %zu < %zu", cap, n);
  if (n) WK_CUDA(cudaMemcpy(dst, e->cols.p, n * 4, cudaMemcpyDefault));
  return WK_OK;
}

wk_status wk_engine_destroy(wk_engine *e) {
  if (!e) return WK_OK;
  wk_layout *l = e->layout;
  int prev = 0;
  cudaGetDevice(&prev);
  if (l) cudaSetDevice(l->device);
  delete e;
  cudaSetDevice(prev);
  layout_release(l);
  return WK_OK;
}

static wk_status run_common(wk_engine *e, int nblocks, int blocksize, int cache, int order, const void *dx,
                            void *dy, void *stream, float *seconds, bool mapped) {
  if (!e || !dx || !dy) return set_error(WK_ERR_INVALID, "NULL argument");
  if (order != WK_ORDER_FAST && order != WK_ORDER_EXACT)
    return set_error(WK_ERR_INVALID, "unknown order %d", order);
  cudaStream_t st = S(stream);
  RunArgs a{e, nblocks, blocksize, cache, order, mapped, dx, dy, st};
  if (!seconds) return launch_spmv(a);
  cudaEvent_t t0, t1;
  WK_CUDA(cudaEventCreate(&t0));
  WK_CUDA(cudaEventCreate(&t1));
  cudaEventRecord(t0, st);
  wk_status s = launch_spmv(a);
  cudaEventRecord(t1, st);
  cudaError_t ce = cudaEventSynchronize(t1);
  float ms = 0.f;
  if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (s != WK_OK) return s;
  if (ce != cudaSuccess) return set_error(WK_ERR_CUDA, "run: %s", cudaGetErrorString(ce));
  *seconds = ms * 1e-3f;
  return WK_OK;
}

wk_status wk_run(wk_engine *e, int nblocks, int blocksize, int cache, int order, const void *dx, void *dy,
                 void *stream, float *seconds) {
  return run_common(e, nblocks, blocksize, cache, order, dx, dy, stream, seconds, true);
}

wk_status wk_run_x(wk_engine *e, int nblocks, int blocksize, int cache, int order, const void *dx, void *dy,
                   void *stream, float *seconds) {
  return run_common(e, nblocks, blocksize, cache, order, dx, dy, stream, seconds, false);
}

wk_status wk_run_host(wk_engine *e, int mapped, int order, const void *x_host, void *y_host, void *stream) {
  if (!e || !x_host || !y_host) return set_error(WK_ERR_INVALID, "NULL argument");
  cudaStream_t st = S(stream);
  const size_t xb = (size_t)e->ncols * dtype_size(e->dtype);
  const size_t yb = (size_t)e->layout->info.nrows * (e->dtype == WK_F64 ? 8 : 4);
  if (!e->xbuf.p) WK_TRY(e->xbuf.alloc(xb));
  if (!e->ybuf.p) WK_TRY(e->ybuf.alloc(yb));
  if (xb) WK_CUDA(cudaMemcpyAsync(e->xbuf.p, x_host, xb, cudaMemcpyHostToDevice, st));
  if (e->layout->info.nznrows < e->layout->info.nrows) WK_CUDA(cudaMemsetAsync(e->ybuf.p, 0, yb, st));
  RunArgs a{e, 0, 0, 1, order, mapped != 0, e->xbuf.p, e->ybuf.p, st};
  WK_TRY(launch_spmv(a));
  if (yb) WK_CUDA(cudaMemcpyAsync(y_host, e->ybuf.p, yb, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  return WK_OK;
}

namespace {
// Streams and events of one wk_run_host_stream call, released on every exit.
struct HostStreamRes {
  cudaStream_t h2d = nullptr, d2h = nullptr;
  cudaEvent_t ev[7] = {};  // h2d done [2], SpMV done [2], d2h done [2], start
  ~HostStreamRes() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (h2d) cudaStreamDestroy(h2d);
    if (d2h) cudaStreamDestroy(d2h);
  }
};
}  // namespace

wk_status wk_run_host_stream(wk_engine *e, int mapped, int order, int count, const void *const *x_host,
                             void *const *y_host, void *stream, float *seconds) {
  if (!e || count < 0 || (count && (!x_host || !y_host))) return set_error(WK_ERR_INVALID, "NULL argument");
  for (int i = 0; i < count; i++)
    if (!x_host[i] || !y_host[i]) return set_error(WK_ERR_INVALID, "vector %d is NULL", i);
  cudaStream_t st = S(stream);
  const size_t xb = (size_t)e->ncols * dtype_size(e->dtype);
  const size_t yb = (size_t)e->layout->info.nrows * (e->dtype == WK_F64 ? 8 : 4);
  if (!e->xbuf.p) WK_TRY(e->xbuf.alloc(xb));
  if (!e->ybuf.p) WK_TRY(e->ybuf.alloc(yb));
  if (!e->xbuf2.p) WK_TRY(e->xbuf2.alloc(xb));
  if (!e->ybuf2.p) WK_TRY(e->ybuf2.alloc(yb));
  wk::DevBuf *xs[2] = {&e->xbuf, &e->xbuf2}, *ys[2] = {&e->ybuf, &e->ybuf2};
  HostStreamRes r;
  WK_CUDA(cudaStreamCreateWithFlags(&r.h2d, cudaStreamNonBlocking));
  WK_CUDA(cudaStreamCreateWithFlags(&r.d2h, cudaStreamNonBlocking));
  for (int k = 0; k < 6; k++) WK_CUDA(cudaEventCreateWithFlags(&r.ev[k], cudaEventDisableTiming));
  cudaEvent_t *h2d_done = r.ev, *run_done = r.ev + 2, *d2h_done = r.ev + 4;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (seconds) {
    WK_CUDA(cudaEventCreate(&r.ev[6]));
    t0 = r.ev[6];
    WK_CUDA(cudaEventRecord(t0, st));
  }
  // empty rows are never written by the SpMV: zero both staging vectors once
  if (e->layout->info.nznrows < e->layout->info.nrows)
    for (int b = 0; b < 2; b++) WK_CUDA(cudaMemsetAsync(ys[b]->p, 0, yb, st));
  WK_CUDA(cudaEventRecord(run_done[0], st));  // uploads start after the memsets
  WK_CUDA(cudaEventRecord(run_done[1], st));
  WK_CUDA(cudaStreamWaitEvent(r.h2d, run_done[0], 0));
  for (int i = 0; i < count; i++) {
    const int b = i & 1;
    // x_i into buffer b once SpMV i-2 (its last reader) is done
    if (i >= 2) WK_CUDA(cudaStreamWaitEvent(r.h2d, run_done[b], 0));
    if (xb) WK_CUDA(cudaMemcpyAsync(xs[b]->p, x_host[i], xb, cudaMemcpyHostToDevice, r.h2d));
    WK_CUDA(cudaEventRecord(h2d_done[b], r.h2d));
    // SpMV i after its upload and after y_{i-2} left buffer b
    WK_CUDA(cudaStreamWaitEvent(st, h2d_done[b], 0));
    if (i >= 2) WK_CUDA(cudaStreamWaitEvent(st, d2h_done[b], 0));
    RunArgs a{e, 0, 0, 1, order, mapped != 0, xs[b]->p, ys[b]->p, st};
    WK_TRY(launch_spmv(a));
    WK_CUDA(cudaEventRecord(run_done[b], st));
    WK_CUDA(cudaStreamWaitEvent(r.d2h, run_done[b], 0));
    if (yb) WK_CUDA(cudaMemcpyAsync(y_host[i], ys[b]->p, yb, cudaMemcpyDeviceToHost, r.d2h));
    WK_CUDA(cudaEventRecord(d2h_done[b], r.d2h));
  }
  if (count) {
    WK_CUDA(cudaStreamWaitEvent(st, d2h_done[(count - 1) & 1], 0));
    if (count > 1) WK_CUDA(cudaStreamWaitEvent(st, d2h_done[count & 1], 0));
  }
  if (seconds) {
    WK_CUDA(cudaEventCreate(&t1));
    cudaEventRecord(t1, st);
  }
  cudaError_t ce = cudaStreamSynchronize(st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(r.d2h);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(r.h2d);
  if (ce == cudaSuccess && seconds) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    *seconds = ms * 1e-3f;
  }
  if (t1) cudaEventDestroy(t1);
  if (ce != cudaSuccess) return set_error(WK_ERR_CUDA, "run_host_stream: %s", cudaGetErrorString(ce));
  return WK_OK;
}

wk_status wk_verify(const wk_layout *l, const double *orig, const double *comp, int *pass, int64_t *first_bad) {
  if (!l || !orig || !comp || !pass) return set_error(WK_ERR_INVALID, "NULL argument");
  const uint32_t n = l->info.nrows;
  *pass = 1;
  if (first_bad) *first_bad = -1;
  for (uint32_t i = 0; i < n; i++) {
    double o = orig[i], c = comp[i];
    if ((std::fabs(o) <= 1e-14 && std::fabs(o - c) > 1e-14) ||
        (std::fabs((o - c) / o) > 1e-5 && std::fabs(o) > 1e-14)) {
      *pass = 0;
      if (first_bad) *first_bad = i;
      break;
    }
  }
  return WK_OK;
}

wk_status wk_verify_x(const wk_layout *l, const double *orig, const double *comp, int strict, int *pass,
                      int64_t *first_bad) {
  if (!l || !orig || !comp || !pass) return set_error(WK_ERR_INVALID, "NULL argument");
  const uint32_t n = l->info.nrows;
  std::vector<int32_t> rm(n);
  WK_TRY(wk_layout_get(l, WK_FIELD_ROW_MAP, rm.data(), n, nullptr));
  *pass = 1;
  if (first_bad) *first_bad = -1;
  for (uint32_t i = 0; i < n; i++) {
    double om = orig[rm[i]], c = comp[i];
    double ou = strict ? om : orig[i];
    if ((std::fabs(om) <= 1e-14 && std::fabs(ou - c) > 1e-14) ||
        (std::fabs((om - c) / om) > 1e-5 && std::fabs(ou) > 1e-14)) {
      *pass = 0;
      if (first_bad) *first_bad = i;
      break;
    }
  }
  return WK_OK;
}

wk_status wk_fe_size(int dim, int ex, int ey, int ez, int dof, int64_t *nrows, int64_t *nnz) {
  if (!nrows || !nnz) return set_error(WK_ERR_INVALID, "NULL argument");
  if ((dim != 2 && dim != 3) || ex < 1 || ey < 1 || dof < 1 || (dim == 3 && ez < 1))
    return set_error(WK_ERR_INVALID, "bad mesh");
  int64_t nx = ex + 1, ny = ey + 1, nzn = dim == 3 ? ez + 1 : 1;
  auto axis = [](int64_t n) { return n == 1 ? (int64_t)1 : 3 * n - 2; };  // sum of neighbour counts
  *nrows = nx * ny * nzn * dof;
  *nnz = axis(nx) * axis(ny) * axis(nzn) * dof * dof;
  return WK_OK;
}

wk_status wk_fe_fill(int dim, int ex, int ey, int ez, int dof, int value_mode, uint64_t seed, int32_t *rowptr,
                     int32_t *cols, double *vals, void *stream) {
  int64_t n = 0, z = 0;
  WK_TRY(wk_fe_size(dim, ex, ey, ez, dof, &n, &z));
  if (z > 0x7fffffffLL) return set_error(WK_ERR_OVERFLOW, "nnz %lld exceeds INT32_MAX", (long long)z);
  if (value_mode != 0 && value_mode != 1) return set_error(WK_ERR_INVALID, "value_mode %d", value_mode);
  return launch_fe_fill(dim, ex, ey, ez, dof, value_mode, seed, rowptr, cols, vals, S(stream));
}

wk_status wk_uniform_vec(uint64_t seed, uint64_t stream_id, double *x, int64_t n, void *stream) {
  if (!x || n < 0) return set_error(WK_ERR_INVALID, "bad argument");
  return launch_uniform(seed, stream_id, x, n, S(stream));
}

wk_status wk_convert(const void *src, int sdt, void *dst, int ddt, int64_t n, void *stream) {
  if (!src || !dst || n < 0 || !dtype_size(sdt) || !dtype_size(ddt))
    return set_error(WK_ERR_INVALID, "bad argument");
  return launch_convert(src, sdt, dst, ddt, n, S(stream));
}

}  // extern "C"

namespace wk {
wk_status make_engine(wk_layout *l, int dtype, const void *d_vals, const int32_t *d_cols, uint32_t ncols,
                      cudaStream_t stream, wk_engine **out) {
  return wk_engine_create(l, dtype, d_vals, d_cols, ncols, stream, out);
}
}  // namespace wk
