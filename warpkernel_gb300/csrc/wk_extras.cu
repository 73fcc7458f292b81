// wk_extras.cu -- the callers and data formats either side of the SpMV:
//  * Matrix Market ingest (the drivers' input, wpk1.cu:43-48, wpk2.cu:54-57);
//  * WPK layout files (the fields of structure::serialize,
//    warpkernel.hpp:253-269, plus WPK2's arrays) so a layout is scanned once;
//  * run_assembly: row sums of the stored values (warpkernel.hpp:78-100,
//    898-929), the finite-element assembly kernel;
//  * reorder_columns_rowsort (warpkernel.hpp:414-444): renumbered columns
//    sorted within each row, with the source positions reorder_A_rows.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "wk_internal.cuh"
#include "wk_spmv_core.cuh"

struct wk_csr {
  int64_t nrows = 0, ncols = 0;
  std::vector<int32_t> rowptr, cols;
  std::vector<double> vals;
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

// ---- run_assembly ----------------------------------------------------------------
// y[row_map[p]] = first slot value, then += each further slot (the reference's
// order), WPK2 rows through the same lockstep tree as run.
template <typename V>
__global__ void k_assembly(const V *__restrict__ pv, const int4 *__restrict__ desc, uint32_t W,
                           const int32_t *__restrict__ row_map, uint32_t nzr, typename core::Tr<V>::Acc *__restrict__ y,
                           const float *__restrict__ wscale) {
  typedef typename core::Tr<V>::Acc Acc;
  const uint32_t lane = threadIdx.x & 31;
  const size_t w = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / WS;
  if (w >= W) return;
  const int4 d = desc[w];
  const uint32_t T = (uint32_t)d.z;
  const uint32_t p = (uint32_t)d.w + lane / T;
  const bool valid = p < nzr;
  Acc s = Acc(0);
  if (valid) {
    size_t o = (size_t)(uint32_t)d.x + lane;
    const size_t end = o + (size_t)WS * (uint32_t)d.y;
    s = core::Tr<V>::acc(pv[o]);
    for (o += WS; o < end; o += WS) s += core::Tr<V>::acc(pv[o]);
  }
  s = core::row_tree(s, T);
  if constexpr (core::Scaled<V>::value) s *= wscale[w];
  if (valid && (lane & (T - 1)) == 0) y[row_map[p]] = s;
}

// ---- rowsort -----------------------------------------------------------------------
// Within each row the renumbered columns row_map_inv[cols[k]] are put in
// ascending order by two stable radix passes (by column, then by row), so
// every row length costs O(nz) and equal columns keep their CSR order.
__global__ void k_rs_keys(const int32_t *__restrict__ cols, const int32_t *__restrict__ row_map_inv, uint32_t nz,
                          uint32_t *__restrict__ key, uint32_t *__restrict__ idx) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nz; i += (size_t)gridDim.x * blockDim.x) {
    key[i] = (uint32_t)row_map_inv[cols[i]];
    idx[i] = (uint32_t)i;
  }
}

__global__ void k_rs_rowkeys(const int32_t *__restrict__ rowptr, uint32_t nrows, const uint32_t *__restrict__ src,
                             uint32_t nz, uint32_t *__restrict__ key, uint32_t *__restrict__ idx) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nz; i += (size_t)gridDim.x * blockDim.x) {
    const int32_t k = (int32_t)src[i];
    uint32_t lo = 0, hi = nrows;  // last row r with rowptr[r] <= k
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) / 2;
      if (rowptr[mid] <= k) lo = mid; else hi = mid;
    }
    key[i] = lo;
    idx[i] = (uint32_t)k;
  }
}

__global__ void k_rs_out(const int32_t *__restrict__ cols, const int32_t *__restrict__ row_map_inv,
                         const uint32_t *__restrict__ src, uint32_t nz, int32_t *__restrict__ out_cols,
                         int32_t *__restrict__ out_src) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nz; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t k = src[i];
    out_src[i] = (int32_t)k;
    out_cols[i] = row_map_inv[cols[k]];
  }
}

int key_bits(uint32_t maxkey) {
  int b = 0;
  while (b < 32 && (maxkey >> b)) b++;
  return b;
}

// ---- Matrix Market ------------------------------------------------------------------
std::string lower(std::string s) {
  for (char &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

wk_status read_mm(const char *path, wk_csr *out) {
  FILE *f = std::fopen(path, "r");
  if (!f) return set_error(WK_ERR_INVALID, "cannot open %s", path);
  char line[4096];
  if (!std::fgets(line, sizeof line, f)) {
    std::fclose(f);
    return set_error(WK_ERR_INVALID, "%s: empty file", path);
  }
  char banner[64] = {0}, object[64] = {0}, format[64] = {0}, field[64] = {0}, sym[64] = {0};
  if (std::sscanf(line, "%63s %63s %63s %63s %63s", banner, object, format, field, sym) != 5 ||
      lower(banner) != "%%matrixmarket" || lower(object) != "matrix") {
    std::fclose(f);
    return set_error(WK_ERR_INVALID, "%s: not a Matrix Market matrix header", path);
  }
  const std::string fmt = lower(format), fld = lower(field), sy = lower(sym);
  if (fmt != "coordinate") {
    std::fclose(f);
    return set_error(WK_ERR_INVALID, "%s: only the coordinate format is supported", path);
  }
  if (fld != "real" && fld != "integer" && fld != "pattern" && fld != "double") {
    std::fclose(f);
    return set_error(WK_ERR_INVALID, "%s: field '%s' is not supported", path, field);
  }
  if (sy != "general" && sy != "symmetric" && sy != "skew-symmetric") {
    std::fclose(f);
    return set_error(WK_ERR_INVALID, "%s: symmetry '%s' is not supported", path, sym);
  }
  long long m = 0, n = 0, nent = 0;
  for (;;) {
    if (!std::fgets(line, sizeof line, f)) {
      std::fclose(f);
      return set_error(WK_ERR_INVALID, "%s: missing size line", path);
    }
    if (line[0] == '%') continue;
    if (std::sscanf(line, "%lld %lld %lld", &m, &n, &nent) == 3) break;
    std::fclose(f);
    return set_error(WK_ERR_INVALID, "%s: bad size line", path);
  }
  if (m < 0 || n < 0 || nent < 0 || m > 0x7fffffffLL || n > 0x7fffffffLL) {
    std::fclose(f);
    return set_error(WK_ERR_INVALID, "%s: sizes out of range", path);
  }
  struct E {
    int32_t r, c;
    double v;
  };
  std::vector<E> e;
  e.reserve((size_t)nent * (sy == "general" ? 1 : 2));
  for (long long i = 0; i < nent; i++) {
    long long r, c;
    double v = 1.0;
    int got;
    do {
      if (!std::fgets(line, sizeof line, f)) {
        std::fclose(f);
        return set_error(WK_ERR_INVALID, "%s: %lld of %lld entries", path, i, nent);
      }
    } while (line[0] == '%' || line[0] == '\n');
    got = fld == "pattern" ? std::sscanf(line, "%lld %lld", &r, &c) : std::sscanf(line, "%lld %lld %lf", &r, &c, &v);
    if (got < (fld == "pattern" ? 2 : 3) || r < 1 || r > m || c < 1 || c > n) {
      std::fclose(f);
      return set_error(WK_ERR_INVALID, "%s: bad entry %lld", path, i + 1);
    }
    e.push_back({(int32_t)(r - 1), (int32_t)(c - 1), v});
    if (sy != "general" && r != c) e.push_back({(int32_t)(c - 1), (int32_t)(r - 1), sy == "skew-symmetric" ? -v : v});
  }
  std::fclose(f);
  if (e.size() > 0x7fffffffULL) return set_error(WK_ERR_OVERFLOW, "%s: more than INT32_MAX entries", path);
  std::stable_sort(e.begin(), e.end(), [](const E &a, const E &b) { return a.r != b.r ? a.r < b.r : a.c < b.c; });
  out->nrows = m;
  out->ncols = n;
  out->rowptr.assign((size_t)m + 1, 0);
  out->cols.resize(e.size());
  out->vals.resize(e.size());
  for (size_t i = 0; i < e.size(); i++) {
    out->rowptr[(size_t)e[i].r + 1]++;
    out->cols[i] = e[i].c;
    out->vals[i] = e[i].v;
  }
  for (long long r = 0; r < m; r++) out->rowptr[(size_t)r + 1] += out->rowptr[(size_t)r];
  return WK_OK;
}

const char kMagic[8] = {'W', 'P', 'K', 'L', 'A', 'Y', 'T', '1'};

template <typename T>
bool put_array(FILE *f, const T *d, uint64_t n) {
  if (std::fwrite(&n, 8, 1, f) != 1) return false;
  if (!n) return true;
  std::vector<T> h(n);
  if (cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess) return false;
  return std::fwrite(h.data(), sizeof(T), n, f) == n;
}

template <typename T>
bool get_array(FILE *f, std::vector<T> &h, uint64_t expect) {
  uint64_t n = 0;
  if (std::fread(&n, 8, 1, f) != 1 || n != expect) return false;
  h.resize(n);
  return !n || std::fread(h.data(), sizeof(T), n, f) == n;
}

}  // namespace
}  // namespace wk

using namespace wk;

extern "C" wk_status wk_run_assembly(wk_engine *e, int nblocks, int blocksize, void *dy, void *stream,
                                     float *seconds) {
  if (!e || !dy) return set_error(WK_ERR_INVALID, "NULL argument");
  WK_TRY(require_interleaved(e->layout, "wk_run_assembly"));
  const wk_layout *l = e->layout;
  unsigned grid, block;
  WK_TRY(launch_shape(l->info.nwarps, nblocks, blocksize, &grid, &block));
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (seconds) {
    WK_CUDA(cudaEventCreate(&t0));
    WK_CUDA(cudaEventCreate(&t1));
    cudaEventRecord(t0, st);
  }
  if (l->info.nwarps) {
    const uint32_t W = l->info.nwarps, nzr = l->info.nznrows;
    switch (e->dtype) {
      case WK_F64: k_assembly<double><<<grid, block, 0, st>>>(e->vals.as<double>(), l->d.warp_desc, W, l->d.row_map, nzr, (double *)dy, nullptr); break;
      case WK_F32: k_assembly<float><<<grid, block, 0, st>>>(e->vals.as<float>(), l->d.warp_desc, W, l->d.row_map, nzr, (float *)dy, nullptr); break;
      case WK_F16S: k_assembly<__half><<<grid, block, 0, st>>>(e->vals.as<__half>(), l->d.warp_desc, W, l->d.row_map, nzr, (float *)dy, e->scale.as<float>()); break;
      default: k_assembly<__nv_bfloat16><<<grid, block, 0, st>>>(e->vals.as<__nv_bfloat16>(), l->d.warp_desc, W, l->d.row_map, nzr, (float *)dy, nullptr); break;
    }
    WK_CHECK_LAUNCH();
  }
  if (seconds) {
    cudaEventRecord(t1, st);
    cudaError_t ce = cudaEventSynchronize(t1);
    float ms = 0.f;
    if (ce == cudaSuccess) cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (ce != cudaSuccess) return set_error(WK_ERR_CUDA, "run_assembly: %s", cudaGetErrorString(ce));
    *seconds = ms * 1e-3f;
  }
  return WK_OK;
}

extern "C" wk_status wk_reorder_columns_rowsort(const wk_layout *l, const int32_t *cols, int32_t *out_cols,
                                                int32_t *reorder_A_rows, void *stream) {
  if (!l || !cols || !out_cols || !reorder_A_rows) return set_error(WK_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t nz = l->info.nz;
  DevView c;
  WK_TRY(c.from(cols, nz * 4, st));
  {
    DevBuf bad;
    WK_TRY(bad.alloc(4));
    WK_CUDA(cudaMemsetAsync(bad.p, 0, 4, st));
    WK_TRY(launch_check_cols((const int32_t *)c.dptr, nz, l->info.nrows, bad.as<int>(), st));
    int h = 0;
    WK_CUDA(cudaMemcpyAsync(&h, bad.p, 4, cudaMemcpyDeviceToHost, st));
    WK_CUDA(cudaStreamSynchronize(st));
    if (h) return set_error(WK_ERR_INVALID, "%d column indices lie outside [0, nrows)", h);
  }
  const bool dev_c = is_device_ptr(out_cols), dev_s = is_device_ptr(reorder_A_rows);
  DevBuf tc, ts;
  int32_t *oc = out_cols, *os = reorder_A_rows;
  if (!dev_c) {
    WK_TRY(tc.alloc(nz * 4));
    oc = tc.as<int32_t>();
  }
  if (!dev_s) {
    WK_TRY(ts.alloc(nz * 4));
    os = ts.as<int32_t>();
  }
  if (nz) {
    const uint32_t n = l->info.nrows;
    DevBuf k0, k1, v0, v1;
    WK_TRY(k0.alloc(nz * 4));
    WK_TRY(k1.alloc(nz * 4));
    WK_TRY(v0.alloc(nz * 4));
    WK_TRY(v1.alloc(nz * 4));
    const unsigned g = grid_for(nz, 256);
    k_rs_keys<<<g, 256, 0, st>>>((const int32_t *)c.dptr, l->d.row_map_inv, (uint32_t)nz, k0.as<uint32_t>(),
                                 v0.as<uint32_t>());
    WK_CHECK_LAUNCH();
    int which = 0;
    WK_TRY(radix_sort_pairs(k0.as<uint32_t>(), k1.as<uint32_t>(), v0.as<uint32_t>(), v1.as<uint32_t>(),
                            (uint32_t)nz, key_bits(n - 1), st, &which));
    uint32_t *rk = which ? k1.as<uint32_t>() : k0.as<uint32_t>(), *rv = which ? v1.as<uint32_t>() : v0.as<uint32_t>();
    uint32_t *fk = which ? k0.as<uint32_t>() : k1.as<uint32_t>(), *fv = which ? v0.as<uint32_t>() : v1.as<uint32_t>();
    k_rs_rowkeys<<<g, 256, 0, st>>>(l->d.rowptr, n, rv, (uint32_t)nz, fk, fv);
    WK_CHECK_LAUNCH();
    WK_TRY(radix_sort_pairs(fk, rk, fv, rv, (uint32_t)nz, key_bits(n - 1), st, &which));
    k_rs_out<<<g, 256, 0, st>>>((const int32_t *)c.dptr, l->d.row_map_inv, which ? rv : fv, (uint32_t)nz, oc, os);
    WK_CHECK_LAUNCH();
    if (!dev_c) WK_CUDA(cudaMemcpyAsync(out_cols, oc, nz * 4, cudaMemcpyDeviceToHost, st));
    if (!dev_s) WK_CUDA(cudaMemcpyAsync(reorder_A_rows, os, nz * 4, cudaMemcpyDeviceToHost, st));
    WK_CUDA(cudaStreamSynchronize(st));
  }
  return WK_OK;
}

extern "C" wk_status wk_process(const wk_layout *l, int dtype, const void *vals, const int32_t *cols, void *pvals,
                                int32_t *pcols, void *stream) {
  if (!l) return set_error(WK_ERR_INVALID, "layout is NULL");
  if ((pvals && !vals) || (pcols && !cols) || (!pvals && !pcols))
    return set_error(WK_ERR_INVALID, "each output needs its input, and at least one output is required");
  if (dtype != WK_F64 && dtype != WK_F32 && dtype != WK_BF16)
    return set_error(WK_ERR_INVALID, "wk_process: dtype must be WK_F64, WK_F32 or WK_BF16");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t eb = dtype_size(dtype), nz = l->info.nz, anz = l->info.allocate_nz;
  DevView v, c;
  if (pvals) WK_TRY(v.from(vals, nz * eb, st));
  if (pcols) WK_TRY(c.from(cols, nz * 4, st));
  const bool dv = pvals && is_device_ptr(pvals), dc = pcols && is_device_ptr(pcols);
  DevBuf tv, tc;
  void *ov = pvals;
  int32_t *oc = pcols;
  if (pvals && !dv) {
    WK_TRY(tv.alloc(anz * eb));
    ov = tv.p;
  }
  if (pcols && !dc) {
    WK_TRY(tc.alloc(anz * 4));
    oc = tc.as<int32_t>();
  }
  WK_TRY(launch_process(l, pvals ? v.dptr : nullptr, (int)eb, pcols ? (const int32_t *)c.dptr : nullptr, ov, oc, false,
                        st));
  if (pvals && !dv && anz) WK_CUDA(cudaMemcpyAsync(pvals, ov, anz * eb, cudaMemcpyDeviceToHost, st));
  if (pcols && !dc && anz) WK_CUDA(cudaMemcpyAsync(pcols, oc, anz * 4, cudaMemcpyDeviceToHost, st));
  WK_CUDA(cudaStreamSynchronize(st));
  return WK_OK;
}

extern "C" wk_status wk_layout_save(const wk_layout *l, const char *path) {
  if (!l || !path) return set_error(WK_ERR_INVALID, "NULL argument");
  FILE *f = std::fopen(path, "wb");
  if (!f) return set_error(WK_ERR_INVALID, "cannot create %s", path);
  const wk_layout_info &I = l->info;
  const uint32_t version = 1;
  bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(&version, 4, 1, f) == 1 &&
            std::fwrite(&I, sizeof I, 1, f) == 1;
  const bool k2 = I.kind == WK_WPK2;
  ok = ok && put_array(f, l->d.row_map, I.nrows) && put_array(f, l->d.row_map_inv, I.nrows) &&
       put_array(f, l->d.reorder_rows, I.nz) && put_array(f, l->d.warp_offsets, (uint64_t)I.nwarps + 1) &&
       put_array(f, l->d.max_nz_rows, I.nwarps) && put_array(f, l->d.threads_per_row, k2 ? I.nwarps : 0) &&
       put_array(f, l->d.row_offset_warp, k2 ? (uint64_t)I.nwarps + 1 : 0) &&
       put_array(f, l->d.rowptr, (uint64_t)I.nrows + 1);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? WK_OK : set_error(WK_ERR_INVALID, "writing %s failed", path);
}

// A layout file is accepted only if it is exactly what a scan of its own row
// offsets produces: the layout is rebuilt on the device (milliseconds) and
// every array and header field is compared, so a corrupt or edited file can
// never hand a kernel an out-of-range offset or index.
extern "C" wk_status wk_layout_load(const char *path, void *stream, wk_layout **out) {
  if (!path || !out) return set_error(WK_ERR_INVALID, "NULL argument");
  *out = nullptr;
  FILE *f = std::fopen(path, "rb");
  if (!f) return set_error(WK_ERR_INVALID, "cannot open %s", path);
  char magic[8];
  uint32_t version = 0;
  wk_layout_info I;
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kMagic, 8) != 0 || std::fread(&version, 4, 1, f) != 1 ||
      version != 1 || std::fread(&I, sizeof I, 1, f) != 1 || (I.kind != WK_WPK1 && I.kind != WK_WPK2) ||
      I.variant > (WK_ABL_NOSORT | WK_ABL_NOCOALESCE) || (I.variant && I.kind != WK_WPK1) ||
      I.nrows > 0x7fffffffu || I.nz > 0x7fffffffu || I.nwarps > 0x7fffffffu || I.allocate_nz > 0x7fffffffu) {
    std::fclose(f);
    return set_error(WK_ERR_INVALID, "%s is not a WPK layout file", path);
  }
  const bool k2 = I.kind == WK_WPK2;
  std::vector<int32_t> rm, rmi, wo, rp;
  std::vector<uint32_t> rr, mx, tpr, row;
  bool ok = get_array(f, rm, I.nrows) && get_array(f, rmi, I.nrows) && get_array(f, rr, I.nz) &&
            get_array(f, wo, (uint64_t)I.nwarps + 1) && get_array(f, mx, I.nwarps) &&
            get_array(f, tpr, k2 ? I.nwarps : 0) && get_array(f, row, k2 ? (uint64_t)I.nwarps + 1 : 0) &&
            get_array(f, rp, (uint64_t)I.nrows + 1);
  std::fclose(f);
  if (!ok) return set_error(WK_ERR_INVALID, "%s: truncated or inconsistent arrays", path);
  wk_layout *l = nullptr;
  WK_TRY(make_layout(rp.data(), I.nrows, I.nz, I.kind, k2 ? (int32_t)I.nmax_per_thread : 0,
                     (cudaStream_t)stream, &l, (int)I.variant));
  const wk_layout_info &B = l->info;
  ok = B.kind == I.kind && B.nrows == I.nrows && B.nznrows == I.nznrows && B.nz == I.nz &&
       B.allocate_nz == I.allocate_nz && B.nwarps == I.nwarps && B.min_nz == I.min_nz && B.max_nz == I.max_nz &&
       B.nmax_per_thread == I.nmax_per_thread && B.variant == I.variant;
  auto same = [&](const void *dev, const void *host, size_t bytes) {
    if (!ok || !bytes) return;
    std::vector<char> h(bytes);
    ok = cudaMemcpy(h.data(), dev, bytes, cudaMemcpyDeviceToHost) == cudaSuccess &&
         std::memcmp(h.data(), host, bytes) == 0;
  };
  same(l->d.row_map, rm.data(), rm.size() * 4);
  same(l->d.row_map_inv, rmi.data(), rmi.size() * 4);
  same(l->d.reorder_rows, rr.data(), rr.size() * 4);
  same(l->d.warp_offsets, wo.data(), wo.size() * 4);
  same(l->d.max_nz_rows, mx.data(), mx.size() * 4);
  if (k2) {
    same(l->d.threads_per_row, tpr.data(), tpr.size() * 4);
    same(l->d.row_offset_warp, row.data(), row.size() * 4);
  }
  if (!ok) {
    wk_layout_destroy(l);
    return set_error(WK_ERR_INVALID, "%s does not match a scan of its own row offsets", path);
  }
  *out = l;
  return WK_OK;
}

extern "C" wk_status wk_mm_read(const char *path, wk_csr **out) {
  if (!path || !out) return set_error(WK_ERR_INVALID, "NULL argument");
  *out = nullptr;
  wk_csr *c = new (std::nothrow) wk_csr();
  if (!c) return set_error(WK_ERR_ALLOC, "host allocation failed");
  wk_status s = read_mm(path, c);
  if (s != WK_OK) {
    delete c;
    return s;
  }
  *out = c;
  return WK_OK;
}

extern "C" wk_status wk_csr_get(const wk_csr *c, int64_t *nrows, int64_t *ncols, int64_t *nnz, const int32_t **rowptr,
                                const int32_t **cols, const double **vals) {
  if (!c) return set_error(WK_ERR_INVALID, "NULL argument");
  if (nrows) *nrows = c->nrows;
  if (ncols) *ncols = c->ncols;
  if (nnz) *nnz = (int64_t)c->cols.size();
  if (rowptr) *rowptr = c->rowptr.data();
  if (cols) *cols = c->cols.data();
  if (vals) *vals = c->vals.data();
  return WK_OK;
}

extern "C" wk_status wk_csr_free(wk_csr *c) {
  delete c;
  return WK_OK;
}
