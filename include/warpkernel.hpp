/*
 * warpkernel.hpp -- drop-in C++ surface of the GB300-native WPK SpMV.
 *
 * Replaces thejonwong/warpkernel's header of the same name (the reference's
 * warpkernel.hpp:215-1022): classes warpkernel::structure, structure2,
 * engine<ValueType, IndexType>, profiler and stats keep their names, member
 * functions, argument meaning and public fields, so host code written
 * against the reference (its wpk1.cu / wpk2.cu drivers) compiles with the
 * container types swapped.  Everything runs through the C ABI of wk_capi.h:
 * the layout is built on the GPU by hand-written sm_103a kernels and copied
 * back into the public std::vector fields after each scan.
 *
 * Differences a user of the reference will notice:
 *  - no CUSP: scan / reorder_* accept any container with size(), operator[]
 *    (contiguous) and resize(); device vectors are warpkernel::device_array;
 *  - errors throw warpkernel::error instead of asserting or exiting;
 *  - run / run_x compute every row whatever the grid size (the reference's
 *    2-D grid for nblocks > 65535 skipped rows, warpkernel.hpp:818-826) and
 *    reject grids that do not cover all warps;
 *  - the `cache` template flag selects read-only non-coherent x gathers
 *    (true, the texture path) or plain L1-caching loads (false, the
 *    reference's x[i]); there are no texture references.
 *
 * Needs the CUDA runtime headers (cuda_runtime.h) and links against
 * libwarpkernel_gb300.so and the CUDA runtime.
 */
#ifndef WARP_KERNEL_GB300_HPP
#define WARP_KERNEL_GB300_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <iostream>
#include <limits>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "wk_capi.h"

#ifndef WARP_SIZE
#define WARP_SIZE 32
#endif

namespace warpkernel {

typedef unsigned int uint;

class error : public std::runtime_error {
 public:
  error(wk_status s, const std::string &m) : std::runtime_error(m), status(s) {}
  wk_status status;
};

inline void check(wk_status s) {
  if (s != WK_OK) {
    char buf[1024];
    wk_last_error(buf, sizeof buf);
    throw error(s, buf);
  }
}

template <typename T>
struct dtype_of;
template <>
struct dtype_of<double> {
  static const int value = WK_F64;
};
template <>
struct dtype_of<float> {
  static const int value = WK_F32;
};

/* Owning device vector (stands in for cusp::array1d<T, device_memory>). */
template <typename T>
class device_array {
 public:
  device_array() {}
  explicit device_array(size_t n, T v = T()) { assign(n, v); }
  template <class Host, class = typename std::enable_if<!std::is_arithmetic<Host>::value>::type>
  device_array(const Host &h) { *this = h; }
  device_array(const device_array &o) { copy_from_device(o.p_, o.n_); }
  ~device_array() { release(); }
  device_array &operator=(const device_array &o) {
    if (this != &o) copy_from_device(o.p_, o.n_);
    return *this;
  }
  template <class Host, class = typename std::enable_if<!std::is_arithmetic<Host>::value>::type>
  device_array &operator=(const Host &h) {
    resize(h.size());
    if (n_) check_cuda(cudaMemcpy(p_, &h[0], n_ * sizeof(T), cudaMemcpyHostToDevice));
    return *this;
  }
  void resize(size_t n) {
    if (n == n_) return;
    release();
    if (n) check_cuda(cudaMalloc(&p_, n * sizeof(T)));
    n_ = n;
  }
  void assign(size_t n, T v) {
    std::vector<T> h(n, v);
    *this = h;
  }
  std::vector<T> to_host() const {
    std::vector<T> h(n_);
    if (n_) check_cuda(cudaMemcpy(h.data(), p_, n_ * sizeof(T), cudaMemcpyDeviceToHost));
    return h;
  }
  operator std::vector<T>() const { return to_host(); }
  T *data() { return p_; }
  const T *data() const { return p_; }
  size_t size() const { return n_; }

 private:
  static void check_cuda(cudaError_t e) {
    if (e != cudaSuccess) throw error(WK_ERR_CUDA, cudaGetErrorString(e));
  }
  void copy_from_device(const T *src, size_t n) {
    resize(n);
    if (n) check_cuda(cudaMemcpy(p_, src, n * sizeof(T), cudaMemcpyDeviceToDevice));
  }
  void release() {
    if (p_) cudaFree(p_);
    p_ = nullptr;
    n_ = 0;
  }
  T *p_ = nullptr;
  size_t n_ = 0;
};

/* Host CSR matrix (stands in for cusp::csr_matrix<int, ValueType, host_memory>
 * with the same member names). */
template <typename IndexType, typename ValueType>
struct csr_matrix {
  uint num_rows = 0, num_cols = 0, num_entries = 0;
  std::vector<IndexType> row_offsets, column_indices;
  std::vector<ValueType> values;
};

/* cusp::io::read_matrix_market_file(A, filename) as the drivers call it
 * (wpk1.cu:43-48, wpk2.cu:54-57): coordinate real/integer/pattern files,
 * general / symmetric / skew-symmetric; entries sorted by row, then column. */
template <typename IndexType, typename ValueType>
void read_matrix_market_file(csr_matrix<IndexType, ValueType> &A, const char *filename) {
  static_assert(sizeof(IndexType) == 4, "32-bit indices expected");
  wk_csr *c = nullptr;
  check(wk_mm_read(filename, &c));
  int64_t n = 0, m = 0, z = 0;
  const int32_t *rp = nullptr, *ci = nullptr;
  const double *v = nullptr;
  wk_csr_get(c, &n, &m, &z, &rp, &ci, &v);
  A.num_rows = (uint)n;
  A.num_cols = (uint)m;
  A.num_entries = (uint)z;
  A.row_offsets.assign(rp, rp + n + 1);
  A.column_indices.assign(ci, ci + z);
  A.values.assign(v, v + z);
  wk_csr_free(c);
}

/* warpkernel::structure (reference warpkernel.hpp:215-551): WPK1 layout. */
class structure {
 public:
  structure() {}
  virtual ~structure() { release(); }
  structure(const structure &) = delete;
  structure &operator=(const structure &) = delete;

  std::vector<int> row_map;      // y[row_map[i]] = y'[i]
  std::vector<int> row_map_inv;  // new_colinds[n] = row_map_inv[colinds[n]]
  std::vector<uint> reorder_rows;  // new_values[reorder_rows[i]] = A[i]
  std::vector<int> reorder_A_rows;
  std::vector<int> warp_offsets;
  std::vector<uint> max_nz_rows;
  uint nrows = 0, nznrows = 0, nz = 0, allocate_nz = 0, nwarps = 0;
  uint variant = 0;  // WK_ABL_* flags of an ablation layout

  /* structure::scan (warpkernel.hpp:309-365): only `rows` is read. */
  template <typename ValueType, typename IndexType>
  void scan(uint &nz_, uint &nrows_, ValueType *A, IndexType *rows, IndexType *colinds) {
    static_assert(sizeof(IndexType) == 4, "32-bit row offsets expected");
    (void)A;
    (void)colinds;
    release();
    check(wk_scan1(reinterpret_cast<const int32_t *>(rows), nrows_, nz_, nullptr, &h_));
    fetch();
  }
  /* The WPK1 ablation layouts of optimization.cu: flags WK_ABL_NOSORT
   * (scan_nosort), WK_ABL_NOCOALESCE (scan_nocoalesced) or both
   * (scan_nocoalesced_nosort). */
  template <typename IndexType>
  void scan_ablation(uint &nz_, uint &nrows_, IndexType *rows, int flags) {
    static_assert(sizeof(IndexType) == 4, "32-bit row offsets expected");
    if (kind() != WK_WPK1) throw error(WK_ERR_INVALID, "the ablation layouts are WPK1 layouts");
    release();
    check(wk_scan1_ablation(reinterpret_cast<const int32_t *>(rows), nrows_, nz_, flags, nullptr, &h_));
    fetch();
  }
  /* scan of a CSR container with row_offsets / column_indices / values. */
  template <class CSR>
  void scan(uint &nz_, uint &nrows_, CSR &A) {
    scan(nz_, nrows_, &A.values[0], &A.row_offsets[0], &A.column_indices[0]);
  }

  /* reorder_columns_coalesced (warpkernel.hpp:447-457): padded, renumbered. */
  template <class Array>
  void reorder_columns_coalesced(Array &colinds) {
    std::vector<int32_t> out(allocate_nz);
    check(wk_reorder_columns_coalesced(h_, reinterpret_cast<const int32_t *>(&colinds[0]), out.data(), nullptr));
    colinds.resize(out.size());
    for (size_t i = 0; i < out.size(); i++) colinds[i] = out[i];
  }
  /* reorder_columns (warpkernel.hpp:401-412): renumbered, CSR order. */
  template <class Array>
  void reorder_columns(Array &colinds) {
    std::vector<int32_t> out(nz);
    check(wk_reorder_columns(h_, reinterpret_cast<const int32_t *>(&colinds[0]), out.data(), nullptr));
    for (size_t i = 0; i < out.size(); i++) colinds[i] = out[i];
  }
  /* reorder_columns_rowsort (warpkernel.hpp:414-444): renumbered columns
   * sorted within each CSR row; fills reorder_A_rows with their sources. */
  template <class Array, class Rows>
  void reorder_columns_rowsort(Array &colinds, Rows &rows) {
    (void)rows;  // the layout keeps its own copy of the row offsets
    std::vector<int32_t> out(nz);
    reorder_A_rows.resize(nz);
    check(wk_reorder_columns_rowsort(handle(), reinterpret_cast<const int32_t *>(&colinds[0]), out.data(),
                                     reorder_A_rows.data(), nullptr));
    for (size_t i = 0; i < out.size(); i++) colinds[i] = out[i];
  }
  /* reorder (warpkernel.hpp:380-398): the padded, interleaved values and
   * columns (padding 0), built on the GPU. */
  template <typename IndexType, typename ValueType>
  void reorder(ValueType *A, IndexType *colinds, device_array<ValueType> &device_values,
               device_array<IndexType> &device_colinds) {
    static_assert(sizeof(IndexType) == 4, "32-bit column indices expected");
    device_values.resize(allocate_nz);
    device_colinds.resize(allocate_nz);
    check(wk_process(handle(), dtype_of<ValueType>::value, A, reinterpret_cast<const int32_t *>(colinds),
                     device_values.data(), reinterpret_cast<int32_t *>(device_colinds.data()), nullptr));
  }
  /* process (warpkernel.hpp:533-548): reorder plus device copies of row_map,
   * max_nz_rows and warp_offsets. */
  template <typename IndexType, typename ValueType>
  void process(ValueType *A, IndexType *colinds, device_array<ValueType> &device_values,
               device_array<IndexType> &device_colinds, device_array<IndexType> &device_row_map,
               device_array<uint> &device_max_nz_per_row, device_array<IndexType> &device_warp_offsets) {
    reorder(A, colinds, device_values, device_colinds);
    device_row_map = row_map;
    device_max_nz_per_row = max_nz_rows;
    device_warp_offsets = warp_offsets;
  }
  /* reorder_values_coalesced (warpkernel.hpp:470-491): padded values only. */
  template <typename ValueType, typename Array>
  void reorder_values_coalesced(Array &values, device_array<ValueType> &dvalues) {
    dvalues.resize(allocate_nz);
    check(wk_process(handle(), dtype_of<ValueType>::value, &values[0], nullptr, dvalues.data(), nullptr, nullptr));
  }
  /* reorder_values_coalesced_GPU / reorder_columns_coalesced_GPU
   * (warpkernel.hpp:494-503, 459-468): the same scatter from device arrays;
   * the layout's own reorder_rows is used (the argument is accepted for the
   * reference's signature). */
  template <typename ValueType>
  void reorder_values_coalesced_GPU(device_array<ValueType> &values, device_array<ValueType> &dvalues,
                                    device_array<uint> &reorder_rows_) {
    (void)reorder_rows_;
    dvalues.resize(allocate_nz);
    check(wk_process(handle(), dtype_of<ValueType>::value, values.data(), nullptr, dvalues.data(), nullptr, nullptr));
  }
  template <typename IndexType>
  void reorder_columns_coalesced_GPU(device_array<IndexType> &values, device_array<IndexType> &dvalues,
                                     device_array<uint> &reorder_rows_) {
    static_assert(sizeof(IndexType) == 4, "32-bit column indices expected");
    (void)reorder_rows_;
    dvalues.resize(allocate_nz);
    check(wk_process(handle(), WK_F32, nullptr, reinterpret_cast<const int32_t *>(values.data()), nullptr,
                     reinterpret_cast<int32_t *>(dvalues.data()), nullptr));
  }

  /* reorder_values_coalesced_rowsort (warpkernel.hpp:505-515), [CPU] as in
   * the reference: dvalues[reorder_rows[i]] = values[reorder_A_rows[i]]. */
  template <class HostArray, typename T>
  void reorder_values_coalesced_rowsort(HostArray &values, device_array<T> &dvalues) {
    if (reorder_A_rows.size() != nz) throw error(WK_ERR_STATE, "reorder_columns_rowsort has not been called");
    std::vector<T> v(allocate_nz, T(0));
    for (uint i = 0; i < nz; i++) v[reorder_rows[i]] = values[reorder_A_rows[i]];
    dvalues = v;
  }
  /* Layout files (the fields of structure::serialize, warpkernel.hpp:253-269). */
  void save(const std::string &path) const { check(wk_layout_save(handle(), path.c_str())); }
  void load(const std::string &path) {
    wk_layout *l = nullptr;
    check(wk_layout_load(path.c_str(), nullptr, &l));
    wk_layout_info i;
    wk_layout_info_get(l, &i);
    if (i.kind != kind()) {
      wk_layout_destroy(l);
      throw error(WK_ERR_INVALID, path + " holds a layout of the other kind");
    }
    release();
    h_ = l;
    fetch();
  }

  /* reorder_x (warpkernel.hpp:518-530): device_x[row_map_inv[r]] = x[r]. */
  template <class HostArray, typename T>
  void reorder_x(HostArray &x, device_array<T> &device_x) {
    device_x.resize(nrows);
    check(wk_reorder_x(h_, dtype_of<T>::value, &x[0], device_x.data(), nullptr));
  }

  wk_layout *handle() const {
    if (!h_) throw error(WK_ERR_STATE, "structure has not been scanned");
    return h_;
  }

 protected:
  virtual int kind() const { return WK_WPK1; }
  void release() {
    if (h_) wk_layout_destroy(h_);
    h_ = nullptr;
  }
  template <typename T>
  void get(int field, std::vector<T> &v) {
    size_t n = 0;
    check(wk_layout_get(h_, field, nullptr, 0, &n));
    v.resize(n);
    if (n) check(wk_layout_get(h_, field, v.data(), n, nullptr));
  }
  virtual void fetch() {
    wk_layout_info i;
    check(wk_layout_info_get(h_, &i));
    nrows = i.nrows;
    nznrows = i.nznrows;
    nz = i.nz;
    allocate_nz = i.allocate_nz;
    nwarps = i.nwarps;
    variant = i.variant;
    get(WK_FIELD_ROW_MAP, row_map);
    get(WK_FIELD_ROW_MAP_INV, row_map_inv);
    get(WK_FIELD_REORDER_ROWS, reorder_rows);
    get(WK_FIELD_WARP_OFFSETS, warp_offsets);
    get(WK_FIELD_MAX_NZ_ROWS, max_nz_rows);
  }
  wk_layout *h_ = nullptr;
};

/* warpkernel::structure2 (reference warpkernel.hpp:553-771): WPK2 layout. */
class structure2 : public structure {
 public:
  std::vector<uint> row_offset_warp;
  std::vector<uint> threads_per_row;
  uint nmax_per_thread = 0;
  uint min_nz = 0, max_nz = 0;

  template <typename ValueType, typename IndexType>
  void scan(uint &nz_, uint &nrows_, ValueType *A, IndexType *rows, IndexType *colinds, IndexType threshold) {
    static_assert(sizeof(IndexType) == 4, "32-bit row offsets expected");
    (void)A;
    (void)colinds;
    release();
    check(wk_scan2(reinterpret_cast<const int32_t *>(rows), nrows_, nz_, (int32_t)threshold, nullptr, &h_));
    fetch();
  }
  template <class CSR, typename IndexType>
  void scan(uint &nz_, uint &nrows_, CSR &A, IndexType threshold) {
    scan(nz_, nrows_, &A.values[0], &A.row_offsets[0], &A.column_indices[0], threshold);
  }

  /* structure2::process (warpkernel.hpp:750-769): also threads_per_row and
   * row_offset_warp on the device. */
  template <typename IndexType, typename ValueType>
  void process(ValueType *A, IndexType *colinds, device_array<ValueType> &device_values,
               device_array<IndexType> &device_colinds, device_array<IndexType> &device_row_map,
               device_array<uint> &device_max_nz_per_row, device_array<IndexType> &device_warp_offsets,
               device_array<uint> &device_threads_per_row, device_array<uint> &device_row_offset_warp) {
    structure::process(A, colinds, device_values, device_colinds, device_row_map, device_max_nz_per_row,
                       device_warp_offsets);
    device_threads_per_row = threads_per_row;
    device_row_offset_warp = row_offset_warp;
  }

 protected:
  int kind() const override { return WK_WPK2; }
  void fetch() override {
    structure::fetch();
    wk_layout_info i;
    check(wk_layout_info_get(h_, &i));
    nmax_per_thread = i.nmax_per_thread;
    min_nz = i.min_nz;
    max_nz = i.max_nz;
    get(WK_FIELD_ROW_OFFSET_WARP, row_offset_warp);
    get(WK_FIELD_THREADS_PER_ROW, threads_per_row);
  }
};

/* warpkernel::engine (reference warpkernel.hpp:773-959). */
template <typename ValueType, typename IndexType>
class engine {
  static_assert(sizeof(IndexType) == 4, "32-bit column indices expected");

 public:
  /* engine.device_colinds: assignable from a host array of allocate_nz
   * padded column indices (wpk1.cu:175, 198), readable as a host vector. */
  class colinds_proxy {
   public:
    explicit colinds_proxy(engine *e) : e_(e) {}
    template <class Array>
    colinds_proxy &operator=(const Array &a) {
      check(wk_engine_set_colinds(e_->handle(), reinterpret_cast<const int32_t *>(&a[0]), nullptr));
      return *this;
    }
    colinds_proxy &operator=(const colinds_proxy &o) { return *this = o.to_host(); }
    std::vector<IndexType> to_host() const {
      std::vector<IndexType> v(e_->kernel->allocate_nz);
      check(wk_engine_get_colinds(e_->handle(), reinterpret_cast<int32_t *>(v.data()), v.size()));
      return v;
    }
    operator std::vector<IndexType>() const { return to_host(); }

   private:
    engine *e_;
  };
  colinds_proxy device_colinds{this};
  /* engine.device_values (warpkernel.hpp:782): readable as a host copy of the
   * allocate_nz padded values; set_values replaces them. */
  class values_proxy {
   public:
    explicit values_proxy(engine *e) : e_(e) {}
    std::vector<ValueType> to_host() const {
      std::vector<ValueType> v(e_->kernel->allocate_nz);
      check(wk_engine_get_values(e_->handle(), v.data(), v.size()));
      return v;
    }
    operator std::vector<ValueType>() const { return to_host(); }

   private:
    engine *e_;
  };
  values_proxy device_values{this};
  void set_values(const ValueType *A) { check(wk_engine_set_values(handle(), A, nullptr)); }

  explicit engine(structure &k) : kernel(&k) {}
  engine(structure &k, ValueType *A, IndexType *colinds) : kernel(&k) { create(A, colinds); }
  engine(structure2 &k, ValueType *A, IndexType *colinds) : kernel(&k) { create(A, colinds); }
  ~engine() {
    if (h_) wk_engine_destroy(h_);
  }
  engine(const engine &) = delete;
  engine &operator=(const engine &) = delete;

  /* run<cache>(nblocks, blocksize, dx, dy): y[row_map[p]] = row sums; returns
   * the kernel time in seconds (synchronous, like the reference). */
  template <bool cache>
  float run(int nblocks, int blocksize, ValueType *dx, ValueType *dy) {
    float s = 0.f;
    check(wk_run(handle(), nblocks, blocksize, cache ? 1 : 0, order, dx, dy, nullptr, &s));
    return s;
  }
  /* run_x<cache>(...): y'[p] = sorted-row sums with the reordered x. */
  template <bool cache>
  float run_x(int nblocks, int blocksize, ValueType *dx, ValueType *dy) {
    float s = 0.f;
    check(wk_run_x(handle(), nblocks, blocksize, cache ? 1 : 0, order, dx, dy, nullptr, &s));
    return s;
  }
  /* run_assembly<cache>(nblocks, blocksize, dy) (warpkernel.hpp:898-929):
   * y[row_map[p]] = sum of the stored values of row p. */
  template <bool cache>
  float run_assembly(int nblocks, int blocksize, ValueType *dy) {
    float s = 0.f;
    check(wk_run_assembly(handle(), nblocks, blocksize, dy, nullptr, &s));
    return s;
  }

  /* verify (warpkernel.hpp:932-943). */
  template <typename R>
  bool verify(R orig, R comp) {
    std::vector<double> o(kernel->nrows), c(kernel->nrows);
    for (uint i = 0; i < kernel->nrows; i++) {
      o[i] = (double)orig[i];
      c[i] = (double)comp[i];
    }
    int pass = 0;
    int64_t bad = -1;
    check(wk_verify(kernel->handle(), o.data(), c.data(), &pass, &bad));
    if (!pass)
      std::cout << "verify: " << o[bad] << "\t" << c[bad] << "\t" << bad << " "
                << std::fabs((o[bad] - c[bad]) / o[bad]) << std::endl;
    return pass != 0;
  }
  /* verify_x (warpkernel.hpp:945-957), with the reference's condition. */
  template <typename R>
  bool verify_x(R orig, R comp) {
    std::vector<double> o(kernel->nrows), c(kernel->nrows);
    for (uint i = 0; i < kernel->nrows; i++) {
      o[i] = (double)orig[i];
      c[i] = (double)comp[i];
    }
    int pass = 0;
    int64_t bad = -1;
    check(wk_verify_x(kernel->handle(), o.data(), c.data(), 0, &pass, &bad));
    if (!pass) std::cout << "verify_x: " << o[kernel->row_map[bad]] << "\t" << c[bad] << "\t" << bad << std::endl;
    return pass != 0;
  }

  wk_engine *handle() const {
    if (!h_) throw error(WK_ERR_STATE, "engine was constructed without values");
    return h_;
  }

  /* WK_ORDER_FAST (default) or WK_ORDER_EXACT (the reference's order). */
  int order = WK_ORDER_FAST;
  structure *kernel;

 private:
  void create(ValueType *A, IndexType *colinds) {
    check(wk_engine_create(kernel->handle(), dtype_of<ValueType>::value, A,
                           reinterpret_cast<const int32_t *>(colinds), kernel->nrows, nullptr, &h_));
  }
  wk_engine *h_ = nullptr;
};

/* profiler (warpkernel.hpp:963-982). */
class profiler {
 public:
  double sum = 0.0;
  int count = 0;
  void add(double secs) {
    sum += secs;
    count++;
  }
  double avg() { return sum / (1. * count); }
};

/* stats (warpkernel.hpp:984-1022). */
class stats {
 public:
  stats() : min_(std::numeric_limits<double>::max()), max_(0.) {}
  void add(double val, std::string ident = "") {
    if (val < min_) {
      min_ = val;
      min_str_ = ident;
    }
    if (val > max_) {
      max_ = val;
      max_str_ = ident;
    }
  }
  double Min() { return min_; }
  std::string Min_str() { return min_str_; }
  double Max() { return max_; }
  std::string Max_str() { return max_str_; }

 protected:
  double min_, max_;
  std::string min_str_, max_str_;
};

}  // namespace warpkernel

#endif
