/*
 * ref_emu.cpp -- tail appended after warpkernel.hpp lines 27-771 when
 * oracle/Makefile builds oracle/_ref/libwkref*.so.  TEST INFRASTRUCTURE ONLY.
 *
 * It closes the reference's `namespace warpkernel` (the engine class that
 * follows line 771 uses CUDA launch syntax and is not compiled) and exposes a
 * small C interface over the reference's own structure / structure2 classes
 * and its WPK1 kernels, which it runs on the CPU thread by thread (they have
 * no cross-thread interaction, so a sequential emulation is exact).
 */
}  // namespace warpkernel

emu_dim3 threadIdx, blockIdx, blockDim;

namespace {
struct handle {
  warpkernel::structure *s;
  warpkernel::structure2 *s2;
  int kind;
  warpkernel::structure *base() { return kind == 2 ? s2 : s; }
};
template <class T>
void copy_out(const std::vector<T> &v, void *dst) {
  if (!v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
}
}  // namespace

extern "C" {

void *ref_scan(const int *rowptr, unsigned nrows, unsigned nz, int kind, int threshold) {
  handle *h = new handle{nullptr, nullptr, kind};
  unsigned nz_ = nz, n_ = nrows;
  int *rows = const_cast<int *>(rowptr);
  if (kind == 1) {
    h->s = new warpkernel::structure();
    h->s->scan(nz_, n_, (double *)nullptr, rows, (int *)nullptr);
  } else {
    h->s2 = new warpkernel::structure2();
    h->s2->scan(nz_, n_, (double *)nullptr, rows, (int *)nullptr, threshold);
  }
  return h;
}

void ref_free(void *hp) {
  handle *h = (handle *)hp;
  delete h->s;
  delete h->s2;
  delete h;
}

/* info[0..7] = nrows, nznrows, nz, allocate_nz, nwarps, min_nz, max_nz, nmax_per_thread */
void ref_info(void *hp, unsigned *info) {
  handle *h = (handle *)hp;
  warpkernel::structure *s = h->base();
  info[0] = s->nrows; info[1] = s->nznrows; info[2] = s->nz; info[3] = s->allocate_nz;
  info[4] = s->nwarps;
  info[5] = h->kind == 2 ? h->s2->min_nz : 0;
  info[6] = h->kind == 2 ? h->s2->max_nz : 0;
  info[7] = h->kind == 2 ? h->s2->nmax_per_thread : 0;
}

/* field: 0 row_map, 1 row_map_inv, 2 reorder_rows, 3 warp_offsets, 4 max_nz_rows,
 * 5 threads_per_row, 6 row_offset_warp.  Returns the element count. */
long ref_field(void *hp, int field, void *dst) {
  handle *h = (handle *)hp;
  warpkernel::structure *s = h->base();
  switch (field) {
    case 0: if (dst) copy_out(s->row_map, dst); return (long)s->row_map.size();
    case 1: if (dst) copy_out(s->row_map_inv, dst); return (long)s->row_map_inv.size();
    case 2: if (dst) copy_out(s->reorder_rows, dst); return (long)s->reorder_rows.size();
    case 3: if (dst) copy_out(s->warp_offsets, dst); return (long)s->warp_offsets.size();
    case 4: if (dst) copy_out(s->max_nz_rows, dst); return (long)s->max_nz_rows.size();
    case 5: if (h->kind != 2) return 0; if (dst) copy_out(h->s2->threads_per_row, dst);
            return (long)h->s2->threads_per_row.size();
    case 6: if (h->kind != 2) return 0; if (dst) copy_out(h->s2->row_offset_warp, dst);
            return (long)h->s2->row_offset_warp.size();
  }
  return -1;
}

/* structure::process / structure2::process with host stand-ins for the
 * device arrays; pvals/pcols receive allocate_nz entries. */
void ref_process(void *hp, const double *vals, const int *cols, double *pvals, int *pcols) {
  handle *h = (handle *)hp;
  typedef warpkernel::DeviceSpace D;
  cusp::array1d<double, D> dv;
  cusp::array1d<int, D> dc, drm, dwo;
  cusp::array1d<uint, D> dmx, dtpr, drow;
  double *A = const_cast<double *>(vals);
  int *C = const_cast<int *>(cols);
  if (h->kind == 1)
    h->s->process(A, C, dv, dc, drm, dmx, dwo);
  else
    h->s2->process(A, C, dv, dc, drm, dmx, dwo, dtpr, drow);
  copy_out(dv, pvals);
  copy_out(dc, pcols);
}

void ref_reorder_columns_coalesced(void *hp, const int *cols, unsigned nz, int *out) {
  handle *h = (handle *)hp;
  cusp::array1d<int, warpkernel::CPUSpace> c(cols, cols + nz);
  h->base()->reorder_columns_coalesced(c);
  copy_out(c, out);
}

void ref_reorder_x(void *hp, const double *x, unsigned n, double *out) {
  handle *h = (handle *)hp;
  cusp::array1d<double, warpkernel::CPUSpace> xx(x, x + n);
  cusp::array1d<double, warpkernel::DeviceSpace> dx;
  h->base()->reorder_x(xx, dx);
  copy_out(dx, out);
}

/* Runs warpKernel (mapped = 1) or warpKernel_reorderx (mapped = 0) for every
 * thread of a launch with `wpb` warps per block, as engine::run/run_x would
 * launch it (warpkernel.hpp:847-855, 884-891) with cache = false. */
void ref_run_wpk1(void *hp, const double *pvals, const int *pcols, const double *x, double *y,
                  int mapped, int wpb) {
  handle *h = (handle *)hp;
  warpkernel::structure *s = h->base();
  unsigned nblocks = (s->nwarps + wpb - 1) / wpb;
  blockDim.x = 32 * wpb;
  double *A = const_cast<double *>(pvals);
  int *C = const_cast<int *>(pcols);
  double *X = const_cast<double *>(x);
  for (unsigned b = 0; b < nblocks; b++) {
    blockIdx.x = b;
    for (unsigned t = 0; t < blockDim.x; t++) {
      threadIdx.x = t;
      if (mapped)
        warpkernel::warpKernel<false, double, int>(s->nznrows, A, C, s->row_map.data(),
                                                   s->max_nz_rows.data(), s->warp_offsets.data(), X, y);
      else
        warpkernel::warpKernel_reorderx<false, double, int>((int)s->nznrows, A, C, s->max_nz_rows.data(),
                                                            s->warp_offsets.data(), X, y);
    }
  }
}

/* The reference's structure::reorder_columns_rowsort (warpkernel.hpp:414-444):
 * out_cols = the reordered colinds, out_src = its reorder_A_rows. */
void ref_reorder_columns_rowsort(void *hp, const int *cols, const int *rowptr, unsigned nz, unsigned nrows,
                                 int *out_cols, int *out_src) {
  handle *h = (handle *)hp;
  cusp::array1d<int, warpkernel::CPUSpace> c(cols, cols + nz);
  cusp::array1d<int, warpkernel::CPUSpace> rows(rowptr, rowptr + nrows + 1);
  h->base()->reorder_columns_rowsort(c, rows);
  copy_out(c, out_cols);
  copy_out(h->base()->reorder_A_rows, out_src);
}

/* warpKernel_assembly (warpkernel.hpp:78-100) for every thread of a WPK1
 * launch with `wpb` warps per block, with the argument list the kernel
 * declares (engine::run_assembly, warpkernel.hpp:913-921, passes one fewer
 * and is not compiled). */
void ref_assembly_wpk1(void *hp, const double *pvals, double *y, int wpb) {
  handle *h = (handle *)hp;
  warpkernel::structure *s = h->base();
  unsigned nblocks = (s->nwarps + wpb - 1) / wpb;
  blockDim.x = 32 * wpb;
  double *A = const_cast<double *>(pvals);
  for (unsigned b = 0; b < nblocks; b++) {
    blockIdx.x = b;
    for (unsigned t = 0; t < blockDim.x; t++) {
      threadIdx.x = t;
      warpkernel::warpKernel_assembly<false, double, int>(s->nznrows, A, s->row_map.data(), s->max_nz_rows.data(),
                                                          s->warp_offsets.data(), y);
    }
  }
}

/* engine::verify / verify_x are members of the engine class, which is not
 * compiled; the oracle restates them (wk_oracle.c). */
}
