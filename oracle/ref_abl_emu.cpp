/*
 * ref_abl_emu.cpp -- tail appended after optimization.cu lines 91-114 and
 * 144-442 when oracle/Makefile builds oracle/_ref/libwkref_abl.so.  TEST
 * INFRASTRUCTURE ONLY.  A C interface over the reference's scan,
 * scan_nosort, scan_nocoalesced and scan_nocoalesced_nosort, and a
 * thread-by-thread CPU run of warpKernel_nocoalesced (no cross-thread
 * interaction, so a sequential emulation is exact).
 */
emu_dim3 threadIdx, blockIdx, blockDim;

namespace {
struct abl {
  uint nz = 0, nrows = 0, nwarps = 0, allocate_nz = 0;
  std::vector<uint> reorder_rows, max_nz_rows;
  std::vector<int> warp_offsets, row_map, row_map_inv;
};
template <class T>
void put(const std::vector<T> &v, void *dst) {
  if (!v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
}
}  // namespace

extern "C" {

/* variant: 0 scan, 1 scan_nosort, 2 scan_nocoalesced, 3 scan_nocoalesced_nosort. */
void *ref_abl_scan(const int *rowptr, unsigned nrows, unsigned nz, int variant) {
  abl *h = new abl();
  h->nz = nz;
  h->nrows = nrows;
  int *rows = const_cast<int *>(rowptr);
  double *A = nullptr;
  int *cols = nullptr;
  uint nznrows = 0;
  switch (variant) {
    case 0:
      scan(h->nz, h->nrows, A, rows, cols, h->nwarps, h->allocate_nz, h->reorder_rows, h->warp_offsets,
           h->max_nz_rows, h->row_map, h->row_map_inv, nznrows);
      break;
    case 1:
      scan_nosort(h->nz, h->nrows, A, rows, cols, h->nwarps, h->allocate_nz, h->reorder_rows, h->warp_offsets,
                  h->max_nz_rows, h->row_map, h->row_map_inv);
      break;
    case 2:
      scan_nocoalesced(h->nz, h->nrows, A, rows, cols, h->nwarps, h->allocate_nz, h->reorder_rows,
                       h->warp_offsets, h->max_nz_rows, h->row_map, h->row_map_inv);
      break;
    default:
      scan_nocoalesced_nosort(h->nz, h->nrows, A, rows, cols, h->nwarps, h->allocate_nz, h->reorder_rows,
                              h->warp_offsets, h->max_nz_rows, h->row_map, h->row_map_inv);
  }
  return h;
}

void ref_abl_info(void *hp, unsigned *info) {
  abl *h = (abl *)hp;
  info[0] = h->nwarps;
  info[1] = h->allocate_nz;
}

/* field: 0 row_map, 1 row_map_inv, 2 reorder_rows, 3 warp_offsets, 4 max_nz_rows */
void ref_abl_field(void *hp, int field, void *dst) {
  abl *h = (abl *)hp;
  switch (field) {
    case 0: put(h->row_map, dst); break;
    case 1: put(h->row_map_inv, dst); break;
    case 2: put(h->reorder_rows, dst); break;
    case 3: put(h->warp_offsets, dst); break;
    default: put(h->max_nz_rows, dst); break;
  }
}

void ref_abl_free(void *hp) { delete (abl *)hp; }

/* warpKernel_nocoalesced<false> for every thread of a launch with `wpb` warps
 * per block, over `nrows` threads as optimization.cu:768-776 launches it;
 * pvals / pcols are the padded arrays of a non-interleaved layout. */
void ref_abl_run_nocoalesced(void *hp, const double *pvals, const int *pcols, const double *x, double *y, int wpb) {
  abl *h = (abl *)hp;
  unsigned nblocks = (h->nwarps + wpb - 1) / wpb;
  blockDim.x = 32 * wpb;
  for (unsigned b = 0; b < nblocks; b++) {
    blockIdx.x = b;
    for (unsigned t = 0; t < blockDim.x; t++) {
      threadIdx.x = t;
      warpKernel_nocoalesced<false, double, int>(h->nrows, const_cast<double *>(pvals), const_cast<int *>(pcols),
                                                 h->row_map.data(), h->max_nz_rows.data(), h->warp_offsets.data(),
                                                 const_cast<double *>(x), y);
    }
  }
}
}
