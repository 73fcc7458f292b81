/*
 * wk_oracle.c -- CPU oracle for the WPK1/WPK2 SpMV path (see wk_oracle.h).
 *
 * TEST INFRASTRUCTURE ONLY: a restatement of warpkernel.hpp's host scan,
 * process and kernel arithmetic in plain C.  Each function cites the lines it
 * follows.  Compiled with -ffp-contract=off so that "separate multiply and add"
 * really is separate, and fma() is called explicitly where contraction is wanted.
 */
#include "wk_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define WS 32u /* WARP_SIZE */

typedef struct {
  uint32_t row, len;
} pair_t;

/* warpkernel.hpp:222-225 checkPairOrder: longer rows first, then the lower
 * row index first.  A strict total order, so any correct sort gives the same
 * permutation as the reference's std::sort (warpkernel.hpp:249). */
static int cmp_pair(const void *a, const void *b) {
  const pair_t *p = (const pair_t *)a, *q = (const pair_t *)b;
  if (p->len != q->len) return p->len > q->len ? -1 : 1;
  return (p->row > q->row) - (p->row < q->row);
}

static int check_csr(const int32_t *rowptr, uint32_t nrows, uint32_t nz) {
  if (rowptr[0] != 0) return 1;
  for (uint32_t r = 0; r < nrows; r++)
    if (rowptr[r + 1] < rowptr[r]) return 2;
  if ((uint32_t)rowptr[nrows] != nz) return 3;
  return 0;
}

/* structure::sort + storemap (warpkernel.hpp:232-250, 288-296). */
static pair_t *sort_rows(const int32_t *rowptr, wko_layout *l) {
  uint32_t n = l->nrows;
  pair_t *nnz_r = (pair_t *)malloc((size_t)(n ? n : 1) * sizeof(pair_t));
  l->row_map = (int32_t *)malloc((size_t)(n ? n : 1) * sizeof(int32_t));
  l->row_map_inv = (int32_t *)malloc((size_t)(n ? n : 1) * sizeof(int32_t));
  if (!nnz_r || !l->row_map || !l->row_map_inv) {
    free(nnz_r);
    return NULL;
  }
  l->nznrows = 0;
  for (uint32_t r = 0; r < n; r++) {
    uint32_t len = (uint32_t)(rowptr[r + 1] - rowptr[r]);
    nnz_r[r].row = r;
    nnz_r[r].len = len;
    if (len > 0) l->nznrows++;
  }
  qsort(nnz_r, n, sizeof(pair_t), cmp_pair);
  for (uint32_t p = 0; p < n; p++) {
    l->row_map[p] = (int32_t)nnz_r[p].row;
    l->row_map_inv[nnz_r[p].row] = (int32_t)p;
  }
  return nnz_r;
}

/* structure::scan, WPK1 (warpkernel.hpp:309-365). */
int wko_scan1(const int32_t *rowptr, uint32_t nrows, uint32_t nz, wko_layout *l) {
  memset(l, 0, sizeof(*l));
  l->kind = 1;
  l->nrows = nrows;
  l->nz = nz;
  if (check_csr(rowptr, nrows, nz)) return 1;
  pair_t *nnz_r = sort_rows(rowptr, l);
  if (!nnz_r) return 2;

  uint32_t W = (l->nznrows + WS - 1) / WS;
  l->nwarps = W;
  l->max_nz_rows = (uint32_t *)calloc(W ? W : 1, sizeof(uint32_t));
  l->warp_offsets = (int32_t *)calloc(W + 1, sizeof(int32_t));
  l->reorder_rows = (uint32_t *)calloc(nz ? nz : 1, sizeof(uint32_t));
  if (!l->max_nz_rows || !l->warp_offsets || !l->reorder_rows) {
    free(nnz_r);
    return 2;
  }
  for (uint32_t w = 0; w < W; w++) {
    uint32_t mx = 0;
    for (uint32_t r = WS * w; r < l->nznrows && r < WS * (w + 1); r++)
      if (nnz_r[r].len > mx) mx = nnz_r[r].len;
    l->max_nz_rows[w] = mx;
  }
  l->warp_offsets[0] = 0;
  for (uint32_t w = 0; w < W; w++)
    l->warp_offsets[w + 1] = (int32_t)((uint32_t)l->warp_offsets[w] + l->max_nz_rows[w] * WS);
  l->allocate_nz = (uint32_t)l->warp_offsets[W];

  for (uint32_t w = 0; w < W; w++) {
    for (uint32_t rs = WS * w; rs < l->nznrows && rs < WS * (w + 1); rs++) {
      uint32_t r = nnz_r[rs].row, len = nnz_r[rs].len;
      for (uint32_t i = 0; i < len; i++)
        l->reorder_rows[rowptr[r] + i] =
            (uint32_t)(l->warp_offsets[w] + (int32_t)(rs % WS) + (int32_t)(i * WS));
    }
  }
  free(nnz_r);
  return 0;
}

/* The row order of optimization.cu's nosort scans (311-318, 385-392): rows
 * with entries in CSR order, then the empty rows in CSR order. */
static pair_t *unsorted_rows(const int32_t *rowptr, wko_layout *l) {
  uint32_t n = l->nrows;
  pair_t *nnz_r = (pair_t *)malloc((size_t)(n ? n : 1) * sizeof(pair_t));
  l->row_map = (int32_t *)malloc((size_t)(n ? n : 1) * sizeof(int32_t));
  l->row_map_inv = (int32_t *)malloc((size_t)(n ? n : 1) * sizeof(int32_t));
  if (!nnz_r || !l->row_map || !l->row_map_inv) {
    free(nnz_r);
    return NULL;
  }
  uint32_t p = 0;
  for (int pass = 0; pass < 2; pass++)
    for (uint32_t r = 0; r < n; r++) {
      uint32_t len = (uint32_t)(rowptr[r + 1] - rowptr[r]);
      if ((len > 0) != (pass == 0)) continue;
      nnz_r[p].row = r;
      nnz_r[p].len = len;
      p++;
    }
  l->nznrows = 0;
  for (uint32_t q = 0; q < n; q++) {
    if (nnz_r[q].len > 0) l->nznrows++;
    l->row_map[q] = (int32_t)nnz_r[q].row;
    l->row_map_inv[nnz_r[q].row] = (int32_t)q;
  }
  return nnz_r;
}

/* optimization.cu scan_nosort / scan_nocoalesced / scan_nocoalesced_nosort:
 * the warp tables of structure::scan over the chosen row order; entry i of
 * the row in lane l of warp w goes to o_w + l + 32 i (interleaved) or to
 * o_w + l * A_w + i (optimization.cu:289-290, 363-364, 437-438). */
int wko_scan1_ablation(const int32_t *rowptr, uint32_t nrows, uint32_t nz, int flags, wko_layout *l) {
  memset(l, 0, sizeof(*l));
  l->kind = 1;
  l->nrows = nrows;
  l->nz = nz;
  l->variant = (uint32_t)flags;
  if (flags & ~(WKO_ABL_NOSORT | WKO_ABL_NOCOALESCE)) return 1;
  if (check_csr(rowptr, nrows, nz)) return 1;
  pair_t *nnz_r = (flags & WKO_ABL_NOSORT) ? unsorted_rows(rowptr, l) : sort_rows(rowptr, l);
  if (!nnz_r) return 2;
  uint32_t W = (l->nznrows + WS - 1) / WS;
  l->nwarps = W;
  l->max_nz_rows = (uint32_t *)calloc(W ? W : 1, sizeof(uint32_t));
  l->warp_offsets = (int32_t *)calloc(W + 1, sizeof(int32_t));
  l->reorder_rows = (uint32_t *)calloc(nz ? nz : 1, sizeof(uint32_t));
  if (!l->max_nz_rows || !l->warp_offsets || !l->reorder_rows) {
    free(nnz_r);
    return 2;
  }
  for (uint32_t w = 0; w < W; w++) {
    uint32_t mx = 0;
    for (uint32_t r = WS * w; r < l->nznrows && r < WS * (w + 1); r++)
      if (nnz_r[r].len > mx) mx = nnz_r[r].len;
    l->max_nz_rows[w] = mx;
  }
  for (uint32_t w = 0; w < W; w++)
    l->warp_offsets[w + 1] = (int32_t)((uint32_t)l->warp_offsets[w] + l->max_nz_rows[w] * WS);
  l->allocate_nz = (uint32_t)l->warp_offsets[W];
  for (uint32_t w = 0; w < W; w++)
    for (uint32_t rs = WS * w; rs < l->nznrows && rs < WS * (w + 1); rs++) {
      uint32_t r = nnz_r[rs].row, len = nnz_r[rs].len, lane = rs % WS;
      for (uint32_t i = 0; i < len; i++)
        l->reorder_rows[rowptr[r] + i] = (flags & WKO_ABL_NOCOALESCE)
                                             ? (uint32_t)l->warp_offsets[w] + lane * l->max_nz_rows[w] + i
                                             : (uint32_t)l->warp_offsets[w] + lane + i * WS;
    }
  free(nnz_r);
  return 0;
}

/* structure2::scan, WPK2 (warpkernel.hpp:579-736).  The reference splits
 * warps by inserting copies in front of the current element of three
 * std::vectors (633-691); the copies are identical, so appending them in
 * order gives the same sequence.  The "partial last warp" branch (660-663)
 * keeps the real row count and emits one warp. */
int wko_scan2(const int32_t *rowptr, uint32_t nrows, uint32_t nz, int32_t threshold,
              wko_layout *l) {
  memset(l, 0, sizeof(*l));
  l->kind = 2;
  l->nrows = nrows;
  l->nz = nz;
  l->nmax_per_thread = (uint32_t)threshold;
  if (check_csr(rowptr, nrows, nz)) return 1;
  pair_t *nnz_r = sort_rows(rowptr, l);
  if (!nnz_r) return 2;

  const uint32_t th = (uint32_t)threshold;
  uint32_t W0 = (l->nznrows + WS - 1) / WS;
  l->min_nz = nrows;
  l->max_nz = 0;
  /* Worst case every warp splits into 32. */
  size_t cap = (size_t)W0 * WS + 1;
  uint32_t *A_w = (uint32_t *)malloc(cap * sizeof(uint32_t));
  uint32_t *rpw = (uint32_t *)malloc(cap * sizeof(uint32_t));
  uint32_t *rows_w = (uint32_t *)malloc(cap * sizeof(uint32_t));
  if (!A_w || !rpw || !rows_w) {
    free(nnz_r); free(A_w); free(rpw); free(rows_w);
    return 2;
  }
  uint32_t W = 0;
  for (uint32_t w = 0; w < W0; w++) {
    uint32_t mx = 0, cnt = 0;
    for (uint32_t r = WS * w; r < l->nznrows && r < WS * (w + 1); r++) {
      uint32_t len = nnz_r[r].len;
      if (len > mx) mx = len;
      cnt++;
      if (len > 0) {
        l->min_nz = len < l->min_nz ? len : l->min_nz;
        l->max_nz = len > l->max_nz ? len : l->max_nz;
      }
    }
    int emitted = 0;
    if (mx > th) {
      const int32_t thmax_per_row = 32;
      int32_t nmax_per_warp = (int32_t)th;
      if (mx > th * (uint32_t)thmax_per_row)
        nmax_per_warp = (int32_t)((mx + (uint32_t)thmax_per_row - 1) / (uint32_t)thmax_per_row);
      for (int32_t i = 2; i <= thmax_per_row; i *= 2) {
        if (mx <= (uint32_t)nmax_per_warp * (uint32_t)i) {
          uint32_t nzpt = (mx + (uint32_t)i - 1) / (uint32_t)i;
          if (cnt * (uint32_t)i < WS) { /* partial: only the last warp */
            A_w[W] = nzpt; rpw[W] = WS / (uint32_t)i; rows_w[W] = cnt; W++;
          } else {
            for (int32_t j = 0; j < i; j++) {
              A_w[W] = nzpt; rpw[W] = WS / (uint32_t)i; rows_w[W] = WS / (uint32_t)i; W++;
            }
          }
          emitted = 1;
          break;
        }
      }
    }
    if (!emitted) {
      A_w[W] = mx; rpw[W] = WS; rows_w[W] = cnt; W++;
    }
  }
  l->nwarps = W;
  l->max_nz_rows = A_w;
  l->warp_offsets = (int32_t *)calloc(W + 1, sizeof(int32_t));
  l->threads_per_row = (uint32_t *)calloc(W ? W : 1, sizeof(uint32_t));
  l->row_offset_warp = (uint32_t *)calloc(W + 1, sizeof(uint32_t));
  l->reorder_rows = (uint32_t *)calloc(nz ? nz : 1, sizeof(uint32_t));
  if (!l->warp_offsets || !l->threads_per_row || !l->row_offset_warp || !l->reorder_rows) {
    free(nnz_r); free(rpw); free(rows_w);
    return 2;
  }
  for (uint32_t w = 0; w < W; w++)
    l->warp_offsets[w + 1] = (int32_t)((uint32_t)l->warp_offsets[w] + A_w[w] * WS);
  l->allocate_nz = (uint32_t)l->warp_offsets[W];
  for (uint32_t w = 0; w < W; w++) l->threads_per_row[w] = WS / rpw[w];
  for (uint32_t w = 0; w < W; w++) l->row_offset_warp[w + 1] = l->row_offset_warp[w] + rows_w[w];
  l->row_offset_warp[W] = nrows; /* warpkernel.hpp:716 */

  for (uint32_t ws = 0; ws < W; ws++) {
    uint32_t tpr = l->threads_per_row[ws], A = A_w[ws];
    for (uint32_t r = 0; r < rpw[ws] && l->row_offset_warp[ws] + r < l->nznrows; r++) {
      uint32_t rs = l->row_offset_warp[ws] + r;
      uint32_t row = nnz_r[rs].row, len = nnz_r[rs].len;
      for (uint32_t t = 0; t < tpr; t++)
        for (uint32_t i = 0; i + t * A < len && i < A; i++)
          l->reorder_rows[rowptr[row] + i + t * A] =
              (uint32_t)(l->warp_offsets[ws] + (int32_t)(t + r * tpr) + (int32_t)(i * WS));
    }
  }
  free(nnz_r); free(rpw); free(rows_w);
  return 0;
}

void wko_free(wko_layout *l) {
  free(l->row_map); free(l->row_map_inv); free(l->reorder_rows); free(l->warp_offsets);
  free(l->max_nz_rows); free(l->threads_per_row); free(l->row_offset_warp);
  memset(l, 0, sizeof(*l));
}

/* structure::reorder (warpkernel.hpp:380-398). */
void wko_process_f64(const wko_layout *l, const double *vals, const int32_t *cols,
                     double *pvals, int32_t *pcols) {
  memset(pvals, 0, (size_t)l->allocate_nz * sizeof(double));
  memset(pcols, 0, (size_t)l->allocate_nz * sizeof(int32_t));
  for (uint32_t i = 0; i < l->nz; i++) {
    pvals[l->reorder_rows[i]] = vals[i];
    pcols[l->reorder_rows[i]] = cols[i];
  }
}

void wko_process_f32(const wko_layout *l, const float *vals, const int32_t *cols,
                     float *pvals, int32_t *pcols) {
  memset(pvals, 0, (size_t)l->allocate_nz * sizeof(float));
  memset(pcols, 0, (size_t)l->allocate_nz * sizeof(int32_t));
  for (uint32_t i = 0; i < l->nz; i++) {
    pvals[l->reorder_rows[i]] = vals[i];
    pcols[l->reorder_rows[i]] = cols[i];
  }
}

/* warpkernel.hpp:447-457. */
void wko_reorder_columns_coalesced(const wko_layout *l, const int32_t *cols, int32_t *out) {
  memset(out, 0, (size_t)l->allocate_nz * sizeof(int32_t));
  for (uint32_t i = 0; i < l->nz; i++) out[l->reorder_rows[i]] = l->row_map_inv[cols[i]];
}

/* warpkernel.hpp:401-412. */
void wko_reorder_columns(const wko_layout *l, const int32_t *cols, int32_t *out) {
  for (uint32_t n = 0; n < l->nz; n++) out[n] = l->row_map_inv[cols[n]];
}

/* warpkernel.hpp:518-530. */
void wko_reorder_x_f64(const wko_layout *l, const double *x, double *xout) {
  for (uint32_t r = 0; r < l->nrows; r++) xout[l->row_map_inv[r]] = x[r];
}

/* One lane's partial sum: first product, then sum += a*x per step of 32
 * (warpkernel.hpp:65-71, 147-153). */
static double lane_sum(const double *A, const int32_t *c, const double *x, int32_t toffset,
                       uint32_t maxrows, int fma_mode) {
  uint32_t maxnz = maxrows * WS + (uint32_t)toffset;
  double sum = A[toffset] * x[c[toffset]];
  for (toffset += (int32_t)WS; (uint32_t)toffset < maxnz; toffset += (int32_t)WS) {
    if (fma_mode)
      sum = fma(A[toffset], x[c[toffset]], sum);
    else
      sum = sum + A[toffset] * x[c[toffset]];
  }
  return sum;
}

/* WPK2 warp: lane partials, then the shared-memory tree of
 * warpkernel.hpp:154-162.  Under lockstep execution every lane reads its
 * neighbour's value from the previous round before anyone writes, so the
 * leader's result is the pairwise tree ((s0+s1)+(s2+s3))+... -- exactly the
 * order of __shfl_down_sync with offsets 1, 2, 4, ... */
static void wpk2_warp(const wko_layout *l, uint32_t w, const double *A, const int32_t *c,
                      const double *x, double *y, int mapped, int fma_mode) {
  uint32_t T = l->threads_per_row[w];
  uint32_t row_start = l->row_offset_warp[w];
  double s[32];
  for (uint32_t lane = 0; lane < WS; lane++) {
    uint32_t rowid = row_start + lane / T;
    s[lane] = 0.0;
    if (rowid < l->nznrows)
      s[lane] = lane_sum(A, c, x, l->warp_offsets[w] + (int32_t)lane, l->max_nz_rows[w], fma_mode);
  }
  for (uint32_t lead = 0; lead < WS; lead += T) {
    uint32_t rowid = row_start + lead / T;
    if (rowid >= l->nznrows) continue;
    double t[32];
    for (uint32_t k = 0; k < T; k++) t[k] = s[lead + k];
    for (uint32_t i = 1; i < T; i <<= 1)
      for (uint32_t k = 0; k + i < T; k += 2 * i) t[k] = t[k] + t[k + i];
    if (mapped)
      y[l->row_map[rowid]] = t[0];
    else
      y[rowid] = t[0];
  }
}

/* warpKernel_nocoalesced (optimization.cu:91-114): the lane's entries are
 * contiguous. */
static double lane_sum_nc(const double *A, const int32_t *c, const double *x, int32_t toffset,
                          uint32_t maxrows, int fma_mode) {
  int32_t end = toffset + (int32_t)maxrows;
  double sum = A[toffset] * x[c[toffset]];
  for (toffset++; toffset < end; toffset++) {
    if (fma_mode)
      sum = fma(A[toffset], x[c[toffset]], sum);
    else
      sum = sum + A[toffset] * x[c[toffset]];
  }
  return sum;
}

static void run_any(const wko_layout *l, const double *A, const int32_t *c, const double *x,
                    double *y, int mapped, int fma_mode) {
  if (l->kind == 1 && (l->variant & WKO_ABL_NOCOALESCE)) {
    for (uint32_t id = 0; id < l->nznrows; id++) {
      uint32_t w = id / WS, lane = id % WS;
      double sum = lane_sum_nc(A, c, x, l->warp_offsets[w] + (int32_t)(lane * l->max_nz_rows[w]),
                               l->max_nz_rows[w], fma_mode);
      if (mapped)
        y[l->row_map[id]] = sum;
      else
        y[id] = sum;
    }
    return;
  }
  if (l->kind == 1) {
    for (uint32_t id = 0; id < l->nznrows; id++) {
      uint32_t w = id / WS, lane = id % WS;
      double sum = lane_sum(A, c, x, l->warp_offsets[w] + (int32_t)lane, l->max_nz_rows[w], fma_mode);
      if (mapped)
        y[l->row_map[id]] = sum;
      else
        y[id] = sum;
    }
  } else {
    for (uint32_t w = 0; w < l->nwarps; w++) wpk2_warp(l, w, A, c, x, y, mapped, fma_mode);
  }
}

/* warpKernel_assembly (warpkernel.hpp:78-100): the lane's slot values
 * summed in slot order. */
static double lane_asum(const double *A, int32_t toffset, uint32_t maxrows) {
  uint32_t maxnz = maxrows * WS + (uint32_t)toffset;
  double sum = A[toffset];
  for (toffset += (int32_t)WS; (uint32_t)toffset < maxnz; toffset += (int32_t)WS) sum = sum + A[toffset];
  return sum;
}

void wko_assembly_f64(const wko_layout *l, const double *pvals, double *y) {
  if (l->kind == 1) {
    for (uint32_t id = 0; id < l->nznrows; id++) {
      uint32_t w = id / WS, lane = id % WS;
      y[l->row_map[id]] = lane_asum(pvals, l->warp_offsets[w] + (int32_t)lane, l->max_nz_rows[w]);
    }
    return;
  }
  for (uint32_t w = 0; w < l->nwarps; w++) {
    uint32_t T = l->threads_per_row[w], row_start = l->row_offset_warp[w];
    double s[32];
    for (uint32_t lane = 0; lane < WS; lane++)
      s[lane] = row_start + lane / T < l->nznrows
                    ? lane_asum(pvals, l->warp_offsets[w] + (int32_t)lane, l->max_nz_rows[w])
                    : 0.0;
    for (uint32_t lead = 0; lead < WS; lead += T) {
      uint32_t rowid = row_start + lead / T;
      if (rowid >= l->nznrows) continue;
      double t[32];
      for (uint32_t k = 0; k < T; k++) t[k] = s[lead + k];
      for (uint32_t i = 1; i < T; i <<= 1)
        for (uint32_t k = 0; k + i < T; k += 2 * i) t[k] = t[k] + t[k + i];
      y[l->row_map[rowid]] = t[0];
    }
  }
}

typedef struct {
  int32_t col, src;
} rs_pair;

static int rs_cmp(const void *a, const void *b) {
  const rs_pair *x = (const rs_pair *)a, *y = (const rs_pair *)b;
  if (x->col != y->col) return x->col < y->col ? -1 : 1;
  return x->src < y->src ? -1 : (x->src > y->src);
}

void wko_reorder_columns_rowsort(const wko_layout *l, const int32_t *rowptr, const int32_t *cols,
                                 int32_t *out_cols, int32_t *out_src) {
  uint32_t maxlen = 0;
  for (uint32_t r = 0; r < l->nrows; r++)
    if ((uint32_t)(rowptr[r + 1] - rowptr[r]) > maxlen) maxlen = (uint32_t)(rowptr[r + 1] - rowptr[r]);
  rs_pair *t = (rs_pair *)malloc((maxlen ? maxlen : 1) * sizeof(rs_pair));
  for (uint32_t r = 0; r < l->nrows; r++) {
    int32_t k0 = rowptr[r], len = rowptr[r + 1] - k0;
    for (int32_t i = 0; i < len; i++) {
      t[i].col = l->row_map_inv[cols[k0 + i]];
      t[i].src = k0 + i;
    }
    qsort(t, (size_t)len, sizeof(rs_pair), rs_cmp);
    for (int32_t i = 0; i < len; i++) {
      out_cols[k0 + i] = t[i].col;
      out_src[k0 + i] = t[i].src;
    }
  }
  free(t);
}

void wko_run_f64(const wko_layout *l, const double *pvals, const int32_t *pcols,
                 const double *x, double *y, int fma_mode) {
  run_any(l, pvals, pcols, x, y, 1, fma_mode);
}

void wko_run_x_f64(const wko_layout *l, const double *pvals, const int32_t *pcols,
                   const double *x, double *y, int fma_mode) {
  run_any(l, pvals, pcols, x, y, 0, fma_mode);
}

int wko_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void wko_run_f64_omp(const wko_layout *l, const double *pvals, const int32_t *pcols,
                     const double *x, double *y, int nthreads) {
  if (nthreads <= 0) nthreads = wko_max_threads();
  long W = (long)l->nwarps;
  if (l->kind == 1) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (long w = 0; w < W; w++) {
      for (uint32_t lane = 0; lane < WS; lane++) {
        uint32_t id = (uint32_t)w * WS + lane;
        if (id >= l->nznrows) break;
        y[l->row_map[id]] =
            lane_sum(pvals, pcols, x, l->warp_offsets[w] + (int32_t)lane, l->max_nz_rows[w], 1);
      }
    }
  } else {
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (long w = 0; w < W; w++) wpk2_warp(l, (uint32_t)w, pvals, pcols, x, y, 1, 1);
  }
}

/* ---- reduced-precision storage ------------------------------------------ */

void wko_round_f32(const double *in, float *out, int64_t n) {
  for (int64_t i = 0; i < n; i++) out[i] = (float)in[i]; /* C conversion: nearest-even */
}

/* fp64 -> bf16 (8 significant bits, float's exponent range), rounded to
 * nearest-even in one step: the quantum of |d| is 2^(e-8) for d = m 2^e,
 * m in [0.5, 1), but never below bf16's subnormal step 2^-133; rint() rounds
 * the scaled value to an integer (ties to even in the default rounding mode),
 * which scaling back leaves exact.  Results of 2^128 and above overflow to inf. */
static uint16_t bf16_rne(double d) {
  const uint16_t sign = signbit(d) ? 0x8000u : 0u;
  if (isnan(d)) return 0x7fffu;
  if (isinf(d)) return sign | 0x7f80u;
  const double a = fabs(d);
  if (a == 0.0) return sign;
  int e;
  (void)frexp(a, &e);
  int qe = e - 8;
  if (qe < -133) qe = -133;
  const double r = ldexp(rint(ldexp(a, -qe)), qe);
  if (r >= 0x1p128) return sign | 0x7f80u;
  const float f = (float)r; /* exact: r has at most 8 significant bits */
  uint32_t u;
  memcpy(&u, &f, 4);
  return (uint16_t)(sign | (u >> 16));
}

void wko_round_bf16(const double *in, uint16_t *out, int64_t n) {
  for (int64_t i = 0; i < n; i++) out[i] = bf16_rne(in[i]);
}

static inline float lp_at(int vtype, const void *v, size_t i) {
  if (vtype == 0) return ((const float *)v)[i];
  uint32_t u = (uint32_t)((const uint16_t *)v)[i] << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

/* lane_sum in FP32: first product (a float multiply), then fmaf per step. */
static float lane_sum_lp(int vt, const void *A, const int32_t *c, const void *x, int32_t toffset,
                         uint32_t maxrows) {
  uint32_t maxnz = maxrows * WS + (uint32_t)toffset;
  float sum = lp_at(vt, A, (size_t)toffset) * lp_at(vt, x, (size_t)c[toffset]);
  for (toffset += (int32_t)WS; (uint32_t)toffset < maxnz; toffset += (int32_t)WS)
    sum = fmaf(lp_at(vt, A, (size_t)toffset), lp_at(vt, x, (size_t)c[toffset]), sum);
  return sum;
}

void wko_run_lp(const wko_layout *l, int vt, const void *pvals, const int32_t *pcols, const void *x,
                float *y, int mapped, int nthreads) {
  if (nthreads <= 0) nthreads = wko_max_threads();
  long W = (long)l->nwarps;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (long wl = 0; wl < W; wl++) {
    const uint32_t w = (uint32_t)wl;
    const uint32_t T = l->kind == 2 ? l->threads_per_row[w] : 1u;
    const uint32_t row_start = l->kind == 2 ? l->row_offset_warp[w] : w * WS;
    float s[32];
    for (uint32_t lane = 0; lane < WS; lane++) {
      s[lane] = 0.0f;
      if (row_start + lane / T < l->nznrows)
        s[lane] = lane_sum_lp(vt, pvals, pcols, x, l->warp_offsets[w] + (int32_t)lane, l->max_nz_rows[w]);
    }
    for (uint32_t lead = 0; lead < WS; lead += T) {
      const uint32_t rowid = row_start + lead / T;
      if (rowid >= l->nznrows) continue;
      float t[32];
      for (uint32_t k = 0; k < T; k++) t[k] = s[lead + k];
      for (uint32_t i = 1; i < T; i <<= 1)
        for (uint32_t k = 0; k + i < T; k += 2 * i) t[k] = t[k] + t[k + i];
      if (mapped)
        y[l->row_map[rowid]] = t[0];
      else
        y[rowid] = t[0];
    }
  }
}

void wko_csr_spmv_f64(const int32_t *rowptr, const int32_t *cols, const double *vals,
                      const double *x, double *y, uint32_t nrows, int nthreads) {
  if (nthreads <= 0) nthreads = wko_max_threads();
  long n = (long)nrows;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (long r = 0; r < n; r++) {
    double s = 0.0;
    for (int32_t k = rowptr[r]; k < rowptr[r + 1]; k++) s = fma(vals[k], x[cols[k]], s);
    y[r] = s;
  }
}

void wko_csr_spmv_t_f64(const int32_t *rowptr, const int32_t *cols, const double *vals,
                        const double *x, double *y, uint32_t nrows, uint32_t ncols) {
  for (uint32_t j = 0; j < ncols; j++) y[j] = 0.0;
  for (uint32_t r = 0; r < nrows; r++)
    for (int32_t k = rowptr[r]; k < rowptr[r + 1]; k++) y[cols[k]] = fma(vals[k], x[r], y[cols[k]]);
}

/* engine::verify (warpkernel.hpp:932-943). */
int wko_verify(uint32_t nrows, const double *orig, const double *comp, long *first_bad) {
  for (uint32_t i = 0; i < nrows; i++) {
    if ((fabs(orig[i]) <= 1e-14 && fabs(orig[i] - comp[i]) > 1e-14) ||
        (fabs((orig[i] - comp[i]) / orig[i]) > 1e-5 && fabs(orig[i]) > 1e-14)) {
      if (first_bad) *first_bad = (long)i;
      return 0;
    }
  }
  if (first_bad) *first_bad = -1;
  return 1;
}

/* engine::verify_x (warpkernel.hpp:945-957), including its mix of the mapped
 * index orig[row_map[i]] and the unmapped orig[i] in the same condition. */
int wko_verify_x(const wko_layout *l, const double *orig, const double *comp, long *first_bad) {
  for (uint32_t i = 0; i < l->nrows; i++) {
    double om = orig[l->row_map[i]];
    if ((fabs(om) <= 1e-14 && fabs(orig[i] - comp[i]) > 1e-14) ||
        (fabs((om - comp[i]) / om) > 1e-5 && fabs(orig[i]) > 1e-14)) {
      if (first_bad) *first_bad = (long)i;
      return 0;
    }
  }
  if (first_bad) *first_bad = -1;
  return 1;
}
