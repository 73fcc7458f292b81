/*
 * wk_oracle.h -- CPU oracle for the WPK1/WPK2 SpMV path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (warpkernel.hpp of thejonwong/warpkernel) against which the CUDA
 * implementation is tested.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arms may load it.  The product library never links,
 * loads or calls anything in this directory.
 *
 * Parity pin: the layout functions are checked byte-for-byte against the
 * reference's own host scan (warpkernel.hpp:215-771) compiled from its sources
 * by oracle/Makefile (target `ref`), and against the committed golden fixtures
 * in tests/golden/ that the same build produced.  The WPK1 arithmetic is
 * checked bit-for-bit against the reference kernels (warpkernel.hpp:53-75,
 * 103-125) executed on the CPU by the same build.
 */
#ifndef WK_ORACLE_H
#define WK_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Layout produced by structure::scan (kind 1) or structure2::scan (kind 2).
 * Field names and element types follow warpkernel.hpp:276-286, 561-565. */
typedef struct {
  int kind;                   /* 1 = WPK1, 2 = WPK2 */
  uint32_t nrows, nznrows, nz, allocate_nz, nwarps;
  uint32_t min_nz, max_nz, nmax_per_thread; /* WPK2 only */
  uint32_t variant;           /* WKO_ABL_* flags of wko_scan1_ablation, else 0 */
  int32_t *row_map;           /* [nrows]   sorted position -> original row */
  int32_t *row_map_inv;       /* [nrows]   original row -> sorted position */
  uint32_t *reorder_rows;     /* [nz]      CSR position -> padded slot      */
  int32_t *warp_offsets;      /* [nwarps+1]                                */
  uint32_t *max_nz_rows;      /* [nwarps]                                  */
  uint32_t *threads_per_row;  /* [nwarps]   WPK2 only                      */
  uint32_t *row_offset_warp;  /* [nwarps+1] WPK2 only                      */
} wko_layout;

/* Returns 0 on success, nonzero on malformed input (rowptr not monotone,
 * rowptr[0] != 0, rowptr[nrows] != nz) or allocation failure. */
int wko_scan1(const int32_t *rowptr, uint32_t nrows, uint32_t nz, wko_layout *out);
int wko_scan2(const int32_t *rowptr, uint32_t nrows, uint32_t nz, int32_t threshold,
              wko_layout *out);
void wko_free(wko_layout *l);

/* The WPK1 ablation layouts of optimization.cu: WKO_ABL_NOSORT = scan_nosort
 * (372-442), WKO_ABL_NOCOALESCE = scan_nocoalesced (233-294), both =
 * scan_nocoalesced_nosort (298-368).  Rows without entries go last and get
 * no warp (as structure::scan), where the optimization.cu scans count warps
 * over all rows; on matrices without empty rows the arrays are the same. */
enum { WKO_ABL_NOSORT = 1, WKO_ABL_NOCOALESCE = 2 };
int wko_scan1_ablation(const int32_t *rowptr, uint32_t nrows, uint32_t nz, int flags, wko_layout *out);

/* structure::reorder (warpkernel.hpp:380-398): padded values/colinds. */
void wko_process_f64(const wko_layout *l, const double *vals, const int32_t *cols,
                     double *pvals, int32_t *pcols);
void wko_process_f32(const wko_layout *l, const float *vals, const int32_t *cols,
                     float *pvals, int32_t *pcols);
/* reorder_columns_coalesced (warpkernel.hpp:447-457). */
void wko_reorder_columns_coalesced(const wko_layout *l, const int32_t *cols, int32_t *out);
/* reorder_columns (warpkernel.hpp:401-412), CSR order. */
void wko_reorder_columns(const wko_layout *l, const int32_t *cols, int32_t *out);
/* reorder_x (warpkernel.hpp:518-530). */
void wko_reorder_x_f64(const wko_layout *l, const double *x, double *xout);
/* reorder_columns_rowsort (warpkernel.hpp:414-444): per CSR row the
 * renumbered columns in ascending order and the CSR position of each
 * (reorder_A_rows); equal columns keep their CSR order. */
void wko_reorder_columns_rowsort(const wko_layout *l, const int32_t *rowptr, const int32_t *cols,
                                 int32_t *out_cols, int32_t *out_src);
/* warpKernel_assembly (warpkernel.hpp:78-100): y[row_map[id]] = sum of the
 * row's padded values, first slot then += each further one; WPK2 lanes of a
 * row are combined by the same lockstep tree as the SpMV. */
void wko_assembly_f64(const wko_layout *l, const double *pvals, double *y);

/* engine::run / run_x in the documented accumulation order
 * (warpkernel.hpp:53-75, 103-125, 127-168, 170-211).
 * fma_mode 1: sum += a*x contracted to fma(a, x, sum); 0: separate mul + add.
 * Rows with no entries are not written (y keeps its content). */
void wko_run_f64(const wko_layout *l, const double *pvals, const int32_t *pcols,
                 const double *x, double *y, int fma_mode);
void wko_run_x_f64(const wko_layout *l, const double *pvals, const int32_t *pcols,
                   const double *x, double *y, int fma_mode);

/* Reduced-precision storage (no reference counterpart): the library rounds
 * fp64 values and x to FP32 or BF16 once, round-to-nearest-even, and sums in
 * FP32.  wko_round_f32 / wko_round_bf16 round each fp64 input in one step
 * (bf16 as raw bits).  wko_run_lp is the documented order of
 * warpkernel.hpp:65-71 / 147-162 in FP32: per lane the first product, then
 * fmaf per step of 32 slots, then the WPK2 pairwise tree; vtype 0 = FP32
 * values and x, 1 = BF16 values and x (raw bits); y is FP32; mapped 1 = run
 * (y[row_map[p]]), 0 = run_x (y[p]).  Rows without entries are not written.
 * OpenMP across layout warps (nthreads <= 0: all threads); the per-row
 * arithmetic does not depend on the thread count. */
void wko_round_f32(const double *in, float *out, int64_t n);
void wko_round_bf16(const double *in, uint16_t *out, int64_t n);
void wko_run_lp(const wko_layout *l, int vtype, const void *pvals, const int32_t *pcols, const void *x,
                float *y, int mapped, int nthreads);

/* Plain CSR multiply y = A x (row-parallel, OpenMP, static schedule); the
 * multicore CPU baseline.  nthreads <= 0 uses all available threads. */
void wko_csr_spmv_f64(const int32_t *rowptr, const int32_t *cols, const double *vals,
                      const double *x, double *y, uint32_t nrows, int nthreads);
/* Transpose product y = A^T x on the CSR, serial, exact column-major order of
 * accumulation (row ascending) -- the host CSR-transpose reference. */
void wko_csr_spmv_t_f64(const int32_t *rowptr, const int32_t *cols, const double *vals,
                        const double *x, double *y, uint32_t nrows, uint32_t ncols);
/* Documented-order WPK run on the CPU with OpenMP across warps (the
 * reference path's arithmetic restated; used as the CPU reference arm). */
void wko_run_f64_omp(const wko_layout *l, const double *pvals, const int32_t *pcols,
                     const double *x, double *y, int nthreads);
int wko_max_threads(void);

/* engine::verify / verify_x (warpkernel.hpp:932-957), including verify_x's
 * mixed use of orig[row_map[i]] and orig[i].  Returns 1 when it passes,
 * 0 otherwise; *first_bad receives the failing index or -1. */
int wko_verify(uint32_t nrows, const double *orig, const double *comp, long *first_bad);
int wko_verify_x(const wko_layout *l, const double *orig, const double *comp, long *first_bad);

/* Finite-element test matrices (CPU restatement of the product generator, same
 * hash and the same floating-point operations, so outputs are bit-identical).
 * dim 2: Q1 quads ex x ey; dim 3: trilinear hexes ex x ey x ez.  dof = dofs
 * per node.  value_mode 0: stencil values (off-diagonal U(-1,0) symmetric,
 * diagonal 1.01 x absolute off-diagonal row sum); 1: assembled random SPD
 * element blocks G G^T / nb + 0.01 I, scaled by the element volume.
 * wko_fe_size returns nrows and nnz; wko_fe_fill writes rowptr[nrows+1],
 * cols[nnz], vals[nnz] (any of them may be NULL). */
int wko_fe_size(int dim, int ex, int ey, int ez, int dof, int64_t *nrows, int64_t *nnz);
int wko_fe_fill(int dim, int ex, int ey, int ez, int dof, int value_mode, uint64_t seed,
                int32_t *rowptr, int32_t *cols, double *vals, int nthreads);
/* Uniform(-1,1) vector from the same hash (stream id selects the vector). */
void wko_uniform_vec(uint64_t seed, uint64_t stream, double *x, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
