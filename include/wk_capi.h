/*
 * wk_capi.h -- C ABI of the GB300-native WPK1/WPK2 sparse matrix-vector
 * multiply (libwarpkernel_gb300.so).
 *
 * This is the boundary a host binding (C++ header, ctypes, cgo, JNI ...)
 * calls.  Signatures use plain pointers, sizes and opaque handles only.
 * Every call returns a wk_status (0 = success) and never exits the process;
 * wk_last_error() describes the last failure of the calling thread.
 *
 * Reference interface replaced: `warpkernel::structure`, `structure2` and
 * `engine<ValueType, IndexType>` of warpkernel.hpp (thejonwong/warpkernel).
 * Each entry point below names the reference member it stands for.
 *
 * Memory: pointer arguments documented as "host or device" are classified
 * with cudaPointerGetAttributes (pageable/pinned host memory or device /
 * managed memory of the current device).  x / y vectors of wk_run* are
 * device pointers, as in the reference (engine::run takes device arrays).
 *
 * Streams: `stream` is a cudaStream_t passed as void* (NULL = legacy default
 * stream).  Calls are stream-ordered; only the ones that return host data or
 * a measured time synchronise.
 */
#ifndef WK_CAPI_H
#define WK_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int wk_status;
enum {
  WK_OK = 0,
  WK_ERR_INVALID = 1,   /* bad argument (null pointer, size, malformed CSR ...) */
  WK_ERR_CUDA = 2,      /* a CUDA runtime call failed */
  WK_ERR_ALLOC = 3,     /* device or host allocation failed */
  WK_ERR_OVERFLOW = 4,  /* layout does not fit the reference's int32 offsets */
  WK_ERR_STATE = 5,     /* handle used in a state that does not allow the call */
  WK_ERR_DEVICE = 6,    /* a kernel reported an error through its status word */
  WK_ERR_NOTCONV = 7    /* an iterative solve stopped before its tolerance */
};

typedef struct wk_layout wk_layout; /* a scanned WPK1/WPK2 layout (device resident) */
typedef struct wk_engine wk_engine; /* padded values + column indices on the device */

/* Element types of values and vectors.  WK_F16S (no reference counterpart):
 * values stored as FP16 relative to a power-of-two scale per layout warp (the
 * warp's largest magnitude maps into [2^14, 2^15)), 2 bytes per value like
 * WK_BF16 but with FP16's 11-bit significand; callers pass FP32 values and
 * FP32 x, and get FP32 y (FP32 accumulation, the row total multiplied by the
 * scale, which is exact). */
enum { WK_F64 = 0, WK_F32 = 1, WK_BF16 = 2, WK_F16S = 3 };

/* Layout kinds: WPK1 = structure, WPK2 = structure2. */
enum { WK_WPK1 = 1, WK_WPK2 = 2 };

/* Arrays of a layout, named as the reference's public members
 * (warpkernel.hpp:276-286, 561-562). */
enum {
  WK_FIELD_ROW_MAP = 0,         /* int32[nrows]     y[row_map[i]] = y'[i]          */
  WK_FIELD_ROW_MAP_INV = 1,     /* int32[nrows]                                   */
  WK_FIELD_REORDER_ROWS = 2,    /* uint32[nz]       new_values[reorder_rows[i]] = A[i] */
  WK_FIELD_WARP_OFFSETS = 3,    /* int32[nwarps+1]                                */
  WK_FIELD_MAX_NZ_ROWS = 4,     /* uint32[nwarps]                                 */
  WK_FIELD_THREADS_PER_ROW = 5, /* uint32[nwarps]   WPK2 only                      */
  WK_FIELD_ROW_OFFSET_WARP = 6  /* uint32[nwarps+1] WPK2 only                      */
};

typedef struct {
  int kind;                  /* WK_WPK1 / WK_WPK2 */
  uint32_t nrows, nznrows, nz, allocate_nz, nwarps;
  uint32_t min_nz, max_nz;   /* WPK2: extreme non-empty row lengths */
  uint32_t nmax_per_thread;  /* WPK2: the threshold it was scanned with */
  uint32_t variant;          /* WK_ABL_* flags of wk_scan1_ablation, else 0 */
} wk_layout_info;

/* ---- diagnostics ------------------------------------------------------- */

/* Copies the calling thread's last error message (NUL-terminated, truncated
 * to `cap`) and returns its full length.  No reference counterpart. */
size_t wk_last_error(char *buf, size_t cap);
/* Library version string.  No reference counterpart. */
const char *wk_version(void);
/* Test hook for the error paths (no reference counterpart): the nth device
 * allocation the library makes from now on fails with WK_ERR_ALLOC without
 * calling cudaMalloc; 0 switches it off. */
void wk_debug_fail_alloc(int nth);

/* ---- scan (layout built on the device) ---------------------------------- */

/* structure::scan(nz, nrows, A, rows, colinds) -- warpkernel.hpp:309-365.
 * rowptr: nrows+1 CSR row offsets, host or device.  The layout arrays are
 * built on the GPU and are bit-identical to the reference's host scan.
 * Fails with WK_ERR_INVALID if rowptr[0] != 0, rowptr is not monotone or
 * rowptr[nrows] != nz, and WK_ERR_OVERFLOW if allocate_nz exceeds INT32_MAX. */
wk_status wk_scan1(const int32_t *rowptr, uint32_t nrows, uint32_t nz, void *stream,
                   wk_layout **out);

/* structure2::scan(nz, nrows, A, rows, colinds, threshold) --
 * warpkernel.hpp:579-736.  Same inputs plus the per-thread threshold. */
wk_status wk_scan2(const int32_t *rowptr, uint32_t nrows, uint32_t nz, int32_t threshold,
                   void *stream, wk_layout **out);

/* The WPK1 ablation layouts of optimization.cu, built on the device:
 * WK_ABL_NOSORT -- scan_nosort (optimization.cu:372-442): rows keep their CSR
 *   order (warps of 32 consecutive rows, each padded to its longest row);
 * WK_ABL_NOCOALESCE -- scan_nocoalesced (233-294): sorted rows, but each
 *   lane's entries are contiguous (slot o_w + lane * max_nz_rows[w] + i)
 *   instead of interleaved;
 * both -- scan_nocoalesced_nosort (298-368).
 * Rows without entries are moved to the end and get no warp, as in
 * structure::scan (the optimization.cu scans count warps over all rows, and
 * their nosort forms read past their row list when a row is empty).  Layouts
 * with WK_ABL_NOSORT only are ordinary interleaved WPK1 layouts that every
 * call accepts.  WK_ABL_NOCOALESCE layouts support engine creation and
 * access, the reorderings, run / run_x (the reference's
 * warpKernel_nocoalesced, optimization.cu:91-114, in either order argument),
 * run_host and the files; the solver, adjoint, batched, compressed-column
 * and assembly calls refuse them with WK_ERR_INVALID. */
enum { WK_ABL_NOSORT = 1, WK_ABL_NOCOALESCE = 2 };
wk_status wk_scan1_ablation(const int32_t *rowptr, uint32_t nrows, uint32_t nz, int flags, void *stream,
                            wk_layout **out);

wk_status wk_layout_info_get(const wk_layout *l, wk_layout_info *info);

/* Copies one layout array to host memory.  `dst` may be NULL to query the
 * element count in *count; otherwise `cap` is its capacity in elements. */
wk_status wk_layout_get(const wk_layout *l, int field, void *dst, size_t cap, size_t *count);

/* Releases the caller's reference; device memory is freed when no engine
 * created from the layout remains. */
wk_status wk_layout_destroy(wk_layout *l);

/* ---- reorderings -------------------------------------------------------- */

/* structure::reorder_columns_coalesced(colinds) -- warpkernel.hpp:447-457.
 * cols: nz CSR column indices (host or device); out: allocate_nz padded,
 * renumbered column indices (host or device).  Padding slots are 0. */
wk_status wk_reorder_columns_coalesced(const wk_layout *l, const int32_t *cols, int32_t *out,
                                       void *stream);

/* structure::reorder_columns(colinds) -- warpkernel.hpp:401-412: nz column
 * indices renumbered to sorted order, CSR order kept. */
wk_status wk_reorder_columns(const wk_layout *l, const int32_t *cols, int32_t *out, void *stream);

/* structure::reorder_columns_rowsort(colinds, rows) -- warpkernel.hpp:414-444
 * (used by optimize.cu:655, optimize2.cu:749): per CSR row, the renumbered
 * columns row_map_inv[cols[k]] in ascending order (out_cols, nz entries) and
 * the CSR position each came from (reorder_A_rows, nz entries), so that
 * vals[reorder_A_rows[k]] are the matching values.  Square matrices only:
 * every column must lie in [0, nrows).  Equal columns within a row keep their
 * CSR order (the reference's std::sort leaves their order unspecified).
 * Host or device arrays; synchronous. */
wk_status wk_reorder_columns_rowsort(const wk_layout *l, const int32_t *cols, int32_t *out_cols,
                                     int32_t *reorder_A_rows, void *stream);

/* structure::reorder / process (warpkernel.hpp:380-398, 533-548, 750-769)
 * into caller buffers: pvals gets allocate_nz values of `dtype` (WK_F64,
 * WK_F32 or WK_BF16) and pcols allocate_nz column indices, padding slots 0;
 * vals / cols are the nz CSR-ordered arrays.  Either output may be NULL
 * (with its input), which also gives reorder_values_coalesced (470-491) and
 * the reorder_*_coalesced_GPU scatters (459-468, 494-503).  Inputs and
 * outputs host or device; columns are copied as given (not validated, not
 * renumbered), as the reference copies them.  Synchronous. */
wk_status wk_process(const wk_layout *l, int dtype, const void *vals, const int32_t *cols, void *pvals,
                     int32_t *pcols, void *stream);

/* structure::reorder_x(x, device_x) -- warpkernel.hpp:518-530:
 * x_out[row_map_inv[r]] = x[r].  dtype WK_F64 / WK_F32 / WK_BF16. */
wk_status wk_reorder_x(const wk_layout *l, int dtype, const void *x, void *x_out, void *stream);

/* ---- engine ------------------------------------------------------------- */

/* engine(structure&, A, colinds) / engine(structure2&, A, colinds), which
 * call structure::process -- warpkernel.hpp:794-809, 533-548, 750-769.
 * vals: nz values of type `dtype`, cols: nz column indices (each host or
 * device).  The padded, interleaved arrays are built on the GPU.  ncols is
 * the length of x (every column index must lie in [0, ncols)).  The engine
 * keeps the layout alive. */
wk_status wk_engine_create(wk_layout *l, int dtype, const void *vals, const int32_t *cols,
                           uint32_t ncols, void *stream, wk_engine **out);

/* Replaces the engine's padded column indices by caller-supplied ones
 * (allocate_nz entries, host or device), e.g. the output of
 * wk_reorder_columns_coalesced -- the reference drivers assign
 * `eng.device_colinds = reorder_cols` (wpk1.cu:175, 198).  Indices are
 * validated against ncols. */
wk_status wk_engine_set_colinds(wk_engine *e, const int32_t *padded_cols, void *stream);

/* Replaces the engine's values from CSR-ordered `vals` (nz entries, host or
 * device, of the engine's dtype) without rescanning -- reference process()
 * with the same structure. */
wk_status wk_engine_set_values(wk_engine *e, const void *vals, void *stream);

/* Copies engine.device_values / device_colinds (allocate_nz entries) out. */
wk_status wk_engine_get_values(const wk_engine *e, void *dst, size_t cap);
wk_status wk_engine_get_colinds(const wk_engine *e, int32_t *dst, size_t cap);

wk_status wk_engine_destroy(wk_engine *e);

/* Adds a compact column storage to the engine (no reference counterpart;
 * the mixed-precision paths): every layout warp whose real entries span fewer
 * than 65,536 columns stores them as 16-bit offsets from a per-warp base, the
 * others keep 32-bit indices in a side array.  Afterwards WK_ORDER_FAST runs
 * of WK_F32, WK_BF16 and WK_F16S engines stream 2 B instead of 4 B of index
 * per slot; results are bit-identical to the uncompressed fast order.
 * WK_F64 engines keep reading 32-bit indices in wk_run / wk_run_x and the CG
 * (their SpMV is bound by GB300's FP64 rate, and the offsets measured 7 %
 * slower); the adjoint uses the compact storage for every type.
 * *wide_warps (optional) = warps left 32-bit.  wk_engine_set_colinds
 * rebuilds the compact storage. */
wk_status wk_engine_compress_cols(wk_engine *e, void *stream, uint32_t *wide_warps);

/* x windows (no reference counterpart; shared-memory staging of x in place of
 * the reference's texture fetch, warpkernel.hpp:27-49).  With windows on,
 * wk_engine_compress_cols also gives every narrow layout warp with at most
 * 512 distinct columns, in at most 32 chunks of <= 32 consecutive columns,
 * an x window: its distinct columns as chunks, and per slot the window
 * position of its column (2 B, a second per-slot array).  Fast-order wk_run /
 * wk_run_x then copy each such warp's x values into shared memory, one
 * warp-wide copy per chunk, and gather from there instead of from L1/L2; the
 * sums are the same bits.  On by default for WK_F32 and WK_F16S engines
 * (4-byte x: the copy is asynchronous and overlaps the first loads of the
 * matrix stream; hex 96^3 with 16-bit columns, 1-2 % faster than the L1/L2
 * gathers), off for WK_BF16 (2-byte x is staged by loads and stores before
 * the stream starts: 9 % slower).  `on` = 1 switches them on (building them
 * if the compact columns exist; WK_ERR_STATE without them), `on` = 0 off.
 * *window_warps (optional) = warps that have a window (0 while none are
 * built). */
wk_status wk_engine_set_windows(wk_engine *e, int on, uint32_t *window_warps);

/* ---- SpMV --------------------------------------------------------------- */

/* Accumulation order of wk_run / wk_run_x. */
enum {
  WK_ORDER_FAST = 0,  /* 256/128-bit loads; each lane's slots re-associated */
  WK_ORDER_EXACT = 1  /* the reference's order, bit-identical to the oracle  */
};
/* WK_ORDER_FAST on a layout of short warps (slot-weighted mean step count
 * below 32 for fp64, 20 for fp32 and bf16, 16 for scaled FP16) runs the exact-order
 * kernel, which is the faster one there; its results then equal
 * WK_ORDER_EXACT's and compressed columns are not used. */

/* engine::run<cache>(nblocks, blocksize, dx, dy) -- warpkernel.hpp:811-860:
 * y[row_map[p]] = sum over row p.  dx: ncols device values, dy: nrows device
 * values of the engine's dtype (FP32 accumulation and FP32 y for WK_BF16
 * engines).  blocksize: threads per block (a multiple of 32, <= 1024);
 * nblocks must cover nwarps / (blocksize/32) blocks; nblocks <= 0 or
 * blocksize <= 0 selects the launch shape automatically.  cache != 0 gathers
 * x with read-only non-coherent loads (the texture-cache path of the
 * reference), 0 with plain L1-caching loads (the reference's x[i]).
 * If `seconds` is non-NULL the call synchronises and stores the kernel time
 * measured with CUDA events (the reference returns elapsed seconds);
 * otherwise it returns right after the launch.  Rows without entries are not
 * written. */
wk_status wk_run(wk_engine *e, int nblocks, int blocksize, int cache, int order, const void *dx,
                 void *dy, void *stream, float *seconds);

/* engine::run_x<cache>(...) -- warpkernel.hpp:862-896: y'[p] = sum over
 * sorted row p (no row_map scatter).  Used with renumbered columns and the
 * reordered x of wk_reorder_x. */
wk_status wk_run_x(wk_engine *e, int nblocks, int blocksize, int cache, int order, const void *dx,
                   void *dy, void *stream, float *seconds);

/* engine::run with HOST vectors: copies x_host (ncols values) to an
 * engine-owned device buffer, runs the SpMV and copies y back into y_host
 * (nrows values; entries of empty rows are written as 0).  This is the
 * reference drivers' sequence (H2D of x, run, D2H of y: wpk1.cu:120, 149,
 * 155) in one call.  `mapped` 1 = run, 0 = run_x.  Pinned host buffers give
 * the fastest copies.  Synchronous. */
wk_status wk_run_host(wk_engine *e, int mapped, int order, const void *x_host, void *y_host,
                      void *stream);

/* `count` SpMVs on host vectors, each as wk_run_host (x_host[i] -> device,
 * run or run_x, y -> y_host[i]) with the same results, but double-buffered
 * on two copy streams: the upload of x_host[i+1] and the download of
 * y_host[i-1] overlap SpMV i, so with pinned buffers the host link is hidden
 * behind the HBM-bound SpMV.  Synchronous: returns when every y_host[i] is
 * written; `seconds` (optional) = elapsed time of the whole sequence. */
wk_status wk_run_host_stream(wk_engine *e, int mapped, int order, int count, const void *const *x_host,
                             void *const *y_host, void *stream, float *seconds);

/* engine::run_assembly<cache>(nblocks, blocksize, dy) -- warpkernel.hpp:898-929
 * with warpKernel_assembly (warpkernel.hpp:78-100): y[row_map[p]] = the sum of
 * the stored values of row p (first slot, then += each further slot, in the
 * reference's order).  WPK2 rows are summed by their threads_per_row lanes
 * and the same lockstep tree as wk_run (the reference returns -1 for WPK2 and
 * its WPK1 launch passes five arguments to the six-parameter kernel).  dy:
 * nrows device values (FP32 for WK_BF16 engines); rows without entries are
 * not written.  `seconds` as for wk_run. */
wk_status wk_run_assembly(wk_engine *e, int nblocks, int blocksize, void *dy, void *stream,
                          float *seconds);

/* ---- files -------------------------------------------------------------- */

/* Saves a layout -- structure::serialize's fields (warpkernel.hpp:253-269:
 * nrows, nz, allocate_nz, nwarps, ... and the row_map, row_map_inv,
 * reorder_rows, warp_offsets, max_nz_rows arrays) plus WPK2's
 * threads_per_row / row_offset_warp and the CSR row offsets -- to a binary
 * file (little-endian, magic "WPKLAYT1"), so a layout is scanned once and
 * reloaded.  wk_layout_load rebuilds the layout on the current device from
 * the file's row offsets and threshold (nmax_per_thread) and accepts the file
 * only if every array and header field is identical to that scan, so a
 * corrupt or edited file is refused (WK_ERR_INVALID) before any kernel reads
 * it. */
wk_status wk_layout_save(const wk_layout *l, const char *path);
wk_status wk_layout_load(const char *path, void *stream, wk_layout **out);

/* Matrix Market reader -- the drivers' cusp::io::read_matrix_market_file
 * (wpk1.cu:43-48, wpk2.cu:54-57): `coordinate` matrices with real, double,
 * integer or pattern fields (pattern values are 1) and general, symmetric or
 * skew-symmetric symmetry (the mirror entries are added).  The result is CSR
 * with columns ascending within each row (duplicates kept, in file order).
 * wk_csr_get exposes its host arrays until wk_csr_free. */
typedef struct wk_csr wk_csr;
wk_status wk_mm_read(const char *path, wk_csr **out);
wk_status wk_csr_get(const wk_csr *c, int64_t *nrows, int64_t *ncols, int64_t *nnz,
                     const int32_t **rowptr, const int32_t **cols, const double **vals);
wk_status wk_csr_free(wk_csr *c);

/* ---- solver building blocks (no reference counterpart) ------------------ */

/* Residual of an fp64 engine: r = b - A x for every row (rows without
 * entries get r = b) and, if norm2 is non-NULL, *norm2 = ||r||^2 written to
 * DEVICE memory.  x (ncols), b, r (nrows) and norm2 are device pointers.  The
 * norm is reduced in a fixed order (bit-reproducible).  Uses an engine-owned
 * device buffer of per-block partial sums, allocated on the first call.
 * It is the fp64 residual of the iterative-refinement solve (wk_ir_cg). */
wk_status wk_residual(wk_engine *e, const double *x, const double *b, double *r, double *norm2,
                      void *stream);

/* wk_residual without any device allocation.  No counterpart in the
 * reference.  For callers that must not call cudaMalloc while they run --
 * e.g. a solver plugin inside a host application that owns the GPU's whole
 * memory budget, or a latency-critical loop that cannot afford cudaMalloc's
 * implicit device synchronisation.  Same inputs, outputs and results as
 * wk_residual (the caller still provides x, b, r and norm2); the per-block
 * partial sums go to a static device array of 65,536 doubles (512 KiB) that
 * every GPU loading the library keeps until the process exits.  Layouts with
 * more than 262,144 warps are rejected with WK_ERR_INVALID.  The first call on
 * each engine looks up that array's address (cudaGetSymbolAddress) and keeps
 * it in the engine.  Under CUDA's lazy module loading (the default), the first
 * call on a device also loads the code that holds the array, which reserves
 * its 512 KiB at that moment -- itself a device allocation.  So make one call
 * per engine during set-up, before any stream capture and before the phase in
 * which nothing may allocate.  All calls share the array:
 * calls whose kernels overlap on the GPU (other streams, other threads) race
 * and must be serialised by the caller.  Creating the engine allocates; this
 * call does not. */
wk_status wk_residual_static(wk_engine *e, const double *x, const double *b, double *r, double *norm2,
                             void *stream);

/* Conjugate-gradient solves of A x = b for a symmetric positive definite A
 * (no reference counterpart: an SpMV consumer that runs the WPK kernels in
 * a solver loop, with an iterative-refinement form whose inner solve uses a
 * low-precision engine).  Inputs: tol
 * (target ||b - A x|| / ||b||), max_iter (CG iterations, or outer refinement
 * steps for wk_ir_cg), max_inner / inner_tol (inner CG iterations and the
 * relative reduction each inner solve aims for), check_every (iterations
 * between host-side convergence checks; scalars otherwise stay on the
 * device).  Outputs: iters (CG iterations; for wk_ir_cg the inner total),
 * outer, relres (the fp64 relative residual of the returned x) and seconds
 * (device time of the whole solve, CUDA events).  Returns WK_ERR_NOTCONV if
 * tol was not reached. */
typedef struct {
  double tol;
  int max_iter;
  int max_inner;
  double inner_tol;
  int check_every;
  int iters;
  int outer;
  double relres;
  double seconds;
  /* wk_ir_cg: 0 (default) sums the inner solve's dot products p.q and r.r in
   * FP64 (each FP32 element converted once); 1 sums each thread's and each
   * block's share in FP32 and only the block partials in FP64. */
  int inner_dots_fp32;
} wk_cg_params;

/* fp64 CG on an fp64 engine; b, x (initial guess, overwritten) are device
 * vectors of nrows doubles. */
wk_status wk_cg(wk_engine *e, const double *b, double *x, wk_cg_params *p, void *stream);

/* Iterative-refinement CG: the residual b - A x, its norm, the dot products of
 * the outer loop and the update x += d stay fp64 (engine e64); each
 * correction d solves A d = r with an fp32 CG on the low-precision engine `lo`
 * (WK_F32, WK_BF16 or WK_F16S values, compressed columns if
 * wk_engine_compress_cols was called): fp32 vectors updated in fp32
 * arithmetic, the inner dot products summed in fp64 (or, with
 * p->inner_dots_fp32 = 1, in fp32 within a block and fp64 across blocks). */
wk_status wk_ir_cg(wk_engine *e64, wk_engine *lo, const double *b, double *x, wk_cg_params *p,
                   void *stream);

/* ---- adjoint (no reference counterpart; differentiable SpMV) ------------- */

typedef struct wk_adjoint wk_adjoint;

/* Builds A^T's WPK layout (kind WK_WPK1 / WK_WPK2 with `threshold`) and
 * engine on the device from the forward engine `fwd` (WK_F64 or WK_F32):
 * the CSR entries are stably sorted by column, so no atomics touch values and
 * results are deterministic.  `fwd` must outlive the adjoint.  When A is
 * structurally symmetric with sorted rows and kind/threshold equal fwd's,
 * both layouts coincide and wk_adjoint_run uses one fused pass. */
wk_status wk_adjoint_create(wk_engine *fwd, int kind, int32_t threshold, void *stream, wk_adjoint **out);

/* New values: vals_csr (nz, CSR order, host or device, fwd's dtype) are
 * loaded into the forward engine and A^T's engine; vals_csr = NULL re-derives
 * A^T's values from the forward engine's current values. */
wk_status wk_adjoint_refresh(wk_adjoint *a, const void *vals_csr, void *stream);

/* Index order of dvals. */
enum {
  WK_DVALS_CSR = 0,   /* nz entries, CSR order of the values given to the engine */
  WK_DVALS_SLOTS = 1  /* allocate_nz entries, the forward layout's padded slot order
                       * (engine.device_values order; padding slots get 0) */
};

/* dx = A^T dy (ncols entries; NULL to skip) and dvals = dy[row(k)] x[col(k)]
 * for every stored entry k (NULL to skip), in `dvals_order`.  x, dy, dx,
 * dvals are device vectors of fwd's dtype.  WK_DVALS_SLOTS writes the
 * gradient where the values are stored, with coalesced stores (the fastest
 * form; dvals 32-byte aligned).  Stream-ordered. */
wk_status wk_adjoint_run(wk_adjoint *a, const void *x, const void *dy, void *dx, void *dvals,
                         int dvals_order, void *stream);

/* New values in slot order (allocate_nz entries, device or host; padding
 * ignored), loaded into the forward engine and A^T's engine. */
wk_status wk_adjoint_refresh_slots(wk_adjoint *a, const void *vals_slots, void *stream);

/* *symmetric = 1 when the fused path is used; tinfo = A^T's layout info. */
wk_status wk_adjoint_info(const wk_adjoint *a, int *symmetric, wk_layout_info *tinfo);

/* A new reference to A^T's layout (release it with wk_layout_destroy). */
wk_status wk_adjoint_transposed_layout(const wk_adjoint *a, wk_layout **tl);

wk_status wk_adjoint_destroy(wk_adjoint *a);

/* ---- batched multi-RHS (no reference counterpart) ------------------------ */

typedef struct wk_batch wk_batch;

/* Many engines (all WK_F32 or all WK_F64; they must outlive the batch), each
 * with nrhs[m] right-hand sides, computed by one persistent launch: work
 * items (matrix, `chunk` layout warps) ordered by cost are taken from a
 * global queue by the warps of one wave of blocks.  Each loaded value and
 * column is reused for `rhs_tile` right-hand sides (1, 2, 4, 8 or 16).
 * Results equal each engine's own run (same per-row order), whichever warp
 * computes them. */
wk_status wk_batch_create(wk_engine *const *engines, const uint32_t *nrhs, int count, int rhs_tile, int chunk,
                          wk_batch **out);
/* X[m]: device, ncols_m x nrhs_m, row-major, any alignment of the element
 * type; Y[m]: device, nrows_m x nrhs_m (rows without entries are not
 * written).  The batch keeps a blocked copy of X -- the right-hand sides in
 * groups of 16 bytes (4 floats / 2 doubles, zero-filled), each group an
 * ncols_m x group array -- which every launch refreshes from X[m] before the
 * SpMV, so every right-hand-side count is gathered with 16-byte loads (device
 * memory: ncols_m x nrhs_m rounded up to the group, per matrix).  Call again
 * (and wk_batch_capture again) when X or Y move; WK_ERR_INVALID if a
 * matrix's blocked X would hold 2^32 elements or more. */
wk_status wk_batch_set_vectors(wk_batch *b, const void *const *X, void *const *Y);
wk_status wk_batch_set_tile(wk_batch *b, int rhs_tile);
/* Captures the launch (queue reset + persistent kernel) into a CUDA graph
 * that wk_batch_run then replays. */
wk_status wk_batch_capture(wk_batch *b);
/* One launch; seconds (optional) = device time, synchronous. */
wk_status wk_batch_run(wk_batch *b, void *stream, float *seconds);
wk_status wk_batch_info(const wk_batch *b, uint32_t *nitems, uint32_t *grid, int *rhs_tile);
wk_status wk_batch_destroy(wk_batch *b);

/* ---- verification ------------------------------------------------------- */

/* engine::verify(orig, comp) -- warpkernel.hpp:932-943 (host arrays of nrows
 * doubles; 1e-5 relative, 1e-14 absolute for |orig| <= 1e-14).  *pass = 1 if
 * it passes; *first_bad = first failing index or -1. */
wk_status wk_verify(const wk_layout *l, const double *orig, const double *comp, int *pass,
                    int64_t *first_bad);

/* engine::verify_x(orig, comp) -- warpkernel.hpp:945-957.  strict = 0 keeps
 * the reference's condition exactly (it mixes orig[row_map[i]] and orig[i]);
 * strict = 1 uses orig[row_map[i]] throughout. */
wk_status wk_verify_x(const wk_layout *l, const double *orig, const double *comp, int strict,
                      int *pass, int64_t *first_bad);

/* ---- device and test-input utilities (no reference counterpart) --------- */

/* Finite-element test matrix generated on the device (same numbering and
 * bit-identical values as the CPU generator used by the tests).
 * dim 2: ex x ey Q1 quads; dim 3: ex x ey x ez hexes; dof unknowns per node.
 * value_mode 0: off-diagonal U(-1,0) symmetric, diagonal 1.01 x absolute row
 * sum; 1: assembled random SPD element blocks scaled by the element volume.
 * wk_fe_size gives the sizes; wk_fe_fill writes device arrays rowptr
 * (nrows+1), cols (nnz) and vals (nnz, float64); any may be NULL. */
wk_status wk_fe_size(int dim, int ex, int ey, int ez, int dof, int64_t *nrows, int64_t *nnz);
wk_status wk_fe_fill(int dim, int ex, int ey, int ez, int dof, int value_mode, uint64_t seed,
                     int32_t *rowptr, int32_t *cols, double *vals, void *stream);
/* Uniform(-1,1) float64 device vector from the generator's hash. */
wk_status wk_uniform_vec(uint64_t seed, uint64_t stream_id, double *x, int64_t n, void *stream);
/* Element-type conversion of a device vector (float64 -> float32/bf16 with
 * round-to-nearest-even, or back). */
wk_status wk_convert(const void *src, int src_dtype, void *dst, int dst_dtype, int64_t n,
                     void *stream);

#ifdef __cplusplus
}
#endif
#endif /* WK_CAPI_H */
