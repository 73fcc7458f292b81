"""Python mirror of the reference's warpkernel.hpp surface over the C ABI.

    structure   -> warpkernel::structure   (WPK1 scan, reorder_*; warpkernel.hpp:215-551)
    structure2  -> warpkernel::structure2  (WPK2 scan with threshold; 553-771)
    engine      -> warpkernel::engine      (process, run, run_x, verify, verify_x; 773-959)
    profiler, stats                         (961-1022)

The layout is built on the GPU; its public arrays (row_map, reorder_rows,
...) are fetched from the device on first access as numpy arrays, so driver
code that reads them keeps working.  Vectors passed to run / run_x are CUDA
torch tensors (or raw device pointers), as the reference takes device arrays.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import (WK_BF16, WK_F16S, WK_F32, WK_F64, WK_ORDER_EXACT, WK_ORDER_FAST, WK_WPK1, WK_WPK2,
                   LayoutInfo, check, load)

__all__ = ["structure", "structure2", "engine", "profiler", "stats", "DTYPES",
           "WK_ORDER_FAST", "WK_ORDER_EXACT", "csr_matrix", "read_matrix_market_file"]

DTYPES = {"f64": WK_F64, "float64": WK_F64, "f32": WK_F32, "float32": WK_F32,
          "bf16": WK_BF16, "bfloat16": WK_BF16, "f16s": WK_F16S}
_NP_FIELD_DT = {"row_map": np.int32, "row_map_inv": np.int32, "reorder_rows": np.uint32,
                "warp_offsets": np.int32, "max_nz_rows": np.uint32,
                "threads_per_row": np.uint32, "row_offset_warp": np.uint32}


def _ptr(a):
    """Address of a numpy array, torch tensor or raw integer pointer."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    raise TypeError(f"cannot take the address of {type(a)}")


def _stream_ptr(stream):
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except ImportError:
            pass
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class structure:
    """WPK1 layout (warpkernel::structure)."""

    kind = WK_WPK1

    def __init__(self):
        self._h = None
        self._info = None
        self._cache = {}

    # -- scan --------------------------------------------------------------
    def scan(self, nz, nrows, A=None, rows=None, colinds=None, stream=None):
        """structure::scan(nz, nrows, A, rows, colinds) (warpkernel.hpp:309-365).
        Only `rows` (the CSR row offsets, host or device) is used, as in the
        reference."""
        if rows is None:
            raise ValueError("rows (CSR row offsets) are required")
        if isinstance(rows, np.ndarray):
            rows = np.ascontiguousarray(rows, dtype=np.int32)
        self._release()
        h = C.c_void_p()
        check(load().wk_scan1(_ptr(rows), int(nrows), int(nz), _stream_ptr(stream), C.byref(h)))
        self._set(h)
        return self

    def scan_ablation(self, nz, nrows, rows, flags, stream=None):
        """The WPK1 ablation layouts of optimization.cu: flags WK_ABL_NOSORT
        (scan_nosort, rows in CSR order), WK_ABL_NOCOALESCE (scan_nocoalesced,
        each lane's entries contiguous) or both (scan_nocoalesced_nosort)."""
        if self.kind != WK_WPK1:
            raise ValueError("the ablation layouts are WPK1 layouts")
        if isinstance(rows, np.ndarray):
            rows = np.ascontiguousarray(rows, dtype=np.int32)
        self._release()
        h = C.c_void_p()
        check(load().wk_scan1_ablation(_ptr(rows), int(nrows), int(nz), int(flags), _stream_ptr(stream),
                                       C.byref(h)))
        self._set(h)
        return self

    variant = property(lambda s: s._info.variant)

    def _set(self, h):
        self._h = h
        info = LayoutInfo()
        check(load().wk_layout_info_get(h, C.byref(info)))
        self._info = info
        self._cache = {}

    def _release(self):
        if self._h:
            load().wk_layout_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass

    @property
    def handle(self):
        if not self._h:
            raise RuntimeError("structure has not been scanned")
        return self._h

    # -- reference public fields ------------------------------------------
    def _field(self, name):
        if name not in self._cache:
            L = load()
            n = C.c_size_t()
            check(L.wk_layout_get(self.handle, _lib.FIELDS[name], None, 0, C.byref(n)))
            a = np.zeros(n.value, _NP_FIELD_DT[name])
            if n.value:
                check(L.wk_layout_get(self.handle, _lib.FIELDS[name], a.ctypes.data, n.value, None))
            self._cache[name] = a
        return self._cache[name]

    row_map = property(lambda s: s._field("row_map"))
    row_map_inv = property(lambda s: s._field("row_map_inv"))
    reorder_rows = property(lambda s: s._field("reorder_rows"))
    warp_offsets = property(lambda s: s._field("warp_offsets"))
    max_nz_rows = property(lambda s: s._field("max_nz_rows"))
    nrows = property(lambda s: s._info.nrows)
    nznrows = property(lambda s: s._info.nznrows)
    nz = property(lambda s: s._info.nz)
    allocate_nz = property(lambda s: s._info.allocate_nz)
    nwarps = property(lambda s: s._info.nwarps)

    # -- reorderings ----------------------------------------------------------
    def reorder_columns_coalesced(self, colinds, out=None, stream=None):
        """warpkernel.hpp:447-457: returns allocate_nz padded, renumbered columns."""
        colinds = _host_or_dev(colinds, np.int32)
        if out is None:
            out = np.zeros(self.allocate_nz, np.int32) if isinstance(colinds, np.ndarray) else \
                _empty_like_dev(colinds, self.allocate_nz)
        check(load().wk_reorder_columns_coalesced(self.handle, _ptr(colinds), _ptr(out),
                                                  _stream_ptr(stream)))
        return out

    def reorder_columns(self, colinds, out=None, stream=None):
        """warpkernel.hpp:401-412: nz renumbered columns in CSR order."""
        colinds = _host_or_dev(colinds, np.int32)
        if out is None:
            out = np.zeros(self.nz, np.int32) if isinstance(colinds, np.ndarray) else \
                _empty_like_dev(colinds, self.nz)
        check(load().wk_reorder_columns(self.handle, _ptr(colinds), _ptr(out), _stream_ptr(stream)))
        return out

    def process(self, A=None, colinds=None, dtype="f64", stream=None):
        """structure::reorder / process (warpkernel.hpp:380-398, 533-548): the
        padded values and columns (padding 0) as (pvals, pcols); either input
        may be None.  Host arrays in, host arrays out; CUDA tensors in, CUDA
        tensors out."""
        dt = DTYPES[dtype] if isinstance(dtype, str) else int(dtype)
        if dt not in (WK_F64, WK_F32, WK_BF16):
            raise ValueError("process: dtype must be f64, f32 or bf16")
        ref = A if A is not None else colinds
        host = isinstance(ref, np.ndarray)
        pv = pc = None
        if A is not None:
            A = _host_or_dev(A, {WK_F64: np.float64, WK_F32: np.float32, WK_BF16: np.uint16}[dt])
            pv = np.zeros(self.allocate_nz, A.dtype) if host else _empty_like_dev(A, self.allocate_nz)
        if colinds is not None:
            colinds = _host_or_dev(colinds, np.int32)
            pc = np.zeros(self.allocate_nz, np.int32) if host else _empty_like_dev(colinds, self.allocate_nz)
        check(load().wk_process(self.handle, dt, _ptr(A), _ptr(colinds), _ptr(pv), _ptr(pc), _stream_ptr(stream)))
        return pv, pc

    def reorder_values_coalesced(self, values, dtype="f64"):
        """warpkernel.hpp:470-491: the padded value array alone."""
        return self.process(values, None, dtype)[0]

    def reorder_columns_rowsort(self, colinds, rows=None, out=None, stream=None):
        """warpkernel.hpp:414-444: nz renumbered columns sorted within each
        CSR row; sets self.reorder_A_rows to the CSR position each came from
        (host arrays in, host arrays out; CUDA tensors in, CUDA tensors out).
        `rows` is accepted for the reference's signature; the layout keeps its
        own copy of the row offsets."""
        colinds = _host_or_dev(colinds, np.int32)
        host = isinstance(colinds, np.ndarray)
        if out is None:
            out = np.zeros(self.nz, np.int32) if host else _empty_like_dev(colinds, self.nz)
        src = np.zeros(self.nz, np.int32) if host else _empty_like_dev(colinds, self.nz)
        check(load().wk_reorder_columns_rowsort(self.handle, _ptr(colinds), _ptr(out), _ptr(src),
                                                _stream_ptr(stream)))
        self.reorder_A_rows = src
        return out

    def reorder_values_coalesced_rowsort(self, values):
        """warpkernel.hpp:505-515 ([CPU] in the reference too): the padded
        slot array new_values[reorder_rows[i]] = values[reorder_A_rows[i]]."""
        src = getattr(self, "reorder_A_rows", None)
        if src is None:
            raise RuntimeError("reorder_columns_rowsort has not been called")
        src = src if isinstance(src, np.ndarray) else src.cpu().numpy()
        values = np.asarray(values)
        out = np.zeros(self.allocate_nz, values.dtype)
        out[self.reorder_rows] = values[src]
        return out

    def save(self, path):
        """Writes the layout (structure::serialize's fields, warpkernel.hpp:253-269)."""
        check(load().wk_layout_save(self.handle, str(path).encode()))

    def load(self, path, stream=None):
        """Replaces this structure by a layout written with save(); the file
        must hold a layout of this class's kind."""
        h = C.c_void_p()
        check(load().wk_layout_load(str(path).encode(), _stream_ptr(stream), C.byref(h)))
        info = LayoutInfo()
        check(load().wk_layout_info_get(h, C.byref(info)))
        if info.kind != self.kind:
            load().wk_layout_destroy(h)
            raise ValueError(f"{path} holds a WPK{info.kind} layout, not WPK{self.kind}")
        self._release()
        self._set(h)
        return self

    def reorder_x(self, x, device_x=None, stream=None):
        """warpkernel.hpp:518-530: device_x[row_map_inv[r]] = x[r].  Returns a
        CUDA tensor unless `device_x` is given."""
        import torch
        if isinstance(x, np.ndarray):
            x = torch.from_numpy(np.ascontiguousarray(x))
        dt = {torch.float64: WK_F64, torch.float32: WK_F32, torch.bfloat16: WK_BF16}[x.dtype]
        if device_x is None:
            device_x = torch.empty(self.nrows, dtype=x.dtype, device="cuda")
        check(load().wk_reorder_x(self.handle, dt, _ptr(x), _ptr(device_x), _stream_ptr(stream)))
        return device_x

    def info(self):
        i = self._info
        return {k: getattr(i, k) for k, _ in LayoutInfo._fields_}


class structure2(structure):
    """WPK2 layout (warpkernel::structure2)."""

    kind = WK_WPK2

    def scan(self, nz, nrows, A=None, rows=None, colinds=None, threshold=None, stream=None):
        """structure2::scan(nz, nrows, A, rows, colinds, threshold) (579-736)."""
        if rows is None or threshold is None:
            raise ValueError("rows and threshold are required")
        if isinstance(rows, np.ndarray):
            rows = np.ascontiguousarray(rows, dtype=np.int32)
        self._release()
        h = C.c_void_p()
        check(load().wk_scan2(_ptr(rows), int(nrows), int(nz), int(threshold), _stream_ptr(stream),
                              C.byref(h)))
        self._set(h)
        return self

    row_offset_warp = property(lambda s: s._field("row_offset_warp"))
    threads_per_row = property(lambda s: s._field("threads_per_row"))
    nmax_per_thread = property(lambda s: s._info.nmax_per_thread)
    min_nz = property(lambda s: s._info.min_nz)
    max_nz = property(lambda s: s._info.max_nz)


def _host_or_dev(a, dt):
    if isinstance(a, np.ndarray):
        return np.ascontiguousarray(a, dtype=dt)
    return a


def _empty_like_dev(t, n):
    import torch
    return torch.empty(n, dtype=t.dtype, device=t.device)


class engine:
    """warpkernel::engine<ValueType, IndexType>: owns the padded device arrays."""

    def __init__(self, k: structure, A=None, colinds=None, dtype="f64", ncols=None, stream=None):
        self.kernel = k
        self._h = None
        self.dtype = DTYPES[dtype] if isinstance(dtype, str) else int(dtype)
        self.ncols = k.nrows if ncols is None else int(ncols)
        if A is None:
            return  # engine(structure&) of the reference: no arrays yet
        A = _host_or_dev(A, {WK_F64: np.float64, WK_F32: np.float32, WK_F16S: np.float32}.get(self.dtype,
                                                                                            np.uint16))
        colinds = _host_or_dev(colinds, np.int32)
        ncols = k.nrows if ncols is None else int(ncols)
        h = C.c_void_p()
        check(load().wk_engine_create(k.handle, self.dtype, _ptr(A), _ptr(colinds), ncols,
                                      _stream_ptr(stream), C.byref(h)))
        self._h = h
        self.ncols = ncols

    def __del__(self):
        try:
            if self._h:
                load().wk_engine_destroy(self._h)
        except Exception:
            pass
        self._h = None

    @property
    def handle(self):
        if not self._h:
            raise RuntimeError("engine has no device arrays (constructed without A and colinds)")
        return self._h

    # device_colinds / device_values of the reference (warpkernel.hpp:782-783)
    @property
    def device_colinds(self):
        a = np.zeros(self.kernel.allocate_nz, np.int32)
        check(load().wk_engine_get_colinds(self.handle, a.ctypes.data, a.size))
        return a

    @device_colinds.setter
    def device_colinds(self, cols):
        cols = _host_or_dev(cols, np.int32)
        check(load().wk_engine_set_colinds(self.handle, _ptr(cols), _stream_ptr(None)))

    @property
    def device_values(self):
        dt = {WK_F64: np.float64, WK_F32: np.float32, WK_BF16: np.uint16, WK_F16S: np.float32}[self.dtype]
        a = np.zeros(self.kernel.allocate_nz, dt)
        check(load().wk_engine_get_values(self.handle, a.ctypes.data, a.size))
        return a

    def compress_cols(self, stream=None):
        """16-bit column offsets for warps spanning < 65,536 columns (fast
        order); returns the number of warps left with 32-bit indices."""
        wide = C.c_uint32(0)
        check(load().wk_engine_compress_cols(self.handle, _stream_ptr(stream), C.byref(wide)))
        return int(wide.value)

    def set_windows(self, on=True):
        """x windows of the compact column storage on or off (fast order; the
        same bits either way; on by default for f32 and f16s engines, built by
        compress_cols); returns the number of warps that have one."""
        n = C.c_uint32(0)
        check(load().wk_engine_set_windows(self.handle, int(bool(on)), C.byref(n)))
        return int(n.value)

    def set_values(self, A, stream=None):
        check(load().wk_engine_set_values(self.handle, _ptr(A), _stream_ptr(stream)))

    _XDT = {WK_F64: "torch.float64", WK_F32: "torch.float32", WK_BF16: "torch.bfloat16", WK_F16S: "torch.float32"}
    _YDT = {WK_F64: "torch.float64", WK_F32: "torch.float32", WK_BF16: "torch.float32", WK_F16S: "torch.float32"}

    def _check_vectors(self, dx, dy, mapped):
        """Sizes and element types of tensor arguments (raw pointers cannot be
        checked and are taken as given, as the C ABI does)."""
        if hasattr(dx, "numel"):
            if not dx.is_cuda:
                raise ValueError("dx must be a CUDA tensor (use run_host for host vectors)")
            if str(dx.dtype) != self._XDT[self.dtype] or dx.numel() < self.ncols:
                raise ValueError(f"dx must hold >= {self.ncols} values of {self._XDT[self.dtype]}")
        if hasattr(dy, "numel"):
            if not dy.is_cuda:
                raise ValueError("dy must be a CUDA tensor")
            if str(dy.dtype) != self._YDT[self.dtype] or dy.numel() < self.kernel.nrows:
                raise ValueError(f"dy must hold >= {self.kernel.nrows} values of {self._YDT[self.dtype]}")

    def _run(self, fn, nblocks, blocksize, dx, dy, cache, order, stream, timed):
        self._check_vectors(dx, dy, True)
        sec = C.c_float(0.0)
        check(fn(self.handle, int(nblocks), int(blocksize), int(cache), int(order), _ptr(dx), _ptr(dy),
                 _stream_ptr(stream), C.byref(sec) if timed else None))
        return float(sec.value) if timed else None

    def run(self, nblocks, blocksize, dx, dy, cache=True, order=WK_ORDER_FAST, stream=None, timed=True):
        """engine::run<cache>(nblocks, blocksize, dx, dy): y[row_map[p]] = row sums.
        Returns seconds (synchronous) like the reference, or None with timed=False."""
        return self._run(load().wk_run, nblocks, blocksize, dx, dy, cache, order, stream, timed)

    def run_x(self, nblocks, blocksize, dx, dy, cache=True, order=WK_ORDER_FAST, stream=None, timed=True):
        """engine::run_x<cache>: y'[p] = sorted-row sums (reordered x)."""
        return self._run(load().wk_run_x, nblocks, blocksize, dx, dy, cache, order, stream, timed)

    def run_assembly(self, nblocks, blocksize, dy, cache=True, stream=None, timed=True):
        """engine::run_assembly<cache>(nblocks, blocksize, dy)
        (warpkernel.hpp:898-929): y[row_map[p]] = sum of row p's values."""
        self._check_vectors(None, dy, True)
        sec = C.c_float(0.0)
        check(load().wk_run_assembly(self.handle, int(nblocks), int(blocksize), _ptr(dy), _stream_ptr(stream),
                                     C.byref(sec) if timed else None))
        return float(sec.value) if timed else None

    def run_host(self, x_host, y_host, mapped=True, order=WK_ORDER_FAST, stream=None):
        """H2D of x, run (or run_x with mapped=False), D2H of y in one
        synchronous library call; x_host / y_host are host arrays (pinned
        tensors give the fastest copies)."""
        check(load().wk_run_host(self.handle, int(mapped), int(order), _ptr(x_host), _ptr(y_host),
                                 _stream_ptr(stream)))
        return y_host

    def run_host_stream(self, xs, ys, mapped=True, order=WK_ORDER_FAST, stream=None):
        """run_host over a sequence of host vectors with the copies of
        neighbouring steps overlapping each SpMV (double-buffered); returns
        the elapsed seconds of the whole sequence."""
        if len(xs) != len(ys):
            raise ValueError("xs and ys must have the same length")
        n = len(xs)
        xp = (C.c_void_p * max(n, 1))(*[_ptr(x) for x in xs])
        yp = (C.c_void_p * max(n, 1))(*[_ptr(y) for y in ys])
        sec = C.c_float(0.0)
        check(load().wk_run_host_stream(self.handle, int(mapped), int(order), n, xp, yp, _stream_ptr(stream),
                                        C.byref(sec)))
        return float(sec.value)

    def residual(self, x, b, r, norm2=None, stream=None):
        """r = b - A x (fp64 engine, device tensors); norm2: optional 1-element
        float64 CUDA tensor receiving ||r||^2."""
        check(load().wk_residual(self.handle, _ptr(x), _ptr(b), _ptr(r), _ptr(norm2), _stream_ptr(stream)))
        return r

    def verify(self, orig, comp):
        """engine::verify (warpkernel.hpp:932-943) on host arrays."""
        o = np.ascontiguousarray(orig, np.float64)
        c = np.ascontiguousarray(comp, np.float64)
        ok, bad = C.c_int(), C.c_int64()
        check(load().wk_verify(self.kernel.handle, o.ctypes.data, c.ctypes.data, C.byref(ok), C.byref(bad)))
        if not ok.value:
            i = bad.value
            print(f"verify: {o[i]}\t{c[i]}\t{i}")
        return bool(ok.value)

    def verify_x(self, orig, comp, strict=False):
        """engine::verify_x (warpkernel.hpp:945-957) on host arrays."""
        o = np.ascontiguousarray(orig, np.float64)
        c = np.ascontiguousarray(comp, np.float64)
        ok, bad = C.c_int(), C.c_int64()
        check(load().wk_verify_x(self.kernel.handle, o.ctypes.data, c.ctypes.data, int(strict), C.byref(ok),
                                 C.byref(bad)))
        return bool(ok.value)


class csr_matrix:
    """Host CSR matrix with cusp::csr_matrix's member names."""

    def __init__(self, row_offsets, column_indices, values, num_cols=None):
        self.row_offsets = np.ascontiguousarray(row_offsets, np.int32)
        self.column_indices = np.ascontiguousarray(column_indices, np.int32)
        self.values = np.ascontiguousarray(values)
        self.num_rows = len(self.row_offsets) - 1
        self.num_cols = self.num_rows if num_cols is None else int(num_cols)
        self.num_entries = len(self.column_indices)


def read_matrix_market_file(path) -> csr_matrix:
    """cusp::io::read_matrix_market_file as the drivers call it (wpk1.cu:43-48,
    wpk2.cu:54-57): coordinate real/integer/pattern, general / symmetric /
    skew-symmetric, returned as CSR sorted by row, then column.  Runs in the
    library (no CUDA call)."""
    L = load()
    h = C.c_void_p()
    check(L.wk_mm_read(str(path).encode(), C.byref(h)))
    try:
        n, m, z = C.c_int64(), C.c_int64(), C.c_int64()
        rp, ci, v = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(L.wk_csr_get(h, C.byref(n), C.byref(m), C.byref(z), C.byref(rp), C.byref(ci), C.byref(v)))

        def arr(p, cnt, dt):
            if cnt == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                         shape=(cnt,)).copy()
        return csr_matrix(arr(rp, n.value + 1, np.int32), arr(ci, z.value, np.int32),
                          arr(v, z.value, np.float64), m.value)
    finally:
        L.wk_csr_free(h)


def _cg_params(tol, max_iter, max_inner, inner_tol, check_every):
    p = _lib.CGParams()
    p.tol, p.max_iter, p.max_inner, p.inner_tol, p.check_every = tol, max_iter, max_inner, inner_tol, check_every
    return p


def _cg_result(p, status):
    res = {"iters": p.iters, "outer": p.outer, "relres": p.relres, "seconds": p.seconds,
           "converged": status == 0}
    if status not in (0, 7):  # WK_ERR_NOTCONV is reported in the result
        check(status)
    return res


def cg(eng64, b, x, tol=1e-10, max_iter=100000, check_every=10, stream=None):
    """fp64 conjugate gradient on an fp64 engine (device vectors b, x; x is
    the initial guess and is overwritten)."""
    p = _cg_params(tol, max_iter, 0, 0.0, check_every)
    st = load().wk_cg(eng64.handle, _ptr(b), _ptr(x), C.byref(p), _stream_ptr(stream))
    return _cg_result(p, st)


def ir_cg(eng64, eng_lo, b, x, tol=1e-10, max_outer=50, max_inner=2000, inner_tol=1e-4, check_every=10,
          stream=None, inner_dots="fp64"):
    """Iterative refinement: fp64 residual / dots / update, fp32 inner CG on
    the low-precision engine (WK_F32, WK_BF16 or WK_F16S values) whose dot
    products are summed in FP64 (inner_dots="fp64") or in FP32 within each
    block ("fp32")."""
    if inner_dots not in ("fp64", "fp32"):
        raise ValueError("inner_dots must be 'fp64' or 'fp32'")
    p = _cg_params(tol, max_outer, max_inner, inner_tol, check_every)
    p.inner_dots_fp32 = 1 if inner_dots == "fp32" else 0
    st = load().wk_ir_cg(eng64.handle, eng_lo.handle, _ptr(b), _ptr(x), C.byref(p), _stream_ptr(stream))
    return _cg_result(p, st)


class profiler:
    """Running mean of timings (warpkernel.hpp:963-982)."""

    def __init__(self):
        self.sum = 0.0
        self.count = 0

    def add(self, secs):
        self.sum += secs
        self.count += 1

    def avg(self):
        return self.sum / self.count if self.count else math.nan


class stats:
    """Labelled min / max (warpkernel.hpp:984-1022)."""

    def __init__(self):
        self.min_, self.max_ = float("inf"), 0.0
        self.min_str_, self.max_str_ = "", ""

    def add(self, val, ident=""):
        if val < self.min_:
            self.min_, self.min_str_ = val, ident
        if val > self.max_:
            self.max_, self.max_str_ = val, ident

    def Min(self):
        return self.min_

    def Min_str(self):
        return self.min_str_

    def Max(self):
        return self.max_

    def Max_str(self):
        return self.max_str_
