"""ctypes binding for the CPU oracle (libwk_oracle.so) and, where it was built,
the reference's own host scan compiled for the CPU (oracle/_ref/libwkref*.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU arms, to check the CUDA path.  The product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwk_oracle.so")
REF_PATHS = {
    "mul_add": os.path.join(HERE, "_ref", "libwkref.so"),
    "fma": os.path.join(HERE, "_ref", "libwkref_fma.so"),
}

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")


class _Layout(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("nrows", C.c_uint32), ("nznrows", C.c_uint32), ("nz", C.c_uint32),
        ("allocate_nz", C.c_uint32), ("nwarps", C.c_uint32),
        ("min_nz", C.c_uint32), ("max_nz", C.c_uint32), ("nmax_per_thread", C.c_uint32),
        ("variant", C.c_uint32),
        ("row_map", C.POINTER(C.c_int32)), ("row_map_inv", C.POINTER(C.c_int32)),
        ("reorder_rows", C.POINTER(C.c_uint32)), ("warp_offsets", C.POINTER(C.c_int32)),
        ("max_nz_rows", C.POINTER(C.c_uint32)), ("threads_per_row", C.POINTER(C.c_uint32)),
        ("row_offset_warp", C.POINTER(C.c_uint32)),
    ]


_lib = None


def lib():
    """Load libwk_oracle.so (building it with make if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import subprocess
            subprocess.check_call(["make", "-s", "-C", HERE, "libwk_oracle.so"])
        L = C.CDLL(LIB_PATH)
        lp = C.POINTER(_Layout)
        L.wko_scan1.argtypes = [_i32p, C.c_uint32, C.c_uint32, lp]
        L.wko_scan2.argtypes = [_i32p, C.c_uint32, C.c_uint32, C.c_int32, lp]
        L.wko_scan1_ablation.argtypes = [_i32p, C.c_uint32, C.c_uint32, C.c_int, lp]
        L.wko_free.argtypes = [lp]
        L.wko_process_f64.argtypes = [lp, _f64p, _i32p, _f64p, _i32p]
        L.wko_process_f32.argtypes = [lp, _f32p, _i32p, _f32p, _i32p]
        L.wko_reorder_columns_coalesced.argtypes = [lp, _i32p, _i32p]
        L.wko_reorder_columns.argtypes = [lp, _i32p, _i32p]
        L.wko_reorder_x_f64.argtypes = [lp, _f64p, _f64p]
        L.wko_reorder_columns_rowsort.argtypes = [lp, _i32p, _i32p, _i32p, _i32p]
        L.wko_assembly_f64.argtypes = [lp, _f64p, _f64p]
        L.wko_run_f64.argtypes = [lp, _f64p, _i32p, _f64p, _f64p, C.c_int]
        L.wko_run_x_f64.argtypes = [lp, _f64p, _i32p, _f64p, _f64p, C.c_int]
        L.wko_run_f64_omp.argtypes = [lp, _f64p, _i32p, _f64p, _f64p, C.c_int]
        L.wko_csr_spmv_f64.argtypes = [_i32p, _i32p, _f64p, _f64p, _f64p, C.c_uint32, C.c_int]
        L.wko_csr_spmv_t_f64.argtypes = [_i32p, _i32p, _f64p, _f64p, _f64p, C.c_uint32, C.c_uint32]
        L.wko_verify.argtypes = [C.c_uint32, _f64p, _f64p, C.POINTER(C.c_long)]
        L.wko_verify_x.argtypes = [lp, _f64p, _f64p, C.POINTER(C.c_long)]
        L.wko_max_threads.restype = C.c_int
        L.wko_round_f32.argtypes = [_f64p, _f32p, C.c_int64]
        L.wko_round_bf16.argtypes = [_f64p, _u16p, C.c_int64]
        L.wko_run_lp.argtypes = [lp, C.c_int, C.c_void_p, _i32p, C.c_void_p, _f32p, C.c_int, C.c_int]
        L.wko_fe_size.argtypes = [C.c_int] * 5 + [C.POINTER(C.c_int64)] * 2
        L.wko_fe_fill.argtypes = [C.c_int] * 6 + [C.c_uint64, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_int]
        L.wko_uniform_vec.argtypes = [C.c_uint64, C.c_uint64, _f64p, C.c_int64]
        _lib = L
    return _lib


@dataclass
class Layout:
    """Host copy of a WPK1/WPK2 layout (field names of warpkernel.hpp:276-286, 561-565)."""
    kind: int
    nrows: int
    nznrows: int
    nz: int
    allocate_nz: int
    nwarps: int
    min_nz: int = 0
    max_nz: int = 0
    nmax_per_thread: int = 0
    arrays: dict = field(default_factory=dict)
    _c: object = None  # the C struct, kept for calls that take the layout

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays", {})
        if name in arrays:
            return arrays[name]
        raise AttributeError(name)


FIELDS = ("row_map", "row_map_inv", "reorder_rows", "warp_offsets", "max_nz_rows",
          "threads_per_row", "row_offset_warp")


def _wrap(c: _Layout) -> Layout:
    n, W, nz = c.nrows, c.nwarps, c.nz

    def arr(ptr, count, dt):
        if count == 0 or not ptr:
            return np.zeros(0, dt)
        return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dt, copy=True)

    a = {
        "row_map": arr(c.row_map, n, np.int32),
        "row_map_inv": arr(c.row_map_inv, n, np.int32),
        "reorder_rows": arr(c.reorder_rows, nz, np.uint32),
        "warp_offsets": arr(c.warp_offsets, W + 1, np.int32),
        "max_nz_rows": arr(c.max_nz_rows, W, np.uint32),
    }
    if c.kind == 2:
        a["threads_per_row"] = arr(c.threads_per_row, W, np.uint32)
        a["row_offset_warp"] = arr(c.row_offset_warp, W + 1, np.uint32)
    else:
        a["threads_per_row"] = np.zeros(0, np.uint32)
        a["row_offset_warp"] = np.zeros(0, np.uint32)
    return Layout(c.kind, c.nrows, c.nznrows, c.nz, c.allocate_nz, c.nwarps,
                  c.min_nz, c.max_nz, c.nmax_per_thread, a, c)


class OracleLayout:
    """Owns a C layout; use as a context manager or call free()."""

    def __init__(self, rowptr, nz=None, kind=1, threshold=0, ablation=0):
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        nrows = len(rowptr) - 1
        nz = int(rowptr[-1]) if nz is None else int(nz)
        self.c = _Layout()
        L = lib()
        if ablation:
            if kind != 1:
                raise ValueError("the ablation layouts are WPK1 layouts")
            rc = L.wko_scan1_ablation(rowptr, nrows, nz, int(ablation), C.byref(self.c))
        elif kind == 1:
            rc = L.wko_scan1(rowptr, nrows, nz, C.byref(self.c))
        else:
            rc = L.wko_scan2(rowptr, nrows, nz, int(threshold), C.byref(self.c))
        if rc:
            L.wko_free(C.byref(self.c))
            raise ValueError(f"oracle scan rejected the input (code {rc})")
        self.layout = _wrap(self.c)

    def free(self):
        if self.c is not None:
            lib().wko_free(C.byref(self.c))
            self.c = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.free()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    # --- process / reorder -------------------------------------------------
    def process(self, vals, cols):
        L = self.layout
        vals = np.ascontiguousarray(vals)
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        pc = np.zeros(L.allocate_nz, np.int32)
        if vals.dtype == np.float32:
            pv = np.zeros(L.allocate_nz, np.float32)
            lib().wko_process_f32(C.byref(self.c), vals, cols, pv, pc)
        else:
            vals = vals.astype(np.float64, copy=False)
            pv = np.zeros(L.allocate_nz, np.float64)
            lib().wko_process_f64(C.byref(self.c), vals, cols, pv, pc)
        return pv, pc

    def reorder_columns_coalesced(self, cols):
        out = np.zeros(self.layout.allocate_nz, np.int32)
        lib().wko_reorder_columns_coalesced(C.byref(self.c), np.ascontiguousarray(cols, np.int32), out)
        return out

    def reorder_columns(self, cols):
        out = np.zeros(self.layout.nz, np.int32)
        lib().wko_reorder_columns(C.byref(self.c), np.ascontiguousarray(cols, np.int32), out)
        return out

    def reorder_x(self, x):
        out = np.zeros(self.layout.nrows, np.float64)
        lib().wko_reorder_x_f64(C.byref(self.c), np.ascontiguousarray(x, np.float64), out)
        return out

    def reorder_columns_rowsort(self, rowptr, cols):
        """warpkernel.hpp:414-444 -> (renumbered row-sorted columns, reorder_A_rows)."""
        out = np.zeros(self.layout.nz, np.int32)
        src = np.zeros(self.layout.nz, np.int32)
        lib().wko_reorder_columns_rowsort(C.byref(self.c), np.ascontiguousarray(rowptr, np.int32),
                                          np.ascontiguousarray(cols, np.int32), out, src)
        return out, src

    def assembly(self, pvals, y=None):
        """warpKernel_assembly (warpkernel.hpp:78-100): row sums of the padded values."""
        y = np.zeros(self.layout.nrows, np.float64) if y is None else y
        lib().wko_assembly_f64(C.byref(self.c), np.ascontiguousarray(pvals, np.float64), y)
        return y

    # --- arithmetic ----------------------------------------------------------
    def run(self, pvals, pcols, x, y=None, fma=True):
        y = np.zeros(self.layout.nrows, np.float64) if y is None else y
        lib().wko_run_f64(C.byref(self.c), np.ascontiguousarray(pvals, np.float64),
                          np.ascontiguousarray(pcols, np.int32),
                          np.ascontiguousarray(x, np.float64), y, int(fma))
        return y

    def run_x(self, pvals, pcols, x, y=None, fma=True):
        y = np.zeros(self.layout.nrows, np.float64) if y is None else y
        lib().wko_run_x_f64(C.byref(self.c), np.ascontiguousarray(pvals, np.float64),
                            np.ascontiguousarray(pcols, np.int32),
                            np.ascontiguousarray(x, np.float64), y, int(fma))
        return y

    def run_lp(self, pvals, pcols, x, mapped=True, y=None, nthreads=0):
        """Documented order in FP32 (wko_run_lp): pvals / x float32 (FP32
        storage) or uint16 bf16 bits (BF16 storage); returns float32 y."""
        pvals = np.ascontiguousarray(pvals)
        x = np.ascontiguousarray(x)
        if pvals.dtype == np.float32 and x.dtype == np.float32:
            vt = 0
        elif pvals.dtype == np.uint16 and x.dtype == np.uint16:
            vt = 1
        else:
            raise TypeError("pvals and x must both be float32 or both uint16 (bf16 bits)")
        y = np.zeros(self.layout.nrows, np.float32) if y is None else y
        lib().wko_run_lp(C.byref(self.c), vt, pvals.ctypes.data, np.ascontiguousarray(pcols, np.int32),
                         x.ctypes.data, y, int(mapped), int(nthreads))
        return y

    def place(self, vals):
        """structure::reorder for any element type: vals (CSR order) placed at
        reorder_rows, padding slots 0 (warpkernel.hpp:385-394)."""
        out = np.zeros(self.layout.allocate_nz, np.asarray(vals).dtype)
        out[self.layout.reorder_rows] = vals
        return out

    def run_omp(self, pvals, pcols, x, y, nthreads=0):
        lib().wko_run_f64_omp(C.byref(self.c), pvals, pcols, x, y, int(nthreads))
        return y

    def verify(self, orig, comp):
        bad = C.c_long(-1)
        ok = lib().wko_verify(self.layout.nrows, np.ascontiguousarray(orig, np.float64),
                              np.ascontiguousarray(comp, np.float64), C.byref(bad))
        return bool(ok), bad.value

    def verify_x(self, orig, comp):
        bad = C.c_long(-1)
        ok = lib().wko_verify_x(C.byref(self.c), np.ascontiguousarray(orig, np.float64),
                                np.ascontiguousarray(comp, np.float64), C.byref(bad))
        return bool(ok), bad.value


def csr_spmv(rowptr, cols, vals, x, nthreads=0):
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    y = np.zeros(len(rowptr) - 1, np.float64)
    lib().wko_csr_spmv_f64(rowptr, np.ascontiguousarray(cols, np.int32),
                           np.ascontiguousarray(vals, np.float64),
                           np.ascontiguousarray(x, np.float64), y, len(rowptr) - 1, int(nthreads))
    return y


def csr_spmv_t(rowptr, cols, vals, x, ncols):
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    y = np.zeros(ncols, np.float64)
    lib().wko_csr_spmv_t_f64(rowptr, np.ascontiguousarray(cols, np.int32),
                             np.ascontiguousarray(vals, np.float64),
                             np.ascontiguousarray(x, np.float64), y, len(rowptr) - 1, ncols)
    return y


def round_f32(x):
    """fp64 -> FP32, round-to-nearest-even (the library's conversion)."""
    x = np.ascontiguousarray(x, np.float64)
    out = np.zeros(len(x), np.float32)
    lib().wko_round_f32(x, out, len(x))
    return out


def round_bf16(x):
    """fp64 -> BF16 bits (uint16), round-to-nearest-even in one step."""
    x = np.ascontiguousarray(x, np.float64)
    out = np.zeros(len(x), np.uint16)
    lib().wko_round_bf16(x, out, len(x))
    return out


def bf16_to_f32(b):
    """BF16 bits (uint16) -> float32 (exact)."""
    return (np.ascontiguousarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


def max_threads():
    return int(lib().wko_max_threads())


# --- finite-element test matrices (CPU generator) ------------------------------

def fe_size(dim, ex, ey, ez, dof):
    n = C.c_int64()
    z = C.c_int64()
    if lib().wko_fe_size(dim, ex, ey, ez, dof, C.byref(n), C.byref(z)):
        raise ValueError("bad mesh")
    return n.value, z.value


def fe_matrix(dim, ex, ey, ez=0, dof=1, value_mode=1, seed=0, nthreads=0):
    """(rowptr int32, cols int32, vals float64) of the FE test matrix."""
    n, z = fe_size(dim, ex, ey, ez, dof)
    rowptr = np.zeros(n + 1, np.int32)
    cols = np.zeros(z, np.int32)
    vals = np.zeros(z, np.float64)
    rc = lib().wko_fe_fill(dim, ex, ey, ez, dof, value_mode, seed, rowptr.ctypes.data,
                           cols.ctypes.data, vals.ctypes.data, int(nthreads))
    if rc:
        raise ValueError(f"fe_fill failed ({rc})")
    return rowptr, cols, vals


def uniform_vec(seed, stream, n):
    x = np.zeros(n, np.float64)
    lib().wko_uniform_vec(seed, stream, x, n)
    return x


# --- the reference's own scan, compiled from its sources (only where built) ----

class RefLib:
    """The reference's structure/structure2 and WPK1 kernels, run on the CPU."""

    def __init__(self, variant="mul_add"):
        path = REF_PATHS[variant]
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        L.ref_scan.restype = C.c_void_p
        L.ref_scan.argtypes = [_i32p, C.c_uint, C.c_uint, C.c_int, C.c_int]
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_info.argtypes = [C.c_void_p, _u32p]
        L.ref_field.restype = C.c_long
        L.ref_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.ref_process.argtypes = [C.c_void_p, _f64p, _i32p, _f64p, _i32p]
        L.ref_reorder_columns_coalesced.argtypes = [C.c_void_p, _i32p, C.c_uint, _i32p]
        L.ref_reorder_x.argtypes = [C.c_void_p, _f64p, C.c_uint, _f64p]
        L.ref_run_wpk1.argtypes = [C.c_void_p, _f64p, _i32p, _f64p, _f64p, C.c_int, C.c_int]
        L.ref_reorder_columns_rowsort.argtypes = [C.c_void_p, _i32p, _i32p, C.c_uint, C.c_uint, _i32p, _i32p]
        L.ref_assembly_wpk1.argtypes = [C.c_void_p, _f64p, _f64p, C.c_int]
        self.L = L

    @staticmethod
    def available(variant="mul_add"):
        return os.path.exists(REF_PATHS[variant])

    def scan(self, rowptr, kind=1, threshold=0):
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        h = self.L.ref_scan(rowptr, len(rowptr) - 1, int(rowptr[-1]), kind, int(threshold))
        return RefStructure(self.L, h, kind)


class RefAblation:
    """The reference's optimization.cu scans (scan, scan_nosort,
    scan_nocoalesced, scan_nocoalesced_nosort) and warpKernel_nocoalesced,
    compiled for the CPU by `make -C oracle ref` (oracle/_ref/libwkref_abl.so).
    variant: 0 scan, 1 nosort, 2 nocoalesced, 3 both (the WKO_ABL_* flags)."""

    PATH = os.path.join(HERE, "_ref", "libwkref_abl.so")

    @staticmethod
    def available():
        return os.path.exists(RefAblation.PATH)

    def __init__(self, rowptr, variant):
        L = C.CDLL(self.PATH)
        L.ref_abl_scan.restype = C.c_void_p
        L.ref_abl_scan.argtypes = [_i32p, C.c_uint, C.c_uint, C.c_int]
        L.ref_abl_info.argtypes = [C.c_void_p, _u32p]
        L.ref_abl_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.ref_abl_free.argtypes = [C.c_void_p]
        L.ref_abl_run_nocoalesced.argtypes = [C.c_void_p, _f64p, _i32p, _f64p, _f64p, C.c_int]
        self.L = L
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        self.nrows, self.nz = len(rowptr) - 1, int(rowptr[-1])
        self.h = L.ref_abl_scan(rowptr, self.nrows, self.nz, int(variant))
        info = np.zeros(2, np.uint32)
        L.ref_abl_info(self.h, info)
        self.nwarps, self.allocate_nz = int(info[0]), int(info[1])
        sizes = [(np.int32, self.nrows), (np.int32, self.nrows), (np.uint32, self.nz),
                 (np.int32, self.nwarps + 1), (np.uint32, self.nwarps)]
        self.arrays = {}
        for i, name in enumerate(FIELDS[:5]):
            dt, cnt = sizes[i]
            a = np.zeros(cnt, dt)
            if cnt:
                L.ref_abl_field(self.h, i, a.ctypes.data)
            self.arrays[name] = a

    def process(self, vals, cols):
        pv = np.zeros(self.allocate_nz, np.float64)
        pc = np.zeros(self.allocate_nz, np.int32)
        rr = self.arrays["reorder_rows"]
        pv[rr] = vals
        pc[rr] = cols
        return pv, pc

    def run_nocoalesced(self, pvals, pcols, x, wpb=4):
        y = np.zeros(self.nrows, np.float64)
        self.L.ref_abl_run_nocoalesced(self.h, np.ascontiguousarray(pvals, np.float64),
                                       np.ascontiguousarray(pcols, np.int32),
                                       np.ascontiguousarray(x, np.float64), y, int(wpb))
        return y

    def free(self):
        if self.h:
            self.L.ref_abl_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class RefStructure:
    _DT = {0: np.int32, 1: np.int32, 2: np.uint32, 3: np.int32, 4: np.uint32,
           5: np.uint32, 6: np.uint32}

    def __init__(self, L, h, kind):
        self.L, self.h, self.kind = L, h, kind
        info = np.zeros(8, np.uint32)
        L.ref_info(h, info)
        (self.nrows, self.nznrows, self.nz, self.allocate_nz, self.nwarps,
         self.min_nz, self.max_nz, self.nmax_per_thread) = (int(v) for v in info)
        self.arrays = {}
        for i, name in enumerate(FIELDS):
            cnt = L.ref_field(h, i, None)
            a = np.zeros(max(cnt, 0), self._DT[i])
            if cnt > 0:
                L.ref_field(h, i, a.ctypes.data)
            self.arrays[name] = a

    def process(self, vals, cols):
        pv = np.zeros(self.allocate_nz, np.float64)
        pc = np.zeros(self.allocate_nz, np.int32)
        self.L.ref_process(self.h, np.ascontiguousarray(vals, np.float64),
                           np.ascontiguousarray(cols, np.int32), pv, pc)
        return pv, pc

    def reorder_columns_coalesced(self, cols):
        out = np.zeros(self.allocate_nz, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        self.L.ref_reorder_columns_coalesced(self.h, cols, len(cols), out)
        return out

    def reorder_x(self, x):
        x = np.ascontiguousarray(x, np.float64)
        out = np.zeros(len(x), np.float64)
        self.L.ref_reorder_x(self.h, x, len(x), out)
        return out

    def run_wpk1(self, pvals, pcols, x, mapped=True, wpb=4, y=None):
        y = np.zeros(self.nrows, np.float64) if y is None else y
        self.L.ref_run_wpk1(self.h, np.ascontiguousarray(pvals, np.float64),
                            np.ascontiguousarray(pcols, np.int32),
                            np.ascontiguousarray(x, np.float64), y, int(mapped), int(wpb))
        return y

    def reorder_columns_rowsort(self, rowptr, cols):
        out = np.zeros(self.nz, np.int32)
        src = np.zeros(self.nz, np.int32)
        self.L.ref_reorder_columns_rowsort(self.h, np.ascontiguousarray(cols, np.int32),
                                           np.ascontiguousarray(rowptr, np.int32), self.nz, self.nrows, out, src)
        return out, src

    def assembly_wpk1(self, pvals, wpb=4, y=None):
        y = np.zeros(self.nrows, np.float64) if y is None else y
        self.L.ref_assembly_wpk1(self.h, np.ascontiguousarray(pvals, np.float64), y, int(wpb))
        return y

    def free(self):
        if self.h:
            self.L.ref_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
