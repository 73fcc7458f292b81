"""ctypes loader for libwarpkernel_gb300.so (the C ABI of include/wk_capi.h).

The library is built in-tree by warpkernel_gb300.build.  There is no fallback:
if the library is missing or cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwarpkernel_gb300.so")

WK_OK = 0
WK_F64, WK_F32, WK_BF16, WK_F16S = 0, 1, 2, 3
WK_WPK1, WK_WPK2 = 1, 2
WK_ORDER_FAST, WK_ORDER_EXACT = 0, 1
WK_ABL_NOSORT, WK_ABL_NOCOALESCE = 1, 2
FIELDS = {
    "row_map": 0, "row_map_inv": 1, "reorder_rows": 2, "warp_offsets": 3,
    "max_nz_rows": 4, "threads_per_row": 5, "row_offset_warp": 6,
}
STATUS_NAMES = {1: "INVALID", 2: "CUDA", 3: "ALLOC", 4: "OVERFLOW", 5: "STATE", 6: "DEVICE",
                7: "NOTCONV"}

# Every symbol include/wk_capi.h declares, with (restype, argtypes).
vp, i32, u32, i64, u64 = C.c_void_p, C.c_int32, C.c_uint32, C.c_int64, C.c_uint64
_i32p, _u32p, _i64p, _f64p = (C.POINTER(C.c_int32), C.POINTER(C.c_uint32), C.POINTER(C.c_int64),
                              C.POINTER(C.c_double))
_pvp = C.POINTER(C.c_void_p)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_szp = C.POINTER(C.c_size_t)


class LayoutInfo(C.Structure):
    _fields_ = [("kind", C.c_int), ("nrows", u32), ("nznrows", u32), ("nz", u32),
                ("allocate_nz", u32), ("nwarps", u32), ("min_nz", u32), ("max_nz", u32),
                ("nmax_per_thread", u32), ("variant", u32)]


class CGParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int), ("max_inner", C.c_int),
                ("inner_tol", C.c_double), ("check_every", C.c_int), ("iters", C.c_int),
                ("outer", C.c_int), ("relres", C.c_double), ("seconds", C.c_double),
                ("inner_dots_fp32", C.c_int)]


SIGNATURES = {
    "wk_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "wk_version": (C.c_char_p, []),
    "wk_debug_fail_alloc": (None, [C.c_int]),
    "wk_scan1": (C.c_int, [vp, u32, u32, vp, _pvp]),
    "wk_scan2": (C.c_int, [vp, u32, u32, i32, vp, _pvp]),
    "wk_scan1_ablation": (C.c_int, [vp, u32, u32, C.c_int, vp, _pvp]),
    "wk_layout_info_get": (C.c_int, [vp, C.POINTER(LayoutInfo)]),
    "wk_layout_get": (C.c_int, [vp, C.c_int, vp, C.c_size_t, _szp]),
    "wk_layout_destroy": (C.c_int, [vp]),
    "wk_reorder_columns_coalesced": (C.c_int, [vp, vp, vp, vp]),
    "wk_reorder_columns": (C.c_int, [vp, vp, vp, vp]),
    "wk_reorder_x": (C.c_int, [vp, C.c_int, vp, vp, vp]),
    "wk_engine_create": (C.c_int, [vp, C.c_int, vp, vp, u32, vp, _pvp]),
    "wk_engine_set_colinds": (C.c_int, [vp, vp, vp]),
    "wk_engine_set_values": (C.c_int, [vp, vp, vp]),
    "wk_engine_get_values": (C.c_int, [vp, vp, C.c_size_t]),
    "wk_engine_get_colinds": (C.c_int, [vp, vp, C.c_size_t]),
    "wk_engine_destroy": (C.c_int, [vp]),
    "wk_engine_compress_cols": (C.c_int, [vp, vp, _u32p]),
    "wk_engine_set_windows": (C.c_int, [vp, C.c_int, _u32p]),
    "wk_run": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, _fp]),
    "wk_run_x": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, _fp]),
    "wk_run_host": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, vp]),
    "wk_run_host_stream": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, _pvp, _pvp, vp, _fp]),
    "wk_residual": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "wk_residual_static": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "wk_cg": (C.c_int, [vp, vp, vp, C.POINTER(CGParams), vp]),
    "wk_ir_cg": (C.c_int, [vp, vp, vp, vp, C.POINTER(CGParams), vp]),
    "wk_adjoint_create": (C.c_int, [vp, C.c_int, i32, vp, _pvp]),
    "wk_adjoint_refresh": (C.c_int, [vp, vp, vp]),
    "wk_adjoint_run": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, vp]),
    "wk_adjoint_refresh_slots": (C.c_int, [vp, vp, vp]),
    "wk_adjoint_info": (C.c_int, [vp, _ip, C.POINTER(LayoutInfo)]),
    "wk_adjoint_transposed_layout": (C.c_int, [vp, _pvp]),
    "wk_adjoint_destroy": (C.c_int, [vp]),
    "wk_batch_create": (C.c_int, [vp, _u32p, C.c_int, C.c_int, C.c_int, _pvp]),
    "wk_batch_set_vectors": (C.c_int, [vp, vp, vp]),
    "wk_batch_set_tile": (C.c_int, [vp, C.c_int]),
    "wk_batch_capture": (C.c_int, [vp]),
    "wk_batch_run": (C.c_int, [vp, vp, _fp]),
    "wk_batch_info": (C.c_int, [vp, _u32p, _u32p, _ip]),
    "wk_batch_destroy": (C.c_int, [vp]),
    "wk_verify": (C.c_int, [vp, vp, vp, _ip, _i64p]),
    "wk_verify_x": (C.c_int, [vp, vp, vp, C.c_int, _ip, _i64p]),
    "wk_fe_size": (C.c_int, [C.c_int] * 5 + [_i64p, _i64p]),
    "wk_fe_fill": (C.c_int, [C.c_int] * 6 + [u64, vp, vp, vp, vp]),
    "wk_uniform_vec": (C.c_int, [u64, u64, vp, i64, vp]),
    "wk_convert": (C.c_int, [vp, C.c_int, vp, C.c_int, i64, vp]),
    "wk_reorder_columns_rowsort": (C.c_int, [vp, vp, vp, vp, vp]),
    "wk_process": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp]),
    "wk_run_assembly": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, _fp]),
    "wk_layout_save": (C.c_int, [vp, C.c_char_p]),
    "wk_layout_load": (C.c_int, [C.c_char_p, vp, _pvp]),
    "wk_mm_read": (C.c_int, [C.c_char_p, _pvp]),
    "wk_csr_get": (C.c_int, [vp, _i64p, _i64p, _i64p, _pvp, _pvp, _pvp]),
    "wk_csr_free": (C.c_int, [vp]),
}


class WKError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"WK_ERR_{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_lib = None


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() "
                               "(or python -m warpkernel_gb300.build) first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    L = load()
    n = L.wk_last_error(None, 0)
    buf = C.create_string_buffer(n + 1)
    L.wk_last_error(buf, n + 1)
    return buf.value.decode(errors="replace")


def check(status: int):
    if status != WK_OK:
        raise WKError(status, last_error())
