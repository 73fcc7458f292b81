"""Full-size parity of a device-built WPK layout and engine against the oracle.

TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py's parity block (after
its timed region) to check the CUDA path.  The product package never imports
it.

compare() scans the same CSR row offsets with the oracle's restatement of the
reference's host scan (structure::scan, warpkernel.hpp:309-365, or
structure2::scan, 579-736), pads values and columns with its process
(380-398, 533-548, 750-769), renumbers columns and x (447-457, 518-530) and
runs the documented order of run (53-75, 127-168) with fma on the host cores,
then compares every array with the device's: bit for bit, except the fast
order's result, which is compared normwise.
"""
from __future__ import annotations

import time

import numpy as np

from . import wk_oracle as O

FIELDS = ("row_map", "row_map_inv", "reorder_rows", "warp_offsets", "max_nz_rows")
FIELDS2 = ("threads_per_row", "row_offset_warp")
INFO = ("nrows", "nznrows", "nz", "allocate_nz", "nwarps")
INFO2 = ("min_nz", "max_nz", "nmax_per_thread")


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        a = a.view(np.uint64 if a.itemsize == 8 else np.uint32)
        b = b.view(np.uint64 if b.itemsize == 8 else np.uint32)
    return bool(np.array_equal(a, b))


def compare(k, eng, rowptr, cols, vals, x, kind, threshold, y_exact=None, y_fast=None, cols_dev=None,
            x_dev=None, nthreads=0):
    """k, eng: the device structure / fp64 engine built from (rowptr, cols,
    vals); host numpy copies of the CSR and of x; y_exact / y_fast: host
    copies of the device's exact- and fast-order `run` results (optional);
    cols_dev / x_dev: the device CSR columns and x (CUDA tensors, optional)
    for the renumbering calls.  Returns a dict of booleans (bit_identical
    per array), the fast order's normwise relative error and the seconds the
    host side took."""
    t0 = time.perf_counter()
    out = {"bit_identical": {}}
    bi = out["bit_identical"]
    with O.OracleLayout(rowptr, kind=kind, threshold=threshold) as o:
        L = o.layout
        names = INFO + (INFO2 if kind == 2 else ())
        bi["info"] = all(int(getattr(k, f)) == int(getattr(L, f)) for f in names)
        for f in FIELDS + (FIELDS2 if kind == 2 else ()):
            bi[f] = _same(getattr(k, f), getattr(L, f))
        pv, pc = o.process(vals, cols)
        bi["padded_values"] = _same(eng.device_values, pv)
        bi["padded_colinds"] = _same(eng.device_colinds, pc)
        if cols_dev is not None:
            pcr = o.reorder_columns_coalesced(cols)
            bi["reorder_columns_coalesced"] = _same(k.reorder_columns_coalesced(cols_dev).cpu().numpy(), pcr)
            del pcr
        if x_dev is not None:
            bi["reorder_x"] = _same(k.reorder_x(x_dev).cpu().numpy(), o.reorder_x(x))
        if y_exact is not None or y_fast is not None:
            y_ref = np.zeros(L.nrows, np.float64)
            o.run_omp(pv, pc, np.ascontiguousarray(x, np.float64), y_ref, nthreads)
            if y_exact is not None:
                bi["run_exact"] = _same(y_exact, y_ref)
            if y_fast is not None:
                d = float(np.linalg.norm(y_ref))
                out["run_fast_rel_err"] = float(np.linalg.norm(np.asarray(y_fast) - y_ref) / (d if d else 1.0))
        del pv, pc
    out["all_bit_identical"] = all(bi.values())
    out["host_seconds"] = round(time.perf_counter() - t0, 2)
    return out
