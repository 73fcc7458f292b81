"""Finite-element test matrices generated on the GPU (benchmark inputs).

The benchmark configurations use synthetic FE matrices: 2-D Q1 quad meshes
and 3-D trilinear hex meshes with `dof` unknowns per node.  These helpers
return CUDA torch tensors produced by the library's device generator.
"""
from __future__ import annotations

import ctypes as C

from ._lib import check, load
from .wpk import _stream_ptr


def fe_size(dim, ex, ey, ez=0, dof=1):
    n, z = C.c_int64(), C.c_int64()
    check(load().wk_fe_size(dim, ex, ey, ez, dof, C.byref(n), C.byref(z)))
    return n.value, z.value


def fe_matrix(dim, ex, ey, ez=0, dof=1, value_mode=1, seed=0, device="cuda"):
    """(rowptr int32, cols int32, vals float64) CUDA tensors."""
    import torch
    n, z = fe_size(dim, ex, ey, ez, dof)
    rowptr = torch.empty(n + 1, dtype=torch.int32, device=device)
    cols = torch.empty(z, dtype=torch.int32, device=device)
    vals = torch.empty(z, dtype=torch.float64, device=device)
    check(load().wk_fe_fill(dim, ex, ey, ez, dof, value_mode, seed, rowptr.data_ptr(), cols.data_ptr(),
                            vals.data_ptr(), _stream_ptr(None)))
    return rowptr, cols, vals


def uniform_vec(seed, stream_id, n, device="cuda"):
    import torch
    x = torch.empty(n, dtype=torch.float64, device=device)
    check(load().wk_uniform_vec(seed, stream_id, x.data_ptr(), n, _stream_ptr(None)))
    return x


def convert(src, dtype):
    """Element-type conversion on the device (round to nearest even)."""
    import torch
    dt = {torch.float64: 0, torch.float32: 1, torch.bfloat16: 2}
    out = torch.empty(src.numel(), dtype=dtype, device=src.device)
    check(load().wk_convert(src.data_ptr(), dt[src.dtype], out.data_ptr(), dt[dtype], src.numel(),
                            _stream_ptr(None)))
    return out
