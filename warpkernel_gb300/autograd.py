"""Differentiable WPK SpMV: y = A(vals) x as a torch.autograd.Function.

Forward runs engine::run on the GPU; backward runs the library's adjoint:
dx = A^T dy through a transposed WPK layout built on the device, and
dvals = dy[row(k)] * x[col(k)] over the stored pattern.  Both are
deterministic (no atomics on values).  Values and vectors are float64 or
float32 CUDA tensors.

The value tensor is the parameter.  value_order="csr" (default): nz values in
the CSR order the matrix was given in.  value_order="slots": allocate_nz
values in the WPK layout's own storage order (engine.device_values; padding
slots are ignored and receive zero gradient) -- the gradient is then written
where the values are stored, which is the fastest form.  to_slots / to_csr
convert between the two.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import check, load
from .wpk import _ptr, _stream_ptr, engine, structure, structure2

_DT = {torch.float64: "f64", torch.float32: "f32"}
_ORDER = {"csr": 0, "slots": 1}


class WPKMatrix:
    """A sparse matrix with a fixed pattern (CSR row offsets / columns) in the
    WPK layout, whose values come from a (differentiable) tensor."""

    def __init__(self, rowptr, cols, vals, ncols=None, kind=2, threshold=None, value_order="csr"):
        if vals.dtype not in _DT:
            raise TypeError("values must be float32 or float64")
        if value_order not in _ORDER:
            raise ValueError("value_order is 'csr' or 'slots'")
        rp = rowptr.detach().cpu().numpy() if torch.is_tensor(rowptr) else np.asarray(rowptr)
        rp = np.ascontiguousarray(rp, dtype=np.int32)
        self.nrows = len(rp) - 1
        self.nz = int(rp[-1])
        self.ncols = self.nrows if ncols is None else int(ncols)
        lens = np.diff(rp)
        if threshold is None:
            threshold = int(lens.max()) if len(lens) and lens.max() > 0 else 1
        self.k = structure() if kind == 1 else structure2()
        if kind == 1:
            self.k.scan(self.nz, self.nrows, None, rp)
        else:
            self.k.scan(self.nz, self.nrows, None, rp, None, threshold)
        self.allocate_nz = self.k.allocate_nz
        self.value_order = value_order
        cols_t = cols if torch.is_tensor(cols) else torch.from_numpy(np.ascontiguousarray(cols, np.int32))
        cols_t = cols_t.to(device="cuda", dtype=torch.int32).contiguous()
        self.dtype = vals.dtype
        v = vals.detach().to("cuda").contiguous()
        csr_init = v if value_order == "csr" else torch.zeros(self.nz, dtype=v.dtype, device="cuda")
        self.eng = engine(self.k, csr_init, cols_t, dtype=_DT[vals.dtype], ncols=self.ncols)
        h = C.c_void_p()
        check(load().wk_adjoint_create(self.eng.handle, kind, int(threshold), _stream_ptr(None), C.byref(h)))
        self._adj = h
        self._loaded = None
        self._vals_ref = None
        self._reorder = None
        self.load_values(v)

    def __del__(self):
        try:
            if self._adj:
                load().wk_adjoint_destroy(self._adj)
        except Exception:
            pass
        self._adj = None

    @property
    def symmetric(self) -> bool:
        s = C.c_int(0)
        check(load().wk_adjoint_info(self._adj, C.byref(s), None))
        return bool(s.value)

    def _reorder_rows(self):
        if self._reorder is None:
            self._reorder = torch.from_numpy(self.k.reorder_rows.astype(np.int64)).cuda()
        return self._reorder

    def to_slots(self, vals_csr):
        """CSR-ordered values -> the layout's slot order (padding 0)."""
        out = torch.zeros(self.allocate_nz, dtype=vals_csr.dtype, device="cuda")
        out[self._reorder_rows()] = vals_csr.to("cuda")
        return out

    def to_csr(self, vals_slots):
        """Slot-ordered values -> CSR order."""
        return vals_slots.to("cuda")[self._reorder_rows()]

    def load_values(self, vals):
        """Loads the value tensor into the forward and transposed engines when
        it differs from the one last loaded."""
        v = vals.detach()
        key = (v.data_ptr(), v._version)
        if key == self._loaded:
            return
        v = v.contiguous()
        if self.value_order == "csr":
            if v.numel() != self.nz:
                raise ValueError(f"expected {self.nz} values in CSR order")
            check(load().wk_adjoint_refresh(self._adj, _ptr(v), _stream_ptr(None)))
        else:
            if v.numel() != self.allocate_nz:
                raise ValueError(f"expected {self.allocate_nz} values in slot order")
            check(load().wk_adjoint_refresh_slots(self._adj, _ptr(v), _stream_ptr(None)))
        self._loaded = (v.data_ptr(), v._version)
        self._vals_ref = v

    def matvec(self, vals, x):
        """y = A(vals) x, differentiable in vals and x."""
        return _SpMV.apply(vals, x, self)

    def adjoint(self, x, dy, want_dx=True, want_dvals=True):
        dx = torch.empty(self.ncols, dtype=self.dtype, device="cuda") if want_dx else None
        nv = self.nz if self.value_order == "csr" else self.allocate_nz
        dv = torch.empty(nv, dtype=self.dtype, device="cuda") if want_dvals else None
        check(load().wk_adjoint_run(self._adj, _ptr(x), _ptr(dy), _ptr(dx), _ptr(dv), _ORDER[self.value_order],
                                    _stream_ptr(None)))
        return dx, dv


class _SpMV(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vals, x, mat: WPKMatrix):
        if x.dtype != mat.dtype or vals.dtype != mat.dtype:
            raise TypeError("vals and x must have the matrix's dtype")
        mat.load_values(vals)
        x = x.contiguous()
        y = torch.zeros(mat.nrows, dtype=mat.dtype, device="cuda")
        mat.eng.run(0, 128, x, y, timed=False)
        ctx.save_for_backward(x)
        ctx.mat = mat
        return y

    @staticmethod
    def backward(ctx, dy):
        (x,) = ctx.saved_tensors
        mat = ctx.mat
        dx, dv = mat.adjoint(x, dy.contiguous(), ctx.needs_input_grad[1], ctx.needs_input_grad[0])
        return dv, dx, None


def spmv(mat: WPKMatrix, vals, x):
    """Functional form of WPKMatrix.matvec."""
    return _SpMV.apply(vals, x, mat)


__all__ = ["WPKMatrix", "spmv"]
