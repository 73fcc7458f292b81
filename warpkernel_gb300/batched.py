"""Batched multi-RHS SpMV over many WPK matrices in one persistent launch,
and the autotuner that picks its layout threshold and RHS tile.

    mats = batched.fe_matrix_set(512, seed=3)          # the c4 matrix family
    b = batched.Batch.from_fe(mats, dtype="f32")       # engines + queue
    b.set_vectors(X, Y); b.capture(); secs = b.run()   # one graph replay
    best = batched.autotune(mats)                      # threshold / tile choice
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import fe
from ._lib import check, load
from .wpk import _stream_ptr, engine, structure2

TILES = (1, 2, 4, 8, 16)


def fe_matrix_set(count=512, seed=3, rows=(1_000, 200_000)):
    """Specs of `count` FE patches with log-uniform row counts in `rows`:
    2-D Q1 or 3-D hex, 1 or 3 dofs per node, 1-16 right-hand sides."""
    rng = np.random.default_rng(seed)
    out = []
    lo, hi = math.log(rows[0]), math.log(rows[1])
    for i in range(count):
        target = math.exp(rng.uniform(lo, hi))
        dim = int(rng.choice((2, 3)))
        dof = int(rng.choice((1, 3)))
        nodes = target / dof
        ex = max(1, int(round(nodes ** (1.0 / dim))) - 1)
        nrhs = int(rng.integers(1, 17))
        n, z = fe.fe_size(dim, ex, ex, ex if dim == 3 else 0, dof)
        out.append(dict(dim=dim, ex=ex, dof=dof, nrhs=nrhs, nrows=n, nnz=z, seed=int(seed * 100_003 + i)))
    return out


def _engine_for(spec, dtype, threshold_frac=1.0):
    dim, ex, dof = spec["dim"], spec["ex"], spec["dof"]
    rp, cols, vals = fe.fe_matrix(dim, ex, ex, ex if dim == 3 else 0, dof, 1, spec["seed"])
    n, nz = rp.numel() - 1, cols.numel()
    maxlen = (27 if dim == 3 else 9) * dof
    th = max(1, int(round(maxlen * threshold_frac)))
    k = structure2().scan(nz, n, None, rp, None, th)
    v = vals if dtype == "f64" else fe.convert(vals, torch.float32)
    e = engine(k, v, cols, dtype=dtype)
    return k, e


class Batch:
    """A wk_batch over engines that this object keeps alive."""

    def __init__(self, engines, nrhs, rhs_tile=8, chunk=16, keep=()):
        self.engines = list(engines)
        self.keep = list(keep)
        self.nrhs = np.ascontiguousarray(nrhs, dtype=np.uint32)
        arr = (C.c_void_p * len(self.engines))(*[e.handle.value for e in self.engines])
        h = C.c_void_p()
        check(load().wk_batch_create(arr, self.nrhs.ctypes.data_as(C.POINTER(C.c_uint32)), len(self.engines),
                                     int(rhs_tile), int(chunk), C.byref(h)))
        self._h = h
        self._vec = None

    @classmethod
    def from_fe(cls, specs, dtype="f32", threshold_frac=1.0, rhs_tile=8, chunk=16):
        ks, es = [], []
        for s in specs:
            k, e = _engine_for(s, dtype, threshold_frac)
            ks.append(k)
            es.append(e)
        return cls(es, [s["nrhs"] for s in specs], rhs_tile, chunk, keep=ks)

    def __del__(self):
        try:
            if self._h:
                load().wk_batch_destroy(self._h)
        except Exception:
            pass
        self._h = None

    def set_vectors(self, X, Y):
        """X[m]: (ncols_m, nrhs_m) CUDA tensors, Y[m]: (nrows_m, nrhs_m)."""
        xs = (C.c_void_p * len(X))(*[x.data_ptr() for x in X])
        ys = (C.c_void_p * len(Y))(*[y.data_ptr() for y in Y])
        check(load().wk_batch_set_vectors(self._h, xs, ys))
        self._vec = (X, Y)

    def set_tile(self, tile):
        check(load().wk_batch_set_tile(self._h, int(tile)))

    def capture(self):
        check(load().wk_batch_capture(self._h))

    def run(self, timed=True, stream=None):
        s = C.c_float(0.0)
        check(load().wk_batch_run(self._h, _stream_ptr(stream), C.byref(s) if timed else None))
        return float(s.value) if timed else None

    def info(self):
        n, g, t = C.c_uint32(), C.c_uint32(), C.c_int()
        check(load().wk_batch_info(self._h, C.byref(n), C.byref(g), C.byref(t)))
        return dict(items=n.value, grid=g.value, rhs_tile=t.value)


def make_vectors(specs, dtype=torch.float32, seed=3):
    """X uniform(-1, 1) per matrix (ncols x nrhs, row-major) and zeroed Y."""
    X, Y = [], []
    for i, s in enumerate(specs):
        x = fe.uniform_vec(seed, 1000 + i, s["nrows"] * s["nrhs"]).to(dtype).view(s["nrows"], s["nrhs"])
        X.append(x.contiguous())
        Y.append(torch.zeros(s["nrows"], s["nrhs"], dtype=dtype, device="cuda"))
    return X, Y


def _time(b, reps=5):
    b.run()
    return min(b.run() for _ in range(reps))


def autotune(specs, dtype="f32", fracs=(1.0, 0.5, 0.25), tiles=TILES, sample=None, reps=5):
    """Picks the layout threshold (as a fraction of the longest row) and the
    RHS tile by timing whole batched launches.  `sample` (optional) limits
    the tuning to the first `sample` matrices.  Returns the choice and the
    timings."""
    sp = specs if sample is None else specs[:sample]
    X, Y = make_vectors(sp, torch.float32 if dtype == "f32" else torch.float64)
    timings = {}
    best = None
    for f in fracs:
        b = Batch.from_fe(sp, dtype, f, rhs_tile=8)
        b.set_vectors(X, Y)
        for t in tiles:
            b.set_tile(t)
            sec = _time(b, reps)
            timings[(f, t)] = sec
            if best is None or sec < timings[best]:
                best = (f, t)
        del b
    return {"threshold_frac": best[0], "rhs_tile": best[1], "seconds": timings[best],
            "timings": {f"{f}/{t}": s for (f, t), s in timings.items()}}


def algorithmic_bytes(specs, value_bytes=4, vec_bytes=4):
    """sum_m (b_v + 4) z_m + n_m k_m (b_x + b_y)."""
    return sum((value_bytes + 4) * s["nnz"] + s["nrows"] * s["nrhs"] * 2 * vec_bytes for s in specs)
