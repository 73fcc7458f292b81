"""Batched multi-RHS persistent launch: every matrix and right-hand side
equals the oracle's documented-order product of that matrix and column of X
(FP32: wko_run_lp on the FP32-rounded values; fp64: wko_run_f64 with fma),
bit for bit, for every RHS tile, through plain launches and CUDA-graph
replays, whichever warp of the persistent grid computed it."""
import numpy as np
import pytest

from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu


def oracle_products(specs, batch, X, dtype):
    """Per matrix, the (nrows, nrhs) oracle product in the engine's layout."""
    from warpkernel_gb300 import fe
    out = []
    for s, k, x in zip(specs, batch.keep, X):
        dim, ex, dof = s["dim"], s["ex"], s["dof"]
        rp, cols, vals = (a.cpu().numpy() for a in fe.fe_matrix(dim, ex, ex, ex if dim == 3 else 0, dof, 1,
                                                                s["seed"]))
        xh = x.cpu().numpy()
        y = np.zeros((s["nrows"], s["nrhs"]), xh.dtype)
        with O.OracleLayout(rp, kind=2, threshold=k.nmax_per_thread) as o:
            assert np.array_equal(o.layout.row_map, k.row_map)
            _, pc = o.process(vals, cols)
            if dtype == "f32":
                pv = o.place(O.round_f32(vals))
                for j in range(s["nrhs"]):
                    y[:, j] = o.run_lp(pv, pc, np.ascontiguousarray(xh[:, j]))
            else:
                pv, _ = o.process(vals, cols)
                for j in range(s["nrhs"]):
                    y[:, j] = o.run(pv, pc, np.ascontiguousarray(xh[:, j]), fma=True)
        out.append(y)
    return out


def check(Y, ref, tag):
    for m, (y, r) in enumerate(zip(Y, ref)):
        yh = y.cpu().numpy()
        assert np.array_equal(yh.view(np.uint32 if yh.dtype == np.float32 else np.uint64),
                              r.view(np.uint32 if r.dtype == np.float32 else np.uint64)), (tag, m)


def test_batch_matches_the_oracle_fp32():
    from warpkernel_gb300 import batched
    specs = batched.fe_matrix_set(10, seed=7, rows=(500, 20_000))
    specs[0]["nrhs"], specs[1]["nrhs"] = 16, 3  # a full tile and a ragged one
    b = batched.Batch.from_fe(specs, "f32", threshold_frac=0.5, rhs_tile=4, chunk=5)
    X, Y = batched.make_vectors(specs)
    b.set_vectors(X, Y)
    ref = oracle_products(specs, b, X, "f32")
    for tile in batched.TILES:
        b.set_tile(tile)
        for y in Y:
            y.zero_()
        b.run()
        check(Y, ref, tile)
    b.capture()
    for rep in range(2):
        for y in Y:
            y.zero_()
        b.run()
        check(Y, ref, ("graph", rep))
    info = b.info()
    assert info["items"] > 10 and info["grid"] >= 152


def test_batch_every_rhs_count_fp32():
    """RHS counts 1-16 (every remainder of every tile) on small patches."""
    from warpkernel_gb300 import batched
    specs = batched.fe_matrix_set(16, seed=11, rows=(300, 3_000))
    for i, s in enumerate(specs):
        s["nrhs"] = i + 1
    b = batched.Batch.from_fe(specs, "f32", threshold_frac=1.0, rhs_tile=8, chunk=4)
    X, Y = batched.make_vectors(specs)
    b.set_vectors(X, Y)
    ref = oracle_products(specs, b, X, "f32")
    for tile in batched.TILES:
        b.set_tile(tile)
        for y in Y:
            y.zero_()
        b.run()
        check(Y, ref, tile)


def test_batch_fp64_and_validation():
    import ctypes as C

    import torch

    from warpkernel_gb300 import batched
    from warpkernel_gb300._lib import load
    specs = batched.fe_matrix_set(4, seed=2, rows=(1000, 5000))
    specs[0]["nrhs"] = 16  # a full 16-wide tile
    b = batched.Batch.from_fe(specs, "f64", rhs_tile=2)
    X, Y = batched.make_vectors(specs, torch.float64)
    b.set_vectors(X, Y)
    ref = oracle_products(specs, b, X, "f64")
    for tile in batched.TILES:
        b.set_tile(tile)
        for y in Y:
            y.zero_()
        b.run()
        check(Y, ref, tile)
    assert load().wk_batch_set_tile(b._h, 3) == 1
    h = C.c_void_p()
    nr = np.zeros(1, np.uint32)
    arr = (C.c_void_p * 1)(b.engines[0].handle.value)
    assert load().wk_batch_create(arr, nr.ctypes.data_as(C.POINTER(C.c_uint32)), 1, 4, 16, C.byref(h)) == 1


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_batch_more_rhs_than_the_tile(dtype):
    """Right-hand-side counts above the widest tile (17-40): each item runs
    several tiles, the last one narrower (its own 16-byte group count), for
    every tile width; fp32 and fp64 against the oracle, bit for bit."""
    import torch

    from warpkernel_gb300 import batched
    specs = batched.fe_matrix_set(6, seed=13, rows=(400, 4_000))
    for s, k in zip(specs, (17, 20, 23, 31, 33, 40)):
        s["nrhs"] = k
    b = batched.Batch.from_fe(specs, dtype, threshold_frac=1.0, rhs_tile=16, chunk=4)
    X, Y = batched.make_vectors(specs, torch.float32 if dtype == "f32" else torch.float64)
    b.set_vectors(X, Y)
    ref = oracle_products(specs, b, X, dtype)
    for tile in batched.TILES:
        b.set_tile(tile)
        for y in Y:
            y.zero_()
        b.run()
        check(Y, ref, tile)
