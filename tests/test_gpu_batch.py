"""Batched multi-RHS persistent launch: every matrix and right-hand side
equals the engine's own exact-order run, bit for bit, for every RHS tile,
through plain launches and CUDA-graph replays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_matches_per_engine_exact_runs():
    import torch

    from warpkernel_gb300 import batched
    specs = batched.fe_matrix_set(10, seed=7, rows=(500, 20_000))
    specs[0]["nrhs"], specs[1]["nrhs"] = 16, 3  # vector and scalar gathers
    b = batched.Batch.from_fe(specs, "f32", threshold_frac=0.5, rhs_tile=4, chunk=5)
    X, Y = batched.make_vectors(specs)
    b.set_vectors(X, Y)
    ref = []
    for s, e, x in zip(specs, b.engines, X):
        cols = []
        for j in range(s["nrhs"]):
            xj = x[:, j].contiguous()
            yj = torch.zeros(s["nrows"], dtype=torch.float32, device="cuda")
            e.run(0, 128, xj, yj, order=1)
            cols.append(yj)
        ref.append(torch.stack(cols, 1))
    for tile in batched.TILES:
        b.set_tile(tile)
        for y in Y:
            y.zero_()
        b.run()
        for m, (y, r) in enumerate(zip(Y, ref)):
            assert torch.equal(y, r), (tile, m)
    b.capture()
    for rep in range(2):
        for y in Y:
            y.zero_()
        b.run()
        for y, r in zip(Y, ref):
            assert torch.equal(y, r)
    info = b.info()
    assert info["items"] > 10 and info["grid"] >= 152


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
    ref = []
    for s, e, x in zip(specs, b.engines, X):
        cols = []
        for j in range(s["nrhs"]):
            yj = torch.zeros(s["nrows"], dtype=torch.float64, device="cuda")
            e.run(0, 128, x[:, j].contiguous(), yj, order=1)
            cols.append(yj)
        ref.append(torch.stack(cols, 1))
    for tile in batched.TILES:
        b.set_tile(tile)
        for y in Y:
            y.zero_()
        b.run()
        for m, (y, r) in enumerate(zip(Y, ref)):
            assert torch.equal(y, r), (tile, m)
    assert load().wk_batch_set_tile(b._h, 3) == 1
    h = C.c_void_p()
    nr = np.zeros(1, np.uint32)
    arr = (C.c_void_p * 1)(b.engines[0].handle.value)
    assert load().wk_batch_create(arr, nr.ctypes.data_as(C.POINTER(C.c_uint32)), 1, 4, 16, C.byref(h)) == 1
