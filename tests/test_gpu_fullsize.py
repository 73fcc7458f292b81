"""Parity at the benchmark sizes: the device-built layouts, padded arrays,
renumbered columns and x, and the SpMV of the 3-D hex matrices the benchmark
runs, against the oracle's restatement of the reference's host scan,
process, reorderings and documented-order run on the same matrices:

* hex 128^3, 3 dof (6,440,067 rows, 513,599,625 nnz, seed 1): WPK2 with
  threshold 81 (the headline layout) and WPK1;
* hex 96^3, 3 dof (2,738,019 rows, 217,238,121 nnz, seed 2): WPK2 with
  threshold 81 and with threshold 6 (rows of 81 split over 16 lanes).

Every array is compared bit for bit; the exact-order `run` must give the
oracle's bits, the fast order and `run_x` stay within 1e-12 normwise."""
import numpy as np
import pytest

from oracle import parity

pytestmark = pytest.mark.gpu

REL_TOL_FAST = 1e-12


@pytest.mark.parametrize("mesh,seed,kind,th", [(128, 1, 2, 81), (128, 1, 1, 0), (96, 2, 2, 81), (96, 2, 2, 6)])
def test_layout_and_run_at_benchmark_size(mesh, seed, kind, th):
    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300 import fe

    rp, cols, vals = fe.fe_matrix(3, mesh, mesh, mesh, 3, 1, seed)
    n, nnz = rp.numel() - 1, cols.numel()
    x = fe.uniform_vec(seed, 0, n)
    k = wk.structure() if kind == 1 else wk.structure2()
    if kind == 1:
        k.scan(nnz, n, None, rp)
    else:
        k.scan(nnz, n, None, rp, None, th)
    eng = wk.engine(k, vals, cols)
    ys = {}
    for order in (1, 0):
        y = torch.zeros(n, dtype=torch.float64, device="cuda")
        eng.run(0, 128, x, y, order=order, timed=False)
        ys[order] = y.cpu().numpy()
    res = parity.compare(k, eng, rp.cpu().numpy(), cols.cpu().numpy(), vals.cpu().numpy(), x.cpu().numpy(),
                         kind, th, y_exact=ys[1], y_fast=ys[0], cols_dev=cols, x_dev=x)
    bad = [f for f, ok in res["bit_identical"].items() if not ok]
    assert not bad, (mesh, kind, th, bad)
    assert res["run_fast_rel_err"] < REL_TOL_FAST, res
    # run_x over the renumbered columns and the reordered x sums the same
    # products in the same order: y'[p] = y[row_map[p]] of the exact run
    eng.device_colinds = k.reorder_columns_coalesced(cols)
    xr = k.reorder_x(x)
    rm = k.row_map[:k.nznrows].astype(np.int64)
    for order in (1, 0):
        y = torch.zeros(n, dtype=torch.float64, device="cuda")
        eng.run_x(0, 128, xr, y, order=order, timed=False)
        yx = y.cpu().numpy()[:k.nznrows]
        ref = ys[1][rm]
        if order == 1:
            assert np.array_equal(yx.view(np.uint64), ref.view(np.uint64)), (mesh, kind, th)
        else:
            assert np.linalg.norm(yx - ref) / np.linalg.norm(ref) < REL_TOL_FAST
