"""Solver building blocks on the GPU: the fp64 residual r = b - A x and its
norm, against the oracle."""
import numpy as np
import pytest

from conftest import random_csr
from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12


def setup(rp, cols, vals, kind=1, th=0):
    import warpkernel_gb300 as wk
    k = wk.structure() if kind == 1 else wk.structure2()
    k.scan(len(cols), len(rp) - 1, None, rp, None, *(() if kind == 1 else (th,)))
    return k, wk.engine(k, vals, cols)


def test_residual_matches_oracle():
    import torch
    cases = [O.fe_matrix(3, 10, 10, 10, 3, value_mode=1, seed=4), O.fe_matrix(2, 64, 64, 0, 1, value_mode=0)]
    rng = np.random.default_rng(8)
    cases.append(random_csr(rng, 3000, 40, p_empty=0.3))
    for rp, cols, vals in cases:
        n = len(rp) - 1
        for kind, th in ((1, 0), (2, 7)):
            k, eng = setup(rp, cols, vals, kind, th)
            x = rng.uniform(-1, 1, n)
            b = rng.uniform(-1, 1, n)
            y = O.csr_spmv(rp, cols, vals, x)
            r_ref = b - y
            dx, db = torch.from_numpy(x).cuda(), torch.from_numpy(b).cuda()
            r = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
            nrm = torch.zeros(1, dtype=torch.float64, device="cuda")
            eng.residual(dx, db, r, nrm)
            rh = r.cpu().numpy()
            assert np.linalg.norm(rh - r_ref) / np.linalg.norm(r_ref) < REL_TOL
            empty = np.diff(rp) == 0
            assert np.array_equal(rh[empty], b[empty])
            ref2 = float(np.dot(r_ref, r_ref))
            assert abs(nrm.item() - ref2) / ref2 < REL_TOL
            # deterministic: a second call gives identical bits
            r2 = torch.empty_like(r)
            nrm2 = torch.zeros(1, dtype=torch.float64, device="cuda")
            eng.residual(dx, db, r2, nrm2)
            assert torch.equal(r, r2) and nrm.item() == nrm2.item()


def test_residual_rejects_low_precision_engine():
    import torch

    import warpkernel_gb300 as wk
    rp, cols, vals = O.fe_matrix(2, 8, 8, 0, 1, value_mode=0)
    k = wk.structure().scan(len(cols), len(rp) - 1, None, rp)
    eng = wk.engine(k, vals.astype(np.float32), cols, dtype="f32")
    t = torch.zeros(len(rp) - 1, dtype=torch.float64, device="cuda")
    with pytest.raises(wk.WKError, match="F64"):
        eng.residual(t, t, t)


def _spd_case(e=8, seed=4):
    rp, cols, vals = O.fe_matrix(3, e, e, e, 3, value_mode=1, seed=seed)
    n = len(rp) - 1
    A = np.zeros((n, n))
    for r in range(n):
        A[r, cols[rp[r]:rp[r + 1]]] = vals[rp[r]:rp[r + 1]]
    return rp, cols, vals, A


def test_cg_fp64_converges_to_the_dense_solution():
    import torch

    import warpkernel_gb300 as wk
    rp, cols, vals, A = _spd_case()
    n = len(rp) - 1
    xs = O.uniform_vec(2, 0, n)
    b = A @ xs
    for kind, th in ((1, 0), (2, 27)):
        k, eng = setup(rp, cols, vals, kind, th)
        db = torch.from_numpy(b).cuda()
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        res = wk.wpk.cg(eng, db, x, tol=1e-10)
        assert res["converged"] and res["relres"] <= 1e-10, res
        xh = x.cpu().numpy()
        assert np.linalg.norm(b - A @ xh) / np.linalg.norm(b) <= 1.1e-10
        assert np.linalg.norm(xh - xs) / np.linalg.norm(xs) < 1e-6  # A is well enough conditioned here


def test_ir_cg_reaches_fp64_tolerance_with_fp32_and_bf16_inner():
    import torch

    import warpkernel_gb300 as wk
    rp, cols, vals, A = _spd_case(seed=9)
    n = len(rp) - 1
    b = A @ O.uniform_vec(3, 0, n)
    db = torch.from_numpy(b).cuda()
    k, e64 = setup(rp, cols, vals, 2, 27)
    for dtype, tdt in (("f32", torch.float32), ("bf16", torch.bfloat16)):
        lo = wk.engine(k, wk.fe.convert(torch.from_numpy(vals).cuda(), tdt), torch.from_numpy(cols).cuda(),
                       dtype=dtype)
        lo.compress_cols()
        for dots in ("fp64", "fp32"):  # the inner solve's dot products
            x = torch.zeros(n, dtype=torch.float64, device="cuda")
            res = wk.wpk.ir_cg(e64, lo, db, x, tol=1e-10, inner_tol=1e-3 if dtype == "bf16" else 1e-4,
                               inner_dots=dots)
            assert res["converged"] and res["relres"] <= 1e-10 and res["outer"] >= 2, (dtype, dots, res)
            xh = x.cpu().numpy()
            assert np.linalg.norm(b - A @ xh) / np.linalg.norm(b) <= 1.1e-10


def test_cg_reports_non_convergence():
    import torch

    import warpkernel_gb300 as wk
    rp, cols, vals, A = _spd_case()
    n = len(rp) - 1
    k, eng = setup(rp, cols, vals)
    b = torch.from_numpy(A @ np.ones(n)).cuda()
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    res = wk.wpk.cg(eng, b, x, tol=1e-14, max_iter=3, check_every=1)
    assert not res["converged"] and res["iters"] == 3 and res["relres"] > 1e-14


def test_cg_and_ir_cg_repeat_bit_for_bit_across_partial_groups():
    """hex 14^3 x 3 dof (10,125 rows, 317 layout warps): the SpMV-dot's 80
    blocks form one full group of 64 and a partial one, whose sums are made
    by whichever block arrives last.  Two solves give the same iterations and
    the same bits (fp64 CG and IR-CG with an FP32 inner solve), and they
    reach the tolerance against the host CSR product."""
    import torch

    import warpkernel_gb300 as wk
    rp, cols, vals = O.fe_matrix(3, 14, 14, 14, 3, value_mode=1, seed=6)
    n = len(rp) - 1
    b = O.csr_spmv(rp, cols, vals, O.uniform_vec(5, 0, n))
    db = torch.from_numpy(b).cuda()
    k, e64 = setup(rp, cols, vals, 2, 81)
    assert k.nwarps > 4 * 64
    lo = wk.engine(k, wk.fe.convert(torch.from_numpy(vals).cuda(), torch.float32), torch.from_numpy(cols).cuda(),
                   dtype="f32")
    lo.compress_cols()
    for solve in (lambda x: wk.wpk.cg(e64, db, x, tol=1e-10),
                  lambda x: wk.wpk.ir_cg(e64, lo, db, x, tol=1e-10, inner_tol=1e-4)):
        xs, its = [], []
        for _ in range(2):
            x = torch.zeros(n, dtype=torch.float64, device="cuda")
            res = solve(x)
            assert res["converged"], res
            xs.append(x.cpu().numpy())
            its.append((res["iters"], res["outer"]))
        assert its[0] == its[1]
        assert np.array_equal(xs[0].view(np.uint64), xs[1].view(np.uint64))
        r = b - O.csr_spmv(rp, cols, vals, xs[0])
        assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.1e-10
