"""Adjoint of the WPK SpMV: dx = A^T dy and dvals through torch.autograd,
checked against the host CSR-transpose gradient (oracle) and fp64 central
finite differences of loss = 0.5 ||A(vals) x - t||^2."""
import numpy as np
import pytest

from conftest import random_csr
from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu


def host_grads(rp, cols, vals, x, t):
    """Reference gradient of 0.5||A x - t||^2 on the host CSR."""
    y = O.csr_spmv(rp, cols, vals, x)
    dy = y - t
    dx = O.csr_spmv_t(rp, cols, vals, dy, len(x))
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    dvals = dy[rows] * x[cols]
    return y, dx, dvals


def run_autograd(mat, vals, x, t):
    import torch
    v = torch.from_numpy(vals).cuda().requires_grad_(True)
    xx = torch.from_numpy(x).cuda().requires_grad_(True)
    tt = torch.from_numpy(t).cuda()
    y = mat.matvec(v, xx)
    loss = 0.5 * torch.sum((y - tt) ** 2)
    loss.backward()
    return y.detach().cpu().numpy(), xx.grad.cpu().numpy(), v.grad.cpu().numpy(), loss.item()


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_symmetric_fe_matrix_fused_path_fp64():
    from warpkernel_gb300.autograd import WPKMatrix
    rp, cols, vals = O.fe_matrix(3, 6, 6, 6, 3, value_mode=1, seed=4)
    n = len(rp) - 1
    rng = np.random.default_rng(4)
    vals = vals * (1 + 0.1 * rng.standard_normal(len(vals)))  # values no longer symmetric
    x, t = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    for kind in (1, 2):
        import torch
        mat = WPKMatrix(rp, cols, torch.from_numpy(vals), kind=kind, threshold=27 if kind == 2 else None)
        assert mat.symmetric
        y, dx, dv, _ = run_autograd(mat, vals, x, t)
        y_ref, dx_ref, dv_ref = host_grads(rp, cols, vals, x, t)
        assert rel(y, y_ref) < 1e-12
        assert rel(dx, dx_ref) < 1e-12
        assert rel(dv, dv_ref) < 1e-14


def test_general_pattern_transposed_layout_fp64():
    import torch

    from warpkernel_gb300.autograd import WPKMatrix
    rng = np.random.default_rng(7)
    for trial in range(4):
        n, m = 3000, 2500 + 500 * trial  # rectangular, empty rows and columns
        rp, cols, vals = random_csr(rng, n, 40, p_empty=0.2, ncols=m, wpk2_safe=False)
        x, t = rng.uniform(-1, 1, m), rng.uniform(-1, 1, n)
        mat = WPKMatrix(rp, cols, torch.from_numpy(vals), ncols=m, kind=2, threshold=int(rng.integers(1, 30)))
        assert not mat.symmetric
        y, dx, dv, _ = run_autograd(mat, vals, x, t)
        y_ref, dx_ref, dv_ref = host_grads(rp, cols, vals, x, t)
        assert rel(y, y_ref) < 1e-12 and rel(dx, dx_ref) < 1e-12 and rel(dv, dv_ref) < 1e-14


def test_transposed_layout_matches_oracle_scan_of_the_transpose():
    import ctypes as C

    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300._lib import check, load
    from warpkernel_gb300.autograd import WPKMatrix
    rng = np.random.default_rng(2)
    n = 2000
    rp, cols, vals = random_csr(rng, n, 30, p_empty=0.1)
    mat = WPKMatrix(rp, cols, torch.from_numpy(vals), kind=2, threshold=5)
    # CSR of A^T on the host, rows ascending
    order = np.lexsort((np.repeat(np.arange(n), np.diff(rp)), cols))
    counts = np.bincount(cols, minlength=n)
    rpT = np.zeros(n + 1, np.int32)
    rpT[1:] = np.cumsum(counts)
    h = C.c_void_p()
    check(load().wk_adjoint_transposed_layout(mat._adj, C.byref(h)))
    tl = wk.structure2()
    tl._set(h)
    with O.OracleLayout(rpT, kind=2, threshold=5) as o:
        for f in ("row_map", "reorder_rows", "warp_offsets", "max_nz_rows", "threads_per_row", "row_offset_warp"):
            assert np.array_equal(getattr(tl, f), o.layout.arrays[f]), f
    assert len(order) == len(cols)


def test_central_finite_differences_64_entries():
    import torch

    from warpkernel_gb300.autograd import WPKMatrix
    rp, cols, vals = O.fe_matrix(3, 5, 5, 5, 3, value_mode=1, seed=4)
    n = len(rp) - 1
    rng = np.random.default_rng(44)
    x, t = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    mat = WPKMatrix(rp, cols, torch.from_numpy(vals), kind=2, threshold=81)
    _, dx, dv, _ = run_autograd(mat, vals, x, t)

    def loss(v, xx):
        y = O.csr_spmv(rp, cols, v, xx)
        return 0.5 * float(np.dot(y - t, y - t))

    # the loss is quadratic in each entry, so central differences are exact up
    # to rounding; a moderate step keeps the rounding small
    for k in rng.choice(len(vals), 64, replace=False):
        h = 1e-3
        vp, vm = vals.copy(), vals.copy()
        vp[k] += h
        vm[k] -= h
        fd = (loss(vp, x) - loss(vm, x)) / (2 * h)
        assert abs(fd - dv[k]) <= 1e-7 * max(abs(fd), 1e-3), (k, fd, dv[k])
    for i in rng.choice(n, 64, replace=False):
        h = 1e-3
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fd = (loss(vals, xp) - loss(vals, xm)) / (2 * h)
        assert abs(fd - dx[i]) <= 1e-7 * max(abs(fd), 1e-3), (i, fd, dx[i])


def test_slot_order_gradient_matches_csr_order():
    import torch

    from warpkernel_gb300.autograd import WPKMatrix
    rng = np.random.default_rng(13)
    cases = [(O.fe_matrix(3, 6, 6, 6, 3, value_mode=1, seed=4), 27), (random_csr(rng, 4000, 30, p_empty=0.2), 7)]
    for (rp, cols, vals), th in cases:
        n = len(rp) - 1
        x, t = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
        m_csr = WPKMatrix(rp, cols, torch.from_numpy(vals), kind=2, threshold=th)
        _, dx_c, dv_c, _ = run_autograd(m_csr, vals, x, t)
        m_slot = WPKMatrix(rp, cols, m_csr.to_slots(torch.from_numpy(vals).cuda()), kind=2, threshold=th,
                           value_order="slots")
        assert m_slot.symmetric == m_csr.symmetric
        vs = m_slot.to_slots(torch.from_numpy(vals).cuda()).requires_grad_(True)
        xx = torch.from_numpy(x).cuda().requires_grad_(True)
        y = m_slot.matvec(vs, xx)
        (0.5 * torch.sum((y - torch.from_numpy(t).cuda()) ** 2)).backward()
        assert rel(xx.grad.cpu().numpy(), dx_c) < 1e-14
        g = vs.grad
        assert np.array_equal(m_slot.to_csr(g).cpu().numpy(), dv_c)
        pad = torch.ones(m_slot.allocate_nz, dtype=torch.bool, device="cuda")
        pad[m_slot._reorder_rows()] = False
        assert bool((g[pad] == 0).all())
        # with 16-bit column storage on the forward engine (fused path reads it too)
        m_slot.eng.compress_cols()
        vs.grad = None
        xx.grad = None
        y = m_slot.matvec(vs, xx)
        (0.5 * torch.sum((y - torch.from_numpy(t).cuda()) ** 2)).backward()
        assert rel(xx.grad.cpu().numpy(), dx_c) < 1e-14
        assert np.array_equal(m_slot.to_csr(vs.grad).cpu().numpy(), dv_c)


def test_fp32_and_value_updates():
    import torch

    from warpkernel_gb300.autograd import WPKMatrix
    rp, cols, vals = O.fe_matrix(3, 6, 6, 6, 3, value_mode=1, seed=4)
    n = len(rp) - 1
    rng = np.random.default_rng(5)
    x, t = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    v32 = torch.from_numpy(vals.astype(np.float32)).cuda().requires_grad_(True)
    mat = WPKMatrix(rp, cols, v32, kind=2, threshold=81)
    opt = torch.optim.SGD([v32], lr=1e-3)
    x32 = torch.from_numpy(x.astype(np.float32)).cuda()
    t32 = torch.from_numpy(t.astype(np.float32)).cuda()
    for _ in range(3):  # values change every step: the engines must follow
        opt.zero_grad()
        y = mat.matvec(v32, x32)
        loss = 0.5 * torch.sum((y - t32) ** 2)
        loss.backward()
        vh = v32.detach().double().cpu().numpy()
        y_ref, _, dv_ref = host_grads(rp, cols, vh, x.astype(np.float32).astype(np.float64),
                                      t.astype(np.float32).astype(np.float64))
        assert rel(y.detach().double().cpu().numpy(), y_ref) < 1e-5
        assert rel(v32.grad.double().cpu().numpy(), dv_ref) < 1e-5
        opt.step()


@pytest.mark.parametrize("value_order", ["csr", "slots"])
def test_one_sided_adjoints_match_the_full_adjoint(value_order):
    """dx alone (x needs a gradient, vals do not) and dvals alone against the
    run that computes both, on the fused symmetric path and on the
    transposed-layout path.  dvals are single products: the same bits.  dx
    alone runs the transposed engine's SpMV, whose sums may be ordered
    differently from the fused kernel's: equal to rounding (fp64)."""
    import torch

    from warpkernel_gb300.autograd import WPKMatrix
    rng = np.random.default_rng(17)
    cases = [(O.fe_matrix(3, 6, 6, 6, 3, value_mode=1, seed=4), 27), (random_csr(rng, 3000, 40, p_empty=0.1), 5)]
    for (rp, cols, vals), th in cases:
        n = len(rp) - 1
        m = WPKMatrix(rp, cols, torch.from_numpy(vals), kind=2, threshold=th)
        v = torch.from_numpy(vals).cuda()
        if value_order == "slots":
            m = WPKMatrix(rp, cols, m.to_slots(v), kind=2, threshold=th, value_order="slots")
            v = m.to_slots(v)
        m.load_values(v)
        x = torch.from_numpy(rng.uniform(-1, 1, n)).cuda()
        dy = torch.from_numpy(rng.uniform(-1, 1, n)).cuda()
        dx, dv = m.adjoint(x, dy)
        dx1, dv1 = m.adjoint(x, dy, want_dx=True, want_dvals=False)
        dx2, dv2 = m.adjoint(x, dy, want_dx=False, want_dvals=True)
        assert dv1 is None and dx2 is None
        assert torch.equal(dv2, dv)
        assert rel(dx1.cpu().numpy(), dx.cpu().numpy()) < 1e-14
        y_ref = O.csr_spmv_t(rp, cols, vals, dy.cpu().numpy(), n)
        assert rel(dx1.cpu().numpy(), y_ref) < 1e-12


def _pattern_symmetric_csr(rng, n, maxlen):
    """Random CSR whose pattern is symmetric (P ∪ Pᵀ plus the diagonal) and
    whose values are not."""
    rp, cols, _ = random_csr(rng, n, maxlen)
    rows = np.repeat(np.arange(n), np.diff(rp))
    r = np.concatenate([rows, cols, np.arange(n)]).astype(np.int64)
    c = np.concatenate([cols, rows, np.arange(n)]).astype(np.int64)
    key = np.unique(r * n + c)
    r, c = key // n, key % n
    rp2 = np.zeros(n + 1, np.int64)
    np.add.at(rp2, r + 1, 1)
    return np.cumsum(rp2).astype(np.int32), c.astype(np.int32), rng.standard_normal(len(c))


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_fused_path_on_every_small_warp_count(dtype):
    """The fused symmetric adjoint launches several layout warps per block:
    layouts of 1-8 warps (counts that do and do not fill the last block), both
    value orders, 32- and 16-bit columns, against the host gradient; padding
    slots of a slot-order gradient stay 0."""
    import torch

    from warpkernel_gb300.autograd import WPKMatrix
    dt = getattr(torch, dtype)
    rng = np.random.default_rng(11)
    for n in (20, 40, 70, 100, 140, 200, 230):
        rp, cols, vals = _pattern_symmetric_csr(rng, n, min(6, n // 3))
        rows = np.repeat(np.arange(n), np.diff(rp))
        x, dy = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
        npdt = np.float64 if dtype == "float64" else np.float32
        vh, xh, dyh = vals.astype(npdt), x.astype(npdt), dy.astype(npdt)
        dx_ref = O.csr_spmv_t(rp, cols, vh.astype(np.float64), dyh.astype(np.float64), n)
        dv_ref = dyh[rows] * xh[cols]
        xt, dyt = torch.from_numpy(xh).cuda(), torch.from_numpy(dyh).cuda()
        for kind, th in ((1, None), (2, 4)):
            v = torch.from_numpy(vh).cuda()
            m_csr = WPKMatrix(rp, cols, v, kind=kind, threshold=th)
            assert m_csr.symmetric
            m_slot = WPKMatrix(rp, cols, m_csr.to_slots(v), kind=kind, threshold=th, value_order="slots")
            for compress in (False, True):
                for mat in (m_csr, m_slot):
                    if compress:
                        mat.eng.compress_cols()
                    dx, dv = mat.adjoint(xt, dyt)
                    if mat is m_slot:
                        pad = torch.ones(mat.allocate_nz, dtype=torch.bool, device="cuda")
                        pad[mat._reorder_rows()] = False
                        assert not torch.any(dv[pad] != 0)
                        dv = mat.to_csr(dv)
                    tol = 1e-13 if dtype == "float64" else 1e-5
                    assert rel(dx.double().cpu().numpy(), dx_ref) < tol, (n, kind, compress)
                    assert np.array_equal(dv.cpu().numpy(), dv_ref), (n, kind, compress)


@pytest.mark.parametrize("value_order", ["csr", "slots"])
def test_gradient_at_benchmark_size_hex64(value_order):
    """The differentiable-SpMV workload at full size: hex 64^3, 3 dof
    (823,875 rows, 64,701,513 nnz, seed 4), fp64, loss = 0.5 ||A(vals) x -
    t||^2 through torch.autograd: the whole gradient against the host
    CSR-transpose gradient, and 64 value entries and 64 x entries against
    central finite differences.  Each perturbed loss is evaluated on the host
    from scratch for the rows the entry touches (one row for a value, the
    rows of column i for x[i]); the rows it does not touch contribute the
    same terms to both evaluations and cancel exactly."""
    import torch

    from warpkernel_gb300 import fe
    from warpkernel_gb300.autograd import WPKMatrix
    rp_d, cols_d, vals_d = fe.fe_matrix(3, 64, 64, 64, 3, 1, 4)
    rp, cols, vals = rp_d.cpu().numpy(), cols_d.cpu().numpy(), vals_d.cpu().numpy()
    n = len(rp) - 1
    assert (n, len(cols)) == (823_875, 64_701_513)
    x = fe.uniform_vec(4, 0, n).cpu().numpy()
    t = fe.uniform_vec(4, 1, n).cpu().numpy()
    mat = WPKMatrix(rp_d, cols_d, vals_d, kind=2, threshold=81)
    if value_order == "slots":
        mat = WPKMatrix(rp_d, cols_d, mat.to_slots(vals_d), kind=2, threshold=81, value_order="slots")
    assert mat.symmetric
    v = (vals_d if value_order == "csr" else mat.to_slots(vals_d)).clone().requires_grad_(True)
    xx = torch.from_numpy(x).cuda().requires_grad_(True)
    y = mat.matvec(v, xx)
    (0.5 * torch.sum((y - torch.from_numpy(t).cuda()) ** 2)).backward()
    dv = v.grad if value_order == "csr" else mat.to_csr(v.grad)
    dv, dx = dv.cpu().numpy(), xx.grad.cpu().numpy()
    y_ref, dx_ref, dv_ref = host_grads(rp, cols, vals, x, t)
    assert rel(y.detach().cpu().numpy(), y_ref) < 1e-12
    assert rel(dx, dx_ref) < 1e-12
    assert rel(dv, dv_ref) < 1e-14

    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
    csc = np.argsort(cols, kind="stable")  # entries of column i: csc[cp[i]:cp[i+1]]
    cp = np.zeros(n + 1, np.int64)
    cp[1:] = np.cumsum(np.bincount(cols, minlength=n))

    def row_loss(r, vv, xv):
        s = 0.0
        for k in range(rp[r], rp[r + 1]):
            s = s + vv[k - rp[r]] * xv(cols[k])
        return 0.5 * (s - t[r]) ** 2

    rng = np.random.default_rng(64)
    h = 1e-3
    for k in rng.choice(len(vals), 64, replace=False):
        r = int(rows[k])
        seg = vals[rp[r]:rp[r + 1]].copy()
        j = k - rp[r]
        lp = lm = None
        for sign in (1, -1):
            s2 = seg.copy()
            s2[j] += sign * h
            val = row_loss(r, s2, lambda c: x[c])
            lp, lm = (val, lm) if sign == 1 else (lp, val)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - dv[k]) <= 1e-7 * max(abs(fd), 1e-3), (k, fd, dv[k])
    for i in rng.choice(n, 64, replace=False):
        touched = np.unique(rows[csc[cp[i]:cp[i + 1]]])
        tot = {}
        for sign in (1, -1):
            xi = x[i] + sign * h
            tot[sign] = sum(row_loss(int(r), vals[rp[r]:rp[r + 1]], lambda c: xi if c == i else x[c])
                            for r in touched)
        fd = (tot[1] - tot[-1]) / (2 * h)
        assert abs(fd - dx[i]) <= 1e-7 * max(abs(fd), 1e-3), (i, fd, dx[i])


def _periodic_band(n, length):
    """Pattern-symmetric CSR with every row of `length` entries: row i holds
    columns (i + k) mod n for k in -h..h (odd length, with the diagonal) or
    k in -h..h without 0 (even length).  Rows of equal length keep their
    index order in the layout, so every warp's columns form one or two runs."""
    h = length // 2
    ks = [k for k in range(-h, h + 1) if length % 2 or k != 0]
    cols = np.sort((np.arange(n)[:, None] + np.array(ks)[None, :]) % n, axis=1)
    rp = np.arange(n + 1, dtype=np.int32) * len(ks)
    return rp, cols.reshape(-1).astype(np.int32)


def _check_fp32_slot_gradient(rp, cols, vals, kind, th, rng):
    """fp32 slot-order fused adjoint against the host: dvals bit-identical to
    the fp32 products dy[row] x[col], padding slots 0, dx within 1e-5 of the
    fp64 transpose product of the same fp32 inputs."""
    import torch

    from warpkernel_gb300.autograd import WPKMatrix
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    vh = vals.astype(np.float32)
    xh = rng.uniform(-1, 1, n).astype(np.float32)
    dyh = rng.uniform(-1, 1, n).astype(np.float32)
    m_csr = WPKMatrix(rp, cols, torch.from_numpy(vh), kind=kind, threshold=th)
    assert m_csr.symmetric
    v = torch.from_numpy(vh).cuda()
    mat = WPKMatrix(rp, cols, m_csr.to_slots(v), kind=kind, threshold=th, value_order="slots")
    dx, dv = mat.adjoint(torch.from_numpy(xh).cuda(), torch.from_numpy(dyh).cuda())
    pad = torch.ones(mat.allocate_nz, dtype=torch.bool, device="cuda")
    pad[mat._reorder_rows()] = False
    assert not torch.any(dv[pad] != 0)
    assert np.array_equal(mat.to_csr(dv).cpu().numpy(), dyh[rows] * xh[cols])
    dx_ref = O.csr_spmv_t(rp, cols, vh.astype(np.float64), dyh.astype(np.float64), n)
    assert rel(dx.double().cpu().numpy(), dx_ref) < 1e-5


def test_fp32_slot_order_every_remainder():
    """The fp32 slot-order kernel streams units of 8 steps and a partial last
    unit through its shared-memory ring: constant row lengths 1-20 and 40
    (every remainder modulo 8, zero to five full units) in WPK1, and WPK2
    with a threshold that splits the rows; n = 1000 leaves a partial last
    warp.  Every warp of these bands has an x window."""
    rng = np.random.default_rng(23)
    for length in list(range(1, 21)) + [40]:
        rp, cols = _periodic_band(1000, length)
        vals = rng.standard_normal(len(cols))
        _check_fp32_slot_gradient(rp, cols, vals, 1, None, rng)
        if length >= 6:
            _check_fp32_slot_gradient(rp, cols, vals, 2, 4, rng)


def test_fp32_slot_order_mixed_windows():
    """A band whose rows 300-499 also hold 24 random far columns (mirrored,
    so the pattern stays symmetric): their warps see hundreds of distinct
    columns and have no x window, the band's warps keep theirs, and the
    kernel's window and plain-gather paths run side by side."""
    rng = np.random.default_rng(29)
    n = 2000
    rp0, cols0 = _periodic_band(n, 13)
    rows0 = np.repeat(np.arange(n), np.diff(rp0))
    far_r = np.repeat(np.arange(300, 500), 24)
    far_c = rng.integers(0, n, far_r.size)
    r = np.concatenate([rows0, far_r, far_c]).astype(np.int64)
    c = np.concatenate([cols0, far_c, far_r]).astype(np.int64)
    key = np.unique(r * n + c)
    r, c = key // n, key % n
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, r + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    vals = rng.standard_normal(len(c))
    for kind, th in ((1, None), (2, 8)):
        _check_fp32_slot_gradient(rp, c.astype(np.int32), vals, kind, th, rng)


def test_fp32_slot_order_at_benchmark_size_hex64():
    """The differentiable-SpMV benchmark's own path: hex 64^3, 3 dof (seed 4),
    fp32 values, WPK2 threshold 81, gradient in slot order."""
    from warpkernel_gb300 import fe
    rp_d, cols_d, vals_d = fe.fe_matrix(3, 64, 64, 64, 3, 1, 4)
    rp, cols, vals = rp_d.cpu().numpy(), cols_d.cpu().numpy(), vals_d.cpu().numpy()
    _check_fp32_slot_gradient(rp, cols, vals, 2, 81, np.random.default_rng(64))


def test_fp32_slot_order_gradient_alone_and_unsymmetric_patterns():
    """The value gradient without dx (any pattern) and the unsymmetric
    patterns' gradient in fp32 slot order run the staged kernel's
    gradient-only form: dvals bit-identical to the FP32 products dy[row]
    x[col], padding slots 0, the same bits as the full adjoint of a symmetric
    pattern; dx (from A^T's SpMV) within 1e-5 of the host transpose."""
    import torch

    from warpkernel_gb300.autograd import WPKMatrix
    rng = np.random.default_rng(31)
    # unsymmetric: a random pattern, and an FE matrix with 1 % of its
    # off-diagonal entries dropped (most warps keep an x window)
    rp_f, cols_f, vals_f = O.fe_matrix(3, 10, 10, 10, 3, value_mode=1, seed=8)
    rows_f = np.repeat(np.arange(len(rp_f) - 1), np.diff(rp_f))
    keep = (rows_f == cols_f) | (rng.random(len(cols_f)) > 0.01)
    rp_k = np.zeros(len(rp_f), np.int64)
    np.add.at(rp_k, rows_f[keep] + 1, 1)
    cases = [(random_csr(rng, 5000, 60, p_empty=0.05), 7),
             ((np.cumsum(rp_k).astype(np.int32), cols_f[keep], vals_f[keep]), 81)]
    for (rp, cols, vals), th in cases:
        n = len(rp) - 1
        rows = np.repeat(np.arange(n), np.diff(rp))
        vh = vals.astype(np.float32)
        xh = rng.uniform(-1, 1, n).astype(np.float32)
        dyh = rng.uniform(-1, 1, n).astype(np.float32)
        m_csr = WPKMatrix(rp, cols, torch.from_numpy(vh), kind=2, threshold=th)
        assert not m_csr.symmetric
        mat = WPKMatrix(rp, cols, m_csr.to_slots(torch.from_numpy(vh).cuda()), kind=2, threshold=th,
                        value_order="slots")
        dx, dv = mat.adjoint(torch.from_numpy(xh).cuda(), torch.from_numpy(dyh).cuda())
        pad = torch.ones(mat.allocate_nz, dtype=torch.bool, device="cuda")
        pad[mat._reorder_rows()] = False
        assert not torch.any(dv[pad] != 0)
        assert np.array_equal(mat.to_csr(dv).cpu().numpy(), dyh[rows] * xh[cols])
        dx_ref = O.csr_spmv_t(rp, cols, vh.astype(np.float64), dyh.astype(np.float64), n)
        assert rel(dx.double().cpu().numpy(), dx_ref) < 1e-5
    # a symmetric band: the gradient alone against the full adjoint's
    rp, cols = _periodic_band(3000, 27)
    vals = rng.standard_normal(len(cols)).astype(np.float32)
    m_csr = WPKMatrix(rp, cols, torch.from_numpy(vals), kind=2, threshold=27)
    mat = WPKMatrix(rp, cols, m_csr.to_slots(torch.from_numpy(vals).cuda()), kind=2, threshold=27,
                    value_order="slots")
    assert mat.symmetric
    x = torch.from_numpy(rng.uniform(-1, 1, 3000).astype(np.float32)).cuda()
    dy = torch.from_numpy(rng.uniform(-1, 1, 3000).astype(np.float32)).cuda()
    _, dv_full = mat.adjoint(x, dy)
    dx_none, dv_alone = mat.adjoint(x, dy, want_dx=False, want_dvals=True)
    assert dx_none is None and torch.equal(dv_alone, dv_full)
