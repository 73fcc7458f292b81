"""engine::run / run_x on the GPU against the reference's own WPK1 kernel
outputs (golden), the oracle's documented order, and size-independent
properties at full size."""
import numpy as np
import pytest

from conftest import golden_cases, random_csr
from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu

REL_TOL_FAST = 1e-12  # normwise relative, fp64, re-associated order


def wk():
    import warpkernel_gb300
    return warpkernel_gb300


def torch():
    import torch as t
    return t


def make(kind, rp, cols, vals, th=0, dtype="f64"):
    k = wk().structure() if kind == 1 else wk().structure2()
    if kind == 1:
        k.scan(len(cols), len(rp) - 1, vals, rp, cols)
    else:
        k.scan(len(cols), len(rp) - 1, vals, rp, cols, th)
    v = vals if dtype == "f64" else vals.astype(np.float32)
    return k, wk().engine(k, v, cols, dtype=dtype)


def run(eng, x, mapped=True, order=0, cache=True, nblocks=0, blocksize=256, y0=0.0):
    t = torch()
    n = eng.kernel.nrows
    dx = t.from_numpy(np.ascontiguousarray(x)).cuda()
    dy = t.full((n,), y0, dtype=dx.dtype, device="cuda")
    f = eng.run if mapped else eng.run_x
    sec = f(nblocks, blocksize, dx, dy, cache=cache, order=order)
    assert sec >= 0
    return dy.cpu().numpy()


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def relerr(y, ref):
    d = np.linalg.norm(ref)
    return np.linalg.norm(y - ref) / (d if d else 1.0)


def test_wpk1_matches_reference_kernel_outputs(golden):
    """Exact order is bit-identical to the reference's warpKernel /
    warpKernel_reorderx compiled with contraction (golden y_run_fma)."""
    for name, rp, cols, vals, x, layouts in golden_cases(golden):
        tag = f"{name}/k1_t0"
        if f"{tag}/y_run_fma" not in golden:
            continue
        k, eng = make(1, rp, cols, vals)
        y = run(eng, x, order=wk().WK_ORDER_EXACT)
        assert np.array_equal(bits(y), bits(golden[f"{tag}/y_run_fma"])), tag
        y = run(eng, x)
        assert relerr(y, golden[f"{tag}/y_run_fma"]) < REL_TOL_FAST, tag
        eng.device_colinds = golden[f"{tag}/pcols_renum"]
        xr = golden[f"{tag}/x_reordered"]
        y = run(eng, xr, mapped=False, order=wk().WK_ORDER_EXACT)
        assert np.array_equal(bits(y), bits(golden[f"{tag}/y_runx_fma"])), tag
        y = run(eng, xr, mapped=False)
        assert relerr(y, golden[f"{tag}/y_runx_fma"]) < REL_TOL_FAST, tag


def check_all_variants(rp, cols, vals, x, kind, th, tag, shapes=((0, 256),)):
    k, eng = make(kind, rp, cols, vals, th)
    o = O.OracleLayout(rp, kind=kind, threshold=th)
    pv, pc = o.process(vals, cols)
    y_ref = o.run(pv, pc, x, fma=True)
    pcr = o.reorder_columns_coalesced(cols)
    xr = o.reorder_x(x)
    yx_ref = o.run_x(pv, pcr, xr, fma=True)
    for nblocks, bs in shapes:
        for cache in (True, False):
            y = run(eng, x, order=1, cache=cache, nblocks=nblocks, blocksize=bs)
            assert np.array_equal(bits(y), bits(y_ref)), (tag, "exact", bs, cache)
            y = run(eng, x, order=0, cache=cache, nblocks=nblocks, blocksize=bs)
            assert relerr(y, y_ref) < REL_TOL_FAST, (tag, "fast", bs, cache, relerr(y, y_ref))
    # WPK_r (run_x) and WPK_rx (run with renumbered columns and reordered x)
    eng.device_colinds = k.reorder_columns_coalesced(cols)
    y = run(eng, xr, mapped=False, order=1)
    assert np.array_equal(bits(y), bits(yx_ref)), (tag, "run_x exact")
    y = run(eng, xr, mapped=False)
    assert relerr(y, yx_ref) < REL_TOL_FAST, (tag, "run_x fast")
    # verify_x keeps the reference's condition, which mixes orig[row_map[i]]
    # and orig[i] (it fails on matrices with empty rows); strict mode does not
    assert eng.verify_x(y_ref, y) == o.verify_x(y_ref, y)[0], tag
    assert eng.verify_x(y_ref, y, strict=True), tag
    y = run(eng, xr, mapped=True)
    assert relerr(y, y_ref) < REL_TOL_FAST, (tag, "rx fast")
    assert eng.verify(y_ref, y) and o.verify(y_ref, y)[0]
    o.free()


def test_golden_layouts_all_variants(golden):
    for name, rp, cols, vals, x, layouts in golden_cases(golden):
        if len(cols) == 0:
            continue
        for kind, th in layouts:
            check_all_variants(rp, cols, vals, x, kind, th, f"{name}/{kind}/{th}",
                               shapes=((0, 32), (0, 256), (0, 1024), (10000, 64)))


def test_random_matrices():
    rng = np.random.default_rng(17)
    for trial in range(25):
        n = int(rng.integers(2, 5000))
        rp, cols, vals = random_csr(rng, n, int(rng.choice([3, 9, 27, 81, 300])), float(rng.choice([0, 0.2])))
        if len(cols) == 0:
            continue
        x = rng.uniform(-1, 1, n)
        for kind, th in ((1, 0), (2, int(rng.integers(0, 40)))):
            check_all_variants(rp, cols, vals, x, kind, th, (trial, kind, th))


def test_config1_q1_128_threshold_sweep():
    """2-D Q1 128x128, 1 dof (16,641 rows): WPK1 and the WPK2 threshold sweep
    of the reference's wpk2 driver (min_nz..max_nz, 10% steps), every
    warps-per-block of the drivers."""
    rp, cols, vals = O.fe_matrix(2, 128, 128, 0, 1, value_mode=0, seed=0)
    x = O.uniform_vec(0, 0, len(rp) - 1)
    check_all_variants(rp, cols, vals, x, 1, 0, "c1 wpk1",
                       shapes=tuple((0, 32 * w) for w in range(1, 17)))
    k2 = wk().structure2().scan(len(cols), len(rp) - 1, vals, rp, cols, len(rp) - 1)
    lo, hi = k2.min_nz, k2.max_nz
    assert (lo, hi) == (4, 9)
    inc = max(int((hi - lo) * 0.1), 1)
    for th in range(lo, hi + 1, inc):
        check_all_variants(rp, cols, vals, x, 2, th, f"c1 wpk2 th={th}",
                           shapes=tuple((0, 32 * w) for w in (2, 4, 8, 16)))


def test_empty_rows_are_not_written():
    rp = np.array([0, 2, 2, 3, 3], np.int32)
    cols = np.array([0, 3, 1], np.int32)
    vals = np.array([1.0, 2.0, 3.0])
    x = np.array([1.0, 2.0, 3.0, 4.0])
    for kind in (1, 2):
        _, eng = make(kind, rp, cols, vals, 1)
        for order in (0, 1):
            y = run(eng, x, order=order, y0=-7.0)
            assert list(y) == [9.0, -7.0, 6.0, -7.0]


def test_launch_shape_checks():
    rng = np.random.default_rng(1)
    rp, cols, vals = random_csr(rng, 2000, 9)
    k, eng = make(1, rp, cols, vals)
    t = torch()
    dx = t.ones(2000, dtype=t.float64, device="cuda")
    dy = t.zeros(2000, dtype=t.float64, device="cuda")
    with pytest.raises(wk().WKError, match="nblocks"):
        eng.run(1, 64, dx, dy)
    with pytest.raises(wk().WKError, match="blocksize"):
        eng.run(1000, 48, dx, dy)
    nb = (k.nwarps + 3) // 4
    eng.run(nb, 128, dx, dy)  # the drivers' exact grid is accepted


def test_device_generator_matches_cpu_generator():
    t = torch()
    for args, mode in (((2, 20, 17, 0, 1), 0), ((3, 5, 4, 3, 3), 1), ((2, 6, 6, 0, 2), 1), ((3, 2, 2, 2, 1), 0)):
        rp, cols, vals = O.fe_matrix(*args, value_mode=mode, seed=5)
        drp, dcols, dvals = wk().fe.fe_matrix(*args, value_mode=mode, seed=5)
        assert np.array_equal(drp.cpu().numpy(), rp)
        assert np.array_equal(dcols.cpu().numpy(), cols)
        assert np.array_equal(bits(dvals.cpu().numpy()), bits(vals)), args
    x = O.uniform_vec(3, 1, 1000)
    assert np.array_equal(bits(wk().fe.uniform_vec(3, 1, 1000).cpu().numpy()), bits(x))
    assert t.cuda.is_available()


def test_compressed_columns_bit_identical_to_uncompressed():
    """16-bit column storage changes only the bytes streamed, not the sums."""
    t = torch()
    rng = np.random.default_rng(12)
    cases = [O.fe_matrix(3, 10, 10, 10, 3, value_mode=1, seed=3), O.fe_matrix(2, 70, 70, 0, 1, value_mode=0),
             random_csr(rng, 200_000, 30, p_empty=0.1)]  # random columns: wide warps
    for rp, cols, vals in cases:
        n = len(rp) - 1
        x = rng.uniform(-1, 1, n)
        for kind, th in ((1, 0), (2, 5)):
            for dtype, tdt in (("f64", t.float64), ("f32", t.float32), ("bf16", t.bfloat16)):
                k = wk().structure() if kind == 1 else wk().structure2()
                k.scan(len(cols), n, None, rp, None, *(() if kind == 1 else (th,)))
                dv = wk().fe.convert(t.from_numpy(vals).cuda(), tdt)
                eng = wk().engine(k, dv, t.from_numpy(cols).cuda(), dtype=dtype)
                dx = wk().fe.convert(t.from_numpy(x).cuda(), tdt)
                ydt = t.float64 if dtype == "f64" else t.float32
                y0 = t.zeros(n, dtype=ydt, device="cuda")
                eng.run(0, 128, dx, y0, order=0)
                wide = eng.compress_cols()
                y1 = t.zeros(n, dtype=ydt, device="cuda")
                eng.run(0, 128, dx, y1, order=0)
                assert t.equal(y0, y1), (dtype, kind, wide)
                y2 = t.zeros(n, dtype=ydt, device="cuda")
                eng.run_x(0, 128, dx, y2, order=0)  # run_x path of the compressed kernel
                rm = t.from_numpy(k.row_map[:k.nznrows].astype(np.int64)).cuda()
                assert t.equal(y2[:k.nznrows], y1[rm]), (dtype, kind)  # y'[p] = y[row_map[p]]
                # set_colinds rebuilds the compact storage
                eng.device_colinds = eng.device_colinds
                y3 = t.zeros(n, dtype=ydt, device="cuda")
                eng.run(0, 128, dx, y3, order=0)
                assert t.equal(y0, y3)
        if n == 200_000:
            assert wide > 0  # random columns leave warps in 32-bit mode


def test_concurrent_streams_give_the_sequential_results():
    """Calls are stream-ordered and handles independent: two engines (and
    one engine on two output vectors) launched on two streams without
    synchronising in between give the results of sequential runs."""
    t = torch()
    rp1, c1, v1 = O.fe_matrix(3, 10, 9, 8, 3, value_mode=1, seed=11)
    rp2, c2, v2 = O.fe_matrix(2, 150, 140, 0, 1, value_mode=0, seed=12)
    e1 = make(2, rp1, c1, v1, th=81)[1]
    e2 = make(1, rp2, c2, v2)[1]
    n1, n2 = len(rp1) - 1, len(rp2) - 1
    x1 = t.from_numpy(O.uniform_vec(1, 0, n1)).cuda()
    x2 = t.from_numpy(O.uniform_vec(2, 0, n2)).cuda()
    ref = []
    for e, x, n in ((e1, x1, n1), (e2, x2, n2), (e1, x1, n1)):
        y = t.zeros(n, dtype=t.float64, device="cuda")
        e.run(0, 128, x, y, order=0, timed=False)
        t.cuda.synchronize()
        ref.append(y)
    s1, s2 = t.cuda.Stream(), t.cuda.Stream()
    ys = [t.full((n,), float("nan"), dtype=t.float64, device="cuda") for n in (n1, n2, n1)]
    t.cuda.synchronize()
    for rep in range(20):
        e1.run(0, 128, x1, ys[0], order=0, stream=s1, timed=False)
        e2.run(0, 128, x2, ys[1], order=0, stream=s2, timed=False)
        e1.run(0, 128, x1, ys[2], order=0, stream=s2, timed=False)
    t.cuda.synchronize()
    for y, r in zip(ys, ref):
        assert t.equal(y, r)


@pytest.mark.parametrize("dtype", ["f64", "f32", "bf16", "f16s"])
def test_fast_order_on_short_warps_is_the_exact_order(dtype):
    """Layouts whose slot-weighted mean step count is below the type's
    crossover (2-D Q1, 9 entries per row: 9 steps) run the one-slot-per-step
    kernel in fast order: same bits as WK_ORDER_EXACT, for both x paths and
    with 16-bit columns.  A long-warp layout (hex, 3 dof: 81 steps) takes the
    vector path and stays within the fast-order tolerance."""
    t = torch()
    tdt = {"f64": t.float64, "f32": t.float32, "bf16": t.bfloat16, "f16s": t.float32}[dtype]
    ydt = t.float64 if dtype == "f64" else t.float32
    for rp, cols, vals, short in ((*O.fe_matrix(2, 60, 60, 0, 1, value_mode=1, seed=2), True),
                                  (*O.fe_matrix(3, 8, 8, 8, 3, value_mode=1, seed=2), False)):
        n = len(rp) - 1
        k = wk().structure()
        k.scan(len(cols), n, None, rp)
        eng = wk().engine(k, wk().fe.convert(t.from_numpy(vals).cuda(), tdt), t.from_numpy(cols).cuda(), dtype=dtype)
        x = wk().fe.convert(t.from_numpy(O.uniform_vec(5, 0, n)).cuda(), tdt)
        ys = {}
        for comp in (False, True):
            if comp:
                eng.compress_cols()
            for cache in (True, False):
                for order in (0, 1):
                    y = t.zeros(n, dtype=ydt, device="cuda")
                    eng.run(0, 128, x, y, cache=cache, order=order)
                    ys[(comp, cache, order)] = y
        for key, y in ys.items():
            assert t.equal(y, ys[(False, True, 1)]) or not short, (dtype, key)
            if not short:
                ref = ys[(False, True, 1)].double()
                rel = float((y.double() - ref).norm() / ref.norm())
                assert rel < (1e-12 if dtype == "f64" else 1e-5), (dtype, key, rel)


def test_run_calls_capture_into_a_cuda_graph():
    """wk_run / wk_run_x with timed=False are plain stream-ordered launches:
    captured into a CUDA graph and replayed, they give the bits of direct
    calls (fast and exact order, WPK1 and WPK2)."""
    t = torch()
    rp, cols, vals = O.fe_matrix(2, 40, 40, 0, 1, value_mode=0, seed=0)
    n = len(rp) - 1
    for kind, th in ((1, 0), (2, 3)):
        k, eng = make(kind, rp, cols, vals, th)
        x = t.from_numpy(O.uniform_vec(0, 0, n)).cuda()
        for order in (0, 1):
            direct = t.zeros(n, dtype=t.float64, device="cuda")
            eng.run(0, 128, x, direct, order=order)
            y = t.zeros(n, dtype=t.float64, device="cuda")
            s = t.cuda.Stream()
            s.wait_stream(t.cuda.current_stream())
            with t.cuda.stream(s):
                eng.run(0, 128, x, y, order=order, timed=False)  # warm-up outside capture
            t.cuda.current_stream().wait_stream(s)
            g = t.cuda.CUDAGraph()
            with t.cuda.graph(g):
                eng.run(0, 128, x, y, order=order, timed=False)
            y.zero_()
            for _ in range(3):
                g.replay()
            t.cuda.synchronize()
            assert t.equal(y, direct), (kind, order)


@pytest.mark.parametrize("dtype", ["f64", "f32", "bf16", "f16s"])
def test_vector_path_warps_of_every_step_count(dtype):
    """Warps of 1-40 steps among long warps (so the layout takes the vector
    path for all of them): no unit, exact multiples of the slots per lane
    (4 / 8 / 16) and every remainder.  Fast order against the exact order of
    the same engine, within the type's accumulation tolerance, with 32-bit
    and 16-bit columns."""
    t = torch()
    rng = np.random.default_rng(31)
    lens = [120] * 40 + list(range(1, 41))  # one warp (32 rows) per length
    n = 32 * len(lens)
    rp = np.zeros(n + 1, np.int64)
    rp[1:] = np.cumsum(np.repeat(lens, 32))
    cols = rng.integers(0, n, int(rp[-1])).astype(np.int32)
    vals = rng.uniform(-1, 1, int(rp[-1]))
    rp = rp.astype(np.int32)
    tdt = {"f64": t.float64, "f32": t.float32, "bf16": t.bfloat16, "f16s": t.float32}[dtype]
    ydt = t.float64 if dtype == "f64" else t.float32
    k = wk().structure()
    k.scan(len(cols), n, None, rp)
    eng = wk().engine(k, wk().fe.convert(t.from_numpy(vals).cuda(), tdt), t.from_numpy(cols).cuda(), dtype=dtype)
    x = wk().fe.convert(t.from_numpy(rng.uniform(-1, 1, n)).cuda(), tdt)
    ys = {}
    for comp in (False, True):
        if comp:
            eng.compress_cols()
        for order in (0, 1):
            y = t.zeros(n, dtype=ydt, device="cuda")
            eng.run(0, 128, x, y, order=order)
            ys[(comp, order)] = y.double()
    tol = 1e-13 if dtype == "f64" else 1e-5
    ref = ys[(False, 1)]
    for key, y in ys.items():
        err = (y - ref).abs().max().item() / ref.abs().max().item()
        assert err < tol, (dtype, key, err)
    assert t.equal(ys[(True, 0)], ys[(False, 0)])  # 16-bit columns: the same sums
