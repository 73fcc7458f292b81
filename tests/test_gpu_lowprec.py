"""FP32 and BF16 storage (FP32 accumulation) against the oracle's FP32
restatement of the documented order (wko_run_lp): the device rounds fp64
values and x exactly as the oracle does, the exact order gives the oracle's
bits, the fast order stays within REL_TOL_FAST of it, and the 16-bit column
storage changes no bit in either `run` or `run_x`."""
import numpy as np
import pytest

from conftest import random_csr
from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu

REL_TOL_FAST = 1e-6   # normwise relative, FP32 accumulation re-associated
REL_TOL_F32_VS_F64 = 1e-6  # FP32 storage against the fp64 product


def _wk():
    import warpkernel_gb300
    return warpkernel_gb300


def _t():
    import torch
    return torch


def _stored(dtype, a):
    """The oracle's rounding of fp64 `a` to the stored type (float32, or
    uint16 bf16 bits)."""
    return O.round_f32(a) if dtype == "f32" else O.round_bf16(a)


def _dev_bits(t):
    a = t.cpu()
    if a.dtype == _t().bfloat16:
        return a.view(_t().int16).numpy().view(np.uint16)
    return a.numpy()


def relerr(y, ref):
    ref = np.asarray(ref, np.float64)
    d = np.linalg.norm(ref)
    return float(np.linalg.norm(np.asarray(y, np.float64) - ref) / (d if d else 1.0))


def cases():
    rng = np.random.default_rng(44)
    yield "hex 8^3 x3", O.fe_matrix(3, 8, 8, 8, 3, value_mode=1, seed=2), ((1, 0), (2, 81), (2, 27), (2, 6))
    yield "q1 40^2", O.fe_matrix(2, 40, 40, 0, 1, value_mode=0, seed=0), ((1, 0), (2, 3))
    rp, cols, vals = random_csr(rng, 7000, 120, p_empty=0.15)
    yield "ragged+empty", (rp, cols, vals), ((1, 0), (2, 17), (2, 1))
    lens = [150] * 40 + list(range(1, 41))  # long warps beside every short length
    n = 32 * len(lens)
    rp = np.zeros(n + 1, np.int64)
    rp[1:] = np.cumsum(np.repeat(lens, 32))
    cols = rng.integers(0, n, int(rp[-1])).astype(np.int32)
    yield "steps 1-40", (rp.astype(np.int32), cols, rng.uniform(-1, 1, int(rp[-1]))), ((1, 0), (2, 64))


def test_device_rounding_matches_the_oracle():
    """wk_convert (fp64 -> FP32 / BF16) gives the oracle's one-step
    round-to-nearest-even bits, including values where rounding through FP32
    first would differ (double rounding) and the BF16 subnormal range."""
    t = _t()
    rng = np.random.default_rng(3)
    a = rng.standard_normal(400_000) * 10.0 ** rng.integers(-44, 38, 400_000)
    a = np.concatenate([a, [0.0, -0.0, 2.0 ** -134 * (1 + 2.0 ** -30), 2.0 ** -133 * 1.5, 3.3e38, -3.39e38]])
    da = t.from_numpy(a).cuda()
    f = _wk().fe.convert(da, t.float32)
    b = _wk().fe.convert(da, t.bfloat16)
    assert np.array_equal(_dev_bits(f).view(np.uint32), O.round_f32(a).view(np.uint32))
    assert np.array_equal(_dev_bits(b), O.round_bf16(a))


@pytest.mark.parametrize("dtype", ["f32", "bf16"])
def test_exact_order_is_the_oracles_fp32_order(dtype):
    t = _t()
    wk = _wk()
    tdt = t.float32 if dtype == "f32" else t.bfloat16
    for name, (rp, cols, vals), layouts in cases():
        n = len(rp) - 1
        x = np.random.default_rng(n).uniform(-1, 1, n)
        dv = wk.fe.convert(t.from_numpy(vals).cuda(), tdt)
        dx = wk.fe.convert(t.from_numpy(x).cuda(), tdt)
        sv, sx = _stored(dtype, vals), _stored(dtype, x)
        assert np.array_equal(_dev_bits(dv), sv) and np.array_equal(_dev_bits(dx), sx)
        y64 = O.csr_spmv(rp, cols, vals, x)
        for kind, th in layouts:
            tag = (name, dtype, kind, th)
            k = wk.structure() if kind == 1 else wk.structure2()
            k.scan(len(cols), n, None, rp, None, *(() if kind == 1 else (th,)))
            eng = wk.engine(k, dv, t.from_numpy(cols).cuda(), dtype=dtype)
            with O.OracleLayout(rp, kind=kind, threshold=th) as o:
                pv = o.place(sv)
                _, pc = o.process(vals, cols)
                y_ref = o.run_lp(pv, pc, sx, mapped=True)
                pcr = o.reorder_columns_coalesced(cols)
                xr = sx[o.layout.row_map]  # reorder_x: x'[row_map_inv[r]] = x[r]
                yx_ref = o.run_lp(pv, pcr, xr, mapped=False)
            assert np.array_equal(eng.device_values.view(np.uint32 if dtype == "f32" else np.uint16),
                                  pv.view(np.uint32 if dtype == "f32" else np.uint16)), tag
            if dtype == "f32":
                assert relerr(y_ref, y64) < REL_TOL_F32_VS_F64, (tag, relerr(y_ref, y64))
            ys = {}
            for comp in (False, True):
                if comp:
                    eng.compress_cols()
                for cache in (True, False):
                    for order in (1, 0):
                        y = t.zeros(n, dtype=t.float32, device="cuda")
                        eng.run(0, 128, dx, y, cache=cache, order=order)
                        yh = y.cpu().numpy()
                        if order == 1:
                            assert np.array_equal(yh.view(np.uint32), y_ref.view(np.uint32)), (tag, comp, cache)
                        else:
                            assert relerr(yh, y_ref) < REL_TOL_FAST, (tag, comp, cache, relerr(yh, y_ref))
                        ys[(comp, cache, order)] = yh
            # 16-bit columns: the same sums as 32-bit columns in both orders
            for (comp, cache, order), yh in ys.items():
                assert np.array_equal(yh.view(np.uint32), ys[(False, cache, order)].view(np.uint32)), tag
            # run_x with the renumbered columns and the reordered x (WPK_r), on
            # a fresh engine so the first pass runs the 32-bit column kernel
            ex = wk.engine(k, dv, t.from_numpy(cols).cuda(), dtype=dtype)
            ex.device_colinds = pcr
            dxr = wk.fe.convert(t.from_numpy(x).cuda(), tdt)
            dxr = k.reorder_x(dxr)
            assert np.array_equal(_dev_bits(dxr), xr)
            yx = {}
            for comp in (False, True):
                if comp:
                    ex.compress_cols()
                for order in (1, 0):
                    y = t.zeros(n, dtype=t.float32, device="cuda")
                    ex.run_x(0, 128, dxr, y, order=order)
                    yh = y.cpu().numpy()
                    if order == 1:
                        assert np.array_equal(yh.view(np.uint32), yx_ref.view(np.uint32)), (tag, "run_x", comp)
                    else:
                        assert relerr(yh, yx_ref) < REL_TOL_FAST, (tag, "run_x fast", comp)
                    yx[(comp, order)] = yh
            assert np.array_equal(yx[(True, 0)].view(np.uint32), yx[(False, 0)].view(np.uint32)), tag


def test_compressed_run_x_on_original_columns_is_the_mapped_run():
    """run_x over the engine's original columns and x gives y'[p] =
    y[row_map[p]] of run, bit for bit, in the compressed fast kernel as in the
    uncompressed one."""
    t = _t()
    wk = _wk()
    rng = np.random.default_rng(12)
    for rp, cols, vals in (O.fe_matrix(3, 10, 10, 10, 3, value_mode=1, seed=3),
                           random_csr(rng, 200_000, 30, p_empty=0.1)):
        n = len(rp) - 1
        x = rng.uniform(-1, 1, n)
        for kind, th in ((1, 0), (2, 5)):
            for dtype, tdt in (("f32", t.float32), ("bf16", t.bfloat16)):
                k = wk.structure() if kind == 1 else wk.structure2()
                k.scan(len(cols), n, None, rp, None, *(() if kind == 1 else (th,)))
                eng = wk.engine(k, wk.fe.convert(t.from_numpy(vals).cuda(), tdt), t.from_numpy(cols).cuda(),
                                dtype=dtype)
                dx = wk.fe.convert(t.from_numpy(x).cuda(), tdt)
                rm = t.from_numpy(k.row_map.astype(np.int64)).cuda()
                nz = k.nznrows
                out = {}
                for comp in (False, True):
                    if comp:
                        eng.compress_cols()
                    y = t.zeros(n, dtype=t.float32, device="cuda")
                    eng.run(0, 128, dx, y, order=0)
                    yx = t.zeros(n, dtype=t.float32, device="cuda")
                    eng.run_x(0, 128, dx, yx, order=0)
                    assert t.equal(yx[:nz], y[rm[:nz]]), (dtype, kind, comp)
                    out[comp] = yx
                assert t.equal(out[True], out[False]), (dtype, kind)


def test_fp32_storage_error_against_fp64():
    """FP32 storage with FP32 accumulation stays within 1e-6 of the fp64
    product (hex 12^3, 3 dof); BF16's error is stated, not bounded by 1e-3:
    rounding the values and x to 8 significant bits alone gives ~2e-3."""
    t = _t()
    wk = _wk()
    rp, cols, vals = O.fe_matrix(3, 12, 12, 12, 3, value_mode=1, seed=2)
    n = len(rp) - 1
    x = O.uniform_vec(2, 0, n)
    y64 = O.csr_spmv(rp, cols, vals, x)
    k = wk.structure2()
    k.scan(len(cols), n, None, rp, None, 81)
    # the error of BF16-rounded inputs alone, summed exactly in fp64
    vb, xb = O.bf16_to_f32(O.round_bf16(vals)), O.bf16_to_f32(O.round_bf16(x))
    input_err = relerr(O.csr_spmv(rp, cols, vb.astype(np.float64), xb.astype(np.float64)), y64)
    for dtype, tdt in (("f32", t.float32), ("bf16", t.bfloat16)):
        eng = wk.engine(k, wk.fe.convert(t.from_numpy(vals).cuda(), tdt), t.from_numpy(cols).cuda(), dtype=dtype)
        dx = wk.fe.convert(t.from_numpy(x).cuda(), tdt)
        for order in (0, 1):
            y = t.zeros(n, dtype=t.float32, device="cuda")
            eng.run(0, 128, dx, y, order=order)
            err = relerr(y.cpu().numpy(), y64)
            if dtype == "f32":
                assert err < REL_TOL_F32_VS_F64, (order, err)
            else:
                # FP32 accumulation adds almost nothing to the rounding of the inputs
                assert abs(err - input_err) < 0.05 * input_err, (order, err, input_err)


@pytest.mark.parametrize("dtype", ["f32", "bf16", "f16s"])
def test_x_windows_give_the_same_bits(dtype):
    """Fast order with x windows staged in shared memory against the same
    engine with the windows switched off: the same bits for run and run_x,
    WPK1 and WPK2, block sizes of 1-32 warps (the 1,024-thread launch needs
    more than 48 KB of shared memory); FE matrices give most warps a window,
    random columns none."""
    t = _t()
    wk = _wk()
    tdt = t.bfloat16 if dtype == "bf16" else t.float32
    rng = np.random.default_rng(5)
    cases = [("hex 10^3 x3", O.fe_matrix(3, 10, 10, 10, 3, value_mode=1, seed=3), True),
             ("hex 6x7x40 x3", O.fe_matrix(3, 6, 7, 40, 3, value_mode=1, seed=4), True),
             ("q1 90^2", O.fe_matrix(2, 90, 90, 0, 1, value_mode=0, seed=1), False),
             ("random", random_csr(rng, 60_000, 90, p_empty=0.05), False)]
    for name, (rp, cols, vals), fe in cases:
        n = len(rp) - 1
        x = wk.fe.convert(t.from_numpy(rng.uniform(-1, 1, n)).cuda(), tdt)
        for kind, th in ((1, 0), (2, 40)):
            k = wk.structure() if kind == 1 else wk.structure2()
            k.scan(len(cols), n, None, rp, None, *(() if kind == 1 else (th,)))
            eng = wk.engine(k, wk.fe.convert(t.from_numpy(vals).cuda(), tdt), t.from_numpy(cols).cuda(), dtype=dtype)
            eng.compress_cols()
            nwin = eng.set_windows(True)
            if fe:
                assert nwin >= 0.5 * k.nwarps, (name, kind, nwin, k.nwarps)
            for bs in (32, 128, 1024):
                for mapped in (True, False):
                    out = {}
                    for on in (True, False):
                        eng.set_windows(on)
                        y = t.zeros(n, dtype=t.float32, device="cuda")
                        (eng.run if mapped else eng.run_x)(0, bs, x, y, order=0)
                        out[on] = y
                    assert t.equal(out[True], out[False]), (name, dtype, kind, bs, mapped)


def _window_case_sets():
    """Per layout warp: (sorted distinct columns relative to the warp's base,
    whether the warp gets an x window: at most 512 distinct columns in at
    most 32 runs, at most 32 chunks of <= 32 consecutive columns, and a
    span below 65,536)."""
    def runs(starts, length):
        return [s + i for s in starts for i in range(length)]
    cases = [
        (runs(range(0, 16 * 37, 37), 32), True),                               # 512 distinct, 16 chunks
        (runs(range(0, 16 * 37, 37), 32) + [16 * 37 + 5], False),              # 513 distinct
        (runs(range(0, 32 * 5, 5), 3), True),                                  # 32 runs, 32 chunks
        (runs(range(0, 33 * 5, 5), 3), False),                                 # 33 runs
        (runs(range(30, 30 + 12 * 47, 47), 40), True),                         # 2 chunks per run, 24 chunks;
                                                                               # runs cross bitmap words
        (runs(range(0, 7 * 70, 70), 65), True),                                # 3 chunks per run, 21 chunks
        (runs(range(0, 15 * 40, 40), 33) + [700, 710, 720], False),            # 33 chunks, 498 distinct
        (runs(range(0, 17 * 19, 19), 17), True),                               # odd run lengths
        (runs([0, 65535 - 31], 32), True),                                     # span 65,535
        (runs([0, 70000], 32), False),                                         # span above 65,535: 32-bit
    ]
    return cases


@pytest.mark.parametrize("dtype", ["f32", "f16s"])
def test_x_window_limits(dtype):
    """Warps built to sit on every limit of the x windows (distinct columns,
    runs, chunks after splitting runs longer than 32, bitmap word crossings,
    the 16-bit span): exactly the eligible warps get a window, and run /
    run_x give the same bits with the windows on and off, against the
    oracle's FP32 restatement within 1e-6."""
    t = _t()
    wk = _wk()
    rng = np.random.default_rng(21)
    cases = _window_case_sets()
    L, base_step = 32, 140_000
    rows, colsl = [], []
    for j, (cset, _) in enumerate(cases):
        S = len(cset)
        for i in range(32):
            idx = [(i * L + q) % S for q in range(L)]
            colsl.append(sorted(j * base_step + cset[q] for q in idx))
    n, ncols = len(colsl), len(cases) * base_step
    rp = np.arange(n + 1, dtype=np.int32) * L
    cols = np.concatenate(colsl).astype(np.int32)
    vals = rng.uniform(-1, 1, len(cols))
    x = rng.uniform(-1, 1, ncols)
    k = wk.structure()
    k.scan(len(cols), n, None, rp, None)
    assert k.nwarps == len(cases)
    eng = wk.engine(k, wk.fe.convert(t.from_numpy(vals).cuda(), t.float32), t.from_numpy(cols).cuda(), dtype=dtype,
                    ncols=ncols)
    wide = eng.compress_cols()
    assert wide == 1
    assert eng.set_windows(True) == sum(ok for _, ok in cases)
    xd = t.from_numpy(x).cuda().float()
    y_ref = O.csr_spmv(rp, cols, vals, x)
    for mapped in (True, False):
        out = {}
        for on in (True, False):
            eng.set_windows(on)
            y = t.zeros(n, dtype=t.float32, device="cuda")
            (eng.run if mapped else eng.run_x)(0, 128, xd, y, order=0)
            out[on] = y
        assert t.equal(out[True], out[False]), (dtype, mapped)
    yh = out[True].double().cpu().numpy()
    tol = REL_TOL_F32_VS_F64 if dtype == "f32" else 1e-3
    assert np.linalg.norm(yh - y_ref) / np.linalg.norm(y_ref) < tol
