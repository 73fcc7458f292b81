"""The WPK1 ablation layouts (wk_scan1_ablation) on the GPU: device-built
arrays bit-identical to the reference's optimization.cu scans (golden) and to
the oracle, warpKernel_nocoalesced bit-identical to the reference's, and the
calls that need interleaved slots refusing non-interleaved layouts."""
import numpy as np
import pytest

from conftest import golden_cases, random_csr
from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu

FIELDS = ("row_map", "row_map_inv", "reorder_rows", "warp_offsets", "max_nz_rows")


def wk():
    import warpkernel_gb300
    return warpkernel_gb300


def torch():
    import torch as t
    return t


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def run(eng, x, mapped=True, order=0, cache=True):
    t = torch()
    n = eng.kernel.nrows
    dy = t.zeros(n, dtype=t.float64, device="cuda")
    (eng.run if mapped else eng.run_x)(0, 128, t.from_numpy(np.ascontiguousarray(x)).cuda(), dy, cache=cache,
                                       order=order)
    return dy.cpu().numpy()


def test_ablation_layouts_and_nocoalesced_run_match_reference(golden):
    checked = 0
    for name, rp, cols, vals, x, layouts in golden_cases(golden):
        for v in (1, 2, 3):
            tag = f"{name}/abl{v}"
            if f"{tag}/info" not in golden:
                continue
            k = wk().structure().scan_ablation(len(cols), len(rp) - 1, rp, v)
            assert k.variant == v
            assert (k.nwarps, k.allocate_nz) == tuple(int(i) for i in golden[f"{tag}/info"])
            for f in FIELDS:
                np.testing.assert_array_equal(getattr(k, f), golden[f"{tag}/{f}"], err_msg=f"{tag} {f}")
            eng = wk().engine(k, vals, cols)
            if f"{tag}/y" in golden:
                for order in (0, 1):
                    for cache in (True, False):
                        y = run(eng, x, order=order, cache=cache)
                        np.testing.assert_array_equal(bits(y), bits(golden[f"{tag}/y"]), err_msg=tag)
            checked += 1
    assert checked >= 12


@pytest.mark.parametrize("v", [1, 2, 3])
def test_ablation_random_against_oracle(v):
    t = torch()
    rng = np.random.default_rng(40 + v)
    for p_empty in (0.0, 0.2):
        rp, cols, vals = random_csr(rng, 2500, 70, p_empty=p_empty)
        n = len(rp) - 1
        x = O.uniform_vec(3, v, n)
        k = wk().structure().scan_ablation(len(cols), n, rp, v)
        with O.OracleLayout(rp, ablation=v) as L:
            for f in FIELDS:
                np.testing.assert_array_equal(getattr(k, f), L.layout.arrays[f], err_msg=f)
            pv, pc = L.process(vals, cols)
            eng = wk().engine(k, vals, cols)
            np.testing.assert_array_equal(eng.device_values, pv)
            np.testing.assert_array_equal(eng.device_colinds, pc)
            y = run(eng, x, order=1)
            np.testing.assert_array_equal(bits(y), bits(L.run(pv, pc, x, fma=True)))
            # run_x with the renumbered columns and reordered x
            pcr = k.reorder_columns_coalesced(cols)
            np.testing.assert_array_equal(pcr, L.reorder_columns_coalesced(cols))
            eng.device_colinds = pcr
            yx = run(eng, L.reorder_x(x), mapped=False, order=1)
            np.testing.assert_array_equal(bits(yx), bits(L.run_x(pv, pcr, L.reorder_x(x), fma=True)))
            # host vectors
            yh = t.zeros(n, dtype=t.float64)
            eng.device_colinds = pc
            eng.run_host(t.from_numpy(x), yh, order=1)
            np.testing.assert_array_equal(bits(yh.numpy()), bits(y))


def test_nosort_layout_works_with_every_call():
    """A nosort layout is an ordinary interleaved WPK1 layout: fast order,
    compressed columns, residual and CG accept it."""
    t = torch()
    rp, cols, vals = O.fe_matrix(2, 40, 40, 0, 1, value_mode=0)
    n = len(rp) - 1
    k = wk().structure().scan_ablation(len(cols), n, rp, 1)
    eng = wk().engine(k, vals, cols)
    x = O.uniform_vec(1, 0, n)
    ref = O.csr_spmv(rp, cols, vals, x)
    y = run(eng, x, order=0)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-12
    eng.compress_cols()
    y2 = run(eng, x, order=0)
    np.testing.assert_array_equal(bits(y2), bits(y))
    b = t.from_numpy(ref).cuda()
    xs = t.zeros(n, dtype=t.float64, device="cuda")
    res = wk().wpk.cg(eng, b, xs, tol=1e-10)
    assert res["relres"] <= 1e-10
    assert np.linalg.norm(xs.cpu().numpy() - x) / np.linalg.norm(x) < 1e-6


def test_nocoalesced_layout_is_refused_where_slots_must_interleave(tmp_path):
    t = torch()
    rp, cols, vals = O.fe_matrix(2, 12, 12, 0, 1, value_mode=0)
    n = len(rp) - 1
    k = wk().structure().scan_ablation(len(cols), n, rp, 2)
    eng = wk().engine(k, vals, cols)
    z = t.zeros(n, dtype=t.float64, device="cuda")
    calls = [
        lambda: eng.compress_cols(),
        lambda: eng.residual(z, z, z.clone()),
        lambda: eng.run_assembly(0, 0, z),
        lambda: wk().wpk.cg(eng, z, z.clone()),
    ]
    for c in calls:
        with pytest.raises(wk().WKError) as ei:
            c()
        assert ei.value.status == 1 and "WK_ABL_NOCOALESCE" in str(ei.value)
    import ctypes as C
    h = C.c_void_p()
    assert wk().load().wk_adjoint_create(eng.handle, 1, 0, None, C.byref(h)) == 1
    # the layout file round trip keeps the variant
    p = str(tmp_path / "nc.wpk")
    k.save(p)
    k2 = wk().structure().load(p)
    assert k2.variant == 2 and k2.info() == k.info()
    np.testing.assert_array_equal(k2.reorder_rows, k.reorder_rows)
    with pytest.raises(wk().WKError):
        wk().structure().scan_ablation(len(cols), n, rp, 4)
