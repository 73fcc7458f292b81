"""The callers and data formats either side of the SpMV on the GPU:
reorder_columns_rowsort, run_assembly, layout files and Matrix Market input,
against the reference's own outputs (golden) and the oracle."""
import numpy as np
import pytest

from conftest import golden_cases, random_csr
from oracle import wk_oracle as O
from test_formats import _write_mm, canonical_rowsort, check_rowsort

pytestmark = pytest.mark.gpu


def wk():
    import warpkernel_gb300
    return warpkernel_gb300


def torch():
    import torch as t
    return t


def scan(kind, rp, th=0):
    k = wk().structure() if kind == 1 else wk().structure2()
    if kind == 1:
        k.scan(int(rp[-1]), len(rp) - 1, None, rp)
    else:
        k.scan(int(rp[-1]), len(rp) - 1, None, rp, None, th)
    return k


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


# ---- reorder_columns_rowsort ----------------------------------------------------------

def test_rowsort_matches_reference_outputs(golden):
    for name, rp, cols, vals, x, layouts in golden_cases(golden):
        for kind, th in layouts:
            tag = f"{name}/k{kind}_t{th}"
            k = scan(kind, rp, th)
            out = k.reorder_columns_rowsort(cols, rp)
            np.testing.assert_array_equal(out, golden[f"{tag}/cols_rowsort"], err_msg=tag)
            np.testing.assert_array_equal(canonical_rowsort(rp, out, k.reorder_A_rows),
                                          canonical_rowsort(rp, out, golden[f"{tag}/reorder_A_rows"]), err_msg=tag)
            with O.OracleLayout(rp, kind=kind, threshold=th) as L:
                oo, osrc = L.reorder_columns_rowsort(rp, cols)
                # equal columns keep CSR order on both sides: bit-exact
                np.testing.assert_array_equal(k.reorder_A_rows, osrc, err_msg=tag)


def test_rowsort_long_rows_device_arrays_and_duplicates():
    t = torch()
    rng = np.random.default_rng(3)
    n = 3000
    lens = rng.integers(0, 30, n)
    lens[[5, 700, 2999]] = [2999, 1500, 2500]  # long rows (below nrows for WPK2)
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    cols = rng.integers(0, 40, int(rp[-1])).astype(np.int32)  # many equal columns per row
    for kind, th in ((1, 0), (2, 7)):
        k = scan(kind, rp, th)
        out_h = k.reorder_columns_rowsort(cols, rp)
        src_h = k.reorder_A_rows.copy()
        out_d = k.reorder_columns_rowsort(t.from_numpy(cols).cuda(), rp)
        np.testing.assert_array_equal(out_d.cpu().numpy(), out_h)
        np.testing.assert_array_equal(k.reorder_A_rows.cpu().numpy(), src_h)
        with O.OracleLayout(rp, kind=kind, threshold=th) as L:
            oo, osrc = L.reorder_columns_rowsort(rp, cols)
            np.testing.assert_array_equal(out_h, oo)
            np.testing.assert_array_equal(src_h, osrc)
            check_rowsort(rp, cols, L, out_h, src_h)


def test_rowsort_rejects_non_square_columns():
    rp = np.array([0, 2, 3], np.int32)
    k = scan(1, rp)
    with pytest.raises(wk().WKError) as ei:
        k.reorder_columns_rowsort(np.array([0, 2, 1], np.int32), rp)
    assert ei.value.status == 1


def test_rowsort_driver_sequence_runs_and_verifies():
    """optimize2.cu:740-796: scan, reorder_columns_rowsort, reorder_x,
    values gathered through reorder_A_rows, engine, run_x, verify_x; the
    exact order is bit-identical to the oracle's run_x on the same arrays."""
    t = torch()
    rp, cols, vals = O.fe_matrix(3, 6, 5, 4, 3, value_mode=1, seed=4)
    n = len(rp) - 1
    x = O.uniform_vec(9, 0, n)
    y_ref = O.csr_spmv(rp, cols, vals, x)
    for kind, th in ((1, 0), (2, 10)):
        k = scan(kind, rp, th)
        rcols = k.reorder_columns_rowsort(cols, rp)
        xr = k.reorder_x(x)
        new_vals = vals[k.reorder_A_rows]
        eng = wk().engine(k, new_vals, rcols)
        dy = t.zeros(n, dtype=t.float64, device="cuda")
        eng.run_x(0, 128, xr, dy, order=wk().WK_ORDER_EXACT)
        y = dy.cpu().numpy()
        assert eng.verify_x(y_ref, y, strict=True)
        with O.OracleLayout(rp, kind=kind, threshold=th) as L:
            pv, pc = L.process(new_vals, rcols)
            yo = L.run_x(pv, pc, L.reorder_x(x))
        np.testing.assert_array_equal(bits(y), bits(yo))
        # reorder_values_coalesced_rowsort gives the engine's slot array
        np.testing.assert_array_equal(k.reorder_values_coalesced_rowsort(vals), eng.device_values)


# ---- run_assembly ----------------------------------------------------------------------

def test_assembly_matches_reference_kernel(golden):
    t = torch()
    checked = 0
    for name, rp, cols, vals, x, layouts in golden_cases(golden):
        tag = f"{name}/k1_t0"
        if f"{tag}/y_assembly" not in golden:
            continue
        k = scan(1, rp)
        eng = wk().engine(k, vals, cols)
        np.testing.assert_array_equal(eng.device_values, golden[f"{tag}/pvals"])
        dy = t.full((k.nrows,), -7.0, dtype=t.float64, device="cuda")
        sec = eng.run_assembly(0, 128, dy)
        assert sec >= 0
        y = dy.cpu().numpy()
        m = k.row_map[:k.nznrows]
        np.testing.assert_array_equal(bits(y[m]), bits(golden[f"{tag}/y_assembly"][m]), err_msg=tag)
        empty = np.setdiff1d(np.arange(k.nrows), m)
        assert np.all(y[empty] == -7.0)  # rows without entries are not written
        checked += 1
    assert checked >= 6


@pytest.mark.parametrize("dtype", ["f64", "f32", "bf16"])
def test_assembly_wpk1_wpk2_against_oracle(dtype):
    t = torch()
    rng = np.random.default_rng(21)
    rp, cols, vals = random_csr(rng, 4000, 90, p_empty=0.05)
    n = len(rp) - 1
    for kind, th in ((1, 0), (2, 4), (2, 40)):
        k = scan(kind, rp, th)
        v = vals
        if dtype == "bf16":
            v = t.from_numpy(vals).to(t.bfloat16).float().double().numpy()  # the stored values
        eng = wk().engine(k, t.from_numpy(vals).to({"f64": t.float64, "f32": t.float32,
                                                    "bf16": t.bfloat16}[dtype]).cuda(), t.from_numpy(cols).cuda(),
                          dtype=dtype)
        ydt = t.float64 if dtype == "f64" else t.float32
        dy = t.zeros(n, dtype=ydt, device="cuda")
        for nb, bs in ((0, 0), (0, 64), ((k.nwarps + 7) // 8, 256)):
            eng.run_assembly(nb, bs, dy, timed=False)
            t.cuda.synchronize()
            y = dy.double().cpu().numpy()
            with O.OracleLayout(rp, kind=kind, threshold=th) as L:
                pv, _ = L.process(v if dtype != "f32" else vals.astype(np.float32).astype(np.float64), cols)
                yo = L.assembly(pv)
            if dtype == "f64":
                np.testing.assert_array_equal(bits(y), bits(yo))
            else:
                scale = np.abs(v).max() * 90
                assert np.max(np.abs(y - yo)) <= 1e-5 * scale


def test_assembly_rejects_bad_launch_shape():
    rp, cols, vals = O.fe_matrix(2, 20, 20, 0, 1, value_mode=0)
    k = scan(1, rp)
    eng = wk().engine(k, vals, cols)
    dy = torch().zeros(k.nrows, dtype=torch().float64, device="cuda")
    with pytest.raises(wk().WKError):
        eng.run_assembly(1, 32, dy)  # one warp cannot cover every layout warp
    with pytest.raises(wk().WKError):
        eng.run_assembly(1000, 48, dy)  # not a multiple of 32


# ---- layout files ------------------------------------------------------------------------

@pytest.mark.parametrize("kind,th", [(1, 0), (2, 0), (2, 9)])
def test_layout_save_load_roundtrip(tmp_path, kind, th):
    t = torch()
    rng = np.random.default_rng(kind * 10 + th)
    rp, cols, vals = random_csr(rng, 1500, 70, p_empty=0.1)
    n = len(rp) - 1
    k = scan(kind, rp, th)
    p = str(tmp_path / "layout.wpk")
    k.save(p)
    k2 = (wk().structure() if kind == 1 else wk().structure2()).load(p)
    assert k2.info() == k.info()
    fields = ["row_map", "row_map_inv", "reorder_rows", "warp_offsets", "max_nz_rows"]
    if kind == 2:
        fields += ["threads_per_row", "row_offset_warp"]
    for f in fields:
        np.testing.assert_array_equal(getattr(k2, f), getattr(k, f), err_msg=f)
    x = t.from_numpy(O.uniform_vec(2, 0, n)).cuda()
    ys = []
    for kk in (k, k2):
        eng = wk().engine(kk, vals, cols)
        np.testing.assert_array_equal(eng.device_values, wk().engine(k, vals, cols).device_values)
        dy = t.zeros(n, dtype=t.float64, device="cuda")
        eng.run(0, 128, x, dy)
        ys.append(dy.cpu().numpy())
    np.testing.assert_array_equal(bits(ys[0]), bits(ys[1]))
    # a file of the other kind is refused by the class
    other = wk().structure2() if kind == 1 else wk().structure()
    with pytest.raises(ValueError):
        other.load(p)


def test_layout_load_rejects_corrupt_files(tmp_path):
    rng = np.random.default_rng(8)
    rp, cols, vals = random_csr(rng, 300, 20)
    k = scan(2, rp, 5)
    p = tmp_path / "l.wpk"
    k.save(str(p))
    raw = p.read_bytes()
    cases = {
        "magic": b"XXXX" + raw[4:],
        "truncated": raw[:len(raw) // 2],
        "empty": b"",
    }
    # a row_map entry out of range: the first array follows the header
    hdr = 8 + 4 + 10 * 4 + 8  # magic, version, wk_layout_info, array length
    bad = bytearray(raw)
    bad[hdr:hdr + 4] = (10 ** 6).to_bytes(4, "little")
    cases["row_map"] = bytes(bad)
    for what, data in cases.items():
        q = tmp_path / f"bad_{what}.wpk"
        q.write_bytes(data)
        with pytest.raises(wk().WKError) as ei:
            wk().structure2().load(str(q))
        assert ei.value.status == 1, what
    with pytest.raises(wk().WKError):
        wk().structure2().load(str(tmp_path / "missing.wpk"))


# ---- Matrix Market to SpMV -----------------------------------------------------------------

def test_matrix_market_file_to_spmv(tmp_path):
    """wpk1.cu's sequence from a file: read, scan, engine, run, verify."""
    t = torch()
    rp, cols, vals = O.fe_matrix(2, 30, 25, 0, 2, value_mode=1, seed=6)
    n = len(rp) - 1
    ents = []
    for r in range(n):
        for q in range(rp[r], rp[r + 1]):
            if cols[q] <= r:  # lower triangle of the symmetric matrix
                ents.append((r + 1, int(cols[q]) + 1, float(vals[q])))
    p = str(tmp_path / "fe.mtx")
    _write_mm(p, n, n, ents, sym="symmetric")
    A = wk().read_matrix_market_file(p)
    np.testing.assert_array_equal(A.row_offsets, rp)
    np.testing.assert_array_equal(A.column_indices, cols)
    np.testing.assert_allclose(A.values, vals, rtol=0, atol=0)
    x = O.uniform_vec(1, 0, n)
    for kind, th in ((1, 0), (2, 4)):
        k = scan(kind, A.row_offsets, th)
        eng = wk().engine(k, A.values, A.column_indices)
        dy = t.zeros(n, dtype=t.float64, device="cuda")
        eng.run(0, 128, t.from_numpy(x).cuda(), dy)
        assert eng.verify(O.csr_spmv(rp, cols, vals, x), dy.cpu().numpy())
