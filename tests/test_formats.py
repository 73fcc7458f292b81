"""The data formats either side of the SpMV, on the CPU: the oracle's
reorder_columns_rowsort and assembly against the reference's own outputs
(golden fixtures and, where it was built, the reference compiled here), and
the library's Matrix Market reader (host code, no CUDA call) against
scipy's."""
import os

import numpy as np
import pytest

from conftest import golden_cases, random_csr
from oracle import wk_oracle as O


def canonical_rowsort(rp, cols_out, src):
    """reorder_A_rows with each run of equal columns in a row put in
    ascending order: the reference's std::sort leaves the order of equal
    columns unspecified, so two valid results agree on this form."""
    row = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    return src[np.lexsort((src, cols_out, row))]


def check_rowsort(rp, cols, L, out, src):
    """Properties of a row-sorted result, independent of any implementation."""
    rmi = L.arrays["row_map_inv"] if hasattr(L, "arrays") else L.layout.row_map_inv
    for r in range(len(rp) - 1):
        a, b = rp[r], rp[r + 1]
        assert np.all(np.diff(out[a:b]) >= 0)
        assert sorted(src[a:b]) == list(range(a, b))
    np.testing.assert_array_equal(out, rmi[cols[src]])


def test_rowsort_and_assembly_match_golden(golden):
    checked = 0
    for name, rp, cols, vals, x, layouts in golden_cases(golden):
        for kind, th in layouts:
            tag = f"{name}/k{kind}_t{th}"
            with O.OracleLayout(rp, kind=kind, threshold=th) as L:
                out, src = L.reorder_columns_rowsort(rp, cols)
                np.testing.assert_array_equal(out, golden[f"{tag}/cols_rowsort"], err_msg=tag)
                np.testing.assert_array_equal(canonical_rowsort(rp, out, src),
                                              canonical_rowsort(rp, out, golden[f"{tag}/reorder_A_rows"]),
                                              err_msg=tag)
                check_rowsort(rp, cols, L, out, src)
                if f"{tag}/y_assembly" in golden:
                    y = L.assembly(golden[f"{tag}/pvals"])
                    ref = golden[f"{tag}/y_assembly"]
                    nz_rows = L.layout.row_map[:L.layout.nznrows]
                    np.testing.assert_array_equal(y[nz_rows].view(np.int64), ref[nz_rows].view(np.int64),
                                                  err_msg=tag)
                    checked += 1
    assert checked >= 6


def test_assembly_is_row_sums_in_slot_order():
    rng = np.random.default_rng(5)
    rp, cols, vals = random_csr(rng, 500, 40, p_empty=0.1)
    for kind, th in ((1, 0), (2, 3), (2, 12)):
        with O.OracleLayout(rp, kind=kind, threshold=th) as L:
            pv, _ = L.process(vals, cols)
            y = L.assembly(pv)
            sums = np.array([vals[rp[r]:rp[r + 1]].sum() for r in range(len(rp) - 1)])
            assert np.allclose(y, sums, rtol=1e-12, atol=1e-12)


@pytest.mark.skipif(not O.RefLib.available(), reason="reference not built here (make -C oracle ref)")
def test_rowsort_and_assembly_match_reference_random():
    R = O.RefLib()
    rng = np.random.default_rng(11)
    for trial in range(6):
        n = int(rng.integers(33, 700))
        rp, cols, vals = random_csr(rng, n, 60, p_empty=0.15)
        for kind, th in ((1, 0), (2, int(rng.integers(1, 30)))):
            s = R.scan(rp, kind, th)
            ro, rsrc = s.reorder_columns_rowsort(rp, cols)
            with O.OracleLayout(rp, kind=kind, threshold=th) as L:
                out, src = L.reorder_columns_rowsort(rp, cols)
                np.testing.assert_array_equal(out, ro)
                np.testing.assert_array_equal(canonical_rowsort(rp, out, src), canonical_rowsort(rp, ro, rsrc))
                if kind == 1 and L.layout.nwarps:
                    pv, _ = L.process(vals, cols)
                    yr = s.assembly_wpk1(pv)
                    y = L.assembly(pv)
                    m = L.layout.row_map[:L.layout.nznrows]
                    np.testing.assert_array_equal(y[m].view(np.int64), yr[m].view(np.int64))
            s.free()


# ---- Matrix Market ------------------------------------------------------------------

def _lib_or_skip():
    from warpkernel_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    import warpkernel_gb300 as wk
    return wk


def _write_mm(path, m, n, entries, field="real", sym="general", comments=("generated",)):
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {sym}\n")
        for c in comments:
            f.write(f"% {c}\n")
        f.write(f"{m} {n} {len(entries)}\n")
        for e in entries:
            f.write(" ".join(repr(v) if isinstance(v, float) else str(v) for v in e) + "\n")


def _scipy_csr(path):
    sio = pytest.importorskip("scipy.io")
    A = sio.mmread(path, spmatrix=True).tocoo() if "spmatrix" in sio.mmread.__code__.co_varnames \
        else sio.mmread(path).tocoo()
    order = np.lexsort((A.col, A.row))  # stable: duplicates keep their order
    r, c, v = A.row[order], A.col[order], A.data[order]
    rp = np.zeros(A.shape[0] + 1, np.int64)
    np.add.at(rp, r + 1, 1)
    return np.cumsum(rp), c, v.astype(np.float64), A.shape


@pytest.mark.parametrize("sym", ["general", "symmetric", "skew-symmetric"])
def test_matrix_market_reader_matches_scipy(tmp_path, sym):
    wk = _lib_or_skip()
    rng = np.random.default_rng({"general": 1, "symmetric": 2, "skew-symmetric": 3}[sym])
    m = n = 57
    ents = set()
    while len(ents) < 300:
        i, j = (int(v) for v in rng.integers(1, m + 1, 2))
        if sym != "general" and i < j:
            i, j = j, i
        if sym == "skew-symmetric" and i == j:
            continue
        ents.add((i, j))
    ents = [(i, j, float(rng.standard_normal())) for i, j in sorted(ents, key=lambda e: rng.random())]
    p = str(tmp_path / f"a_{sym}.mtx")
    _write_mm(p, m, n, ents, sym=sym)
    A = wk.read_matrix_market_file(p)
    rp, c, v, shape = _scipy_csr(p)
    assert (A.num_rows, A.num_cols) == shape
    np.testing.assert_array_equal(A.row_offsets, rp)
    np.testing.assert_array_equal(A.column_indices, c)
    np.testing.assert_array_equal(A.values, v)


def test_matrix_market_pattern_integer_rectangular_and_empty(tmp_path):
    wk = _lib_or_skip()
    p = str(tmp_path / "pat.mtx")
    _write_mm(p, 3, 5, [(3, 5), (1, 2), (3, 1), (1, 2)], field="pattern")
    A = wk.read_matrix_market_file(p)
    assert (A.num_rows, A.num_cols, A.num_entries) == (3, 5, 4)
    np.testing.assert_array_equal(A.row_offsets, [0, 2, 2, 4])
    np.testing.assert_array_equal(A.column_indices, [1, 1, 0, 4])  # duplicates kept, in file order
    np.testing.assert_array_equal(A.values, [1, 1, 1, 1])
    p = str(tmp_path / "int.mtx")
    _write_mm(p, 2, 2, [(2, 1, 7), (1, 1, -3)], field="integer")
    A = wk.read_matrix_market_file(p)
    np.testing.assert_array_equal(A.values, [-3.0, 7.0])
    p = str(tmp_path / "empty.mtx")
    _write_mm(p, 4, 4, [])
    A = wk.read_matrix_market_file(p)
    np.testing.assert_array_equal(A.row_offsets, [0, 0, 0, 0, 0])
    assert A.num_entries == 0


@pytest.mark.parametrize("text,needle", [
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", "coordinate"),
    ("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n", "field"),
    ("%%MatrixMarket matrix coordinate real hermitian\n1 1 1\n1 1 1\n", "symmetry"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n", "entries"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n", "bad entry"),
    ("not a header\n", "header"),
])
def test_matrix_market_reader_rejects_malformed(tmp_path, text, needle):
    wk = _lib_or_skip()
    p = tmp_path / "bad.mtx"
    p.write_text(text)
    with pytest.raises(wk.WKError) as ei:
        wk.read_matrix_market_file(str(p))
    assert ei.value.status == 1 and needle in str(ei.value)
    with pytest.raises(wk.WKError):
        wk.read_matrix_market_file(str(tmp_path / "missing.mtx"))
