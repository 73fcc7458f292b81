"""The WPK1 ablation layouts of optimization.cu on the CPU: the oracle's
restatement against the reference's own scan / scan_nosort /
scan_nocoalesced / scan_nocoalesced_nosort and warpKernel_nocoalesced
(compiled here by `make -C oracle ref`) and against the golden fixtures made
from them."""
import numpy as np
import pytest

from conftest import golden_cases, random_csr
from oracle import wk_oracle as O

ABL = (1, 2, 3)  # nosort, nocoalesce, both


def full_rows(rng, n, maxlen):
    """Random CSR without empty rows (the optimization.cu nosort scans read
    past their row list when a row is empty)."""
    lens = rng.integers(1, maxlen + 1, n)
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    return rp, rng.integers(0, n, int(rp[-1])).astype(np.int32), rng.standard_normal(int(rp[-1]))


def layout_arrays(L):
    return {f: L.layout.arrays[f] for f in O.FIELDS[:5]}


@pytest.mark.skipif(not O.RefAblation.available(), reason="reference not built here (make -C oracle ref)")
def test_oracle_ablation_layouts_and_run_match_reference():
    rng = np.random.default_rng(3)
    for trial in range(8):
        n = int(rng.integers(1, 400))
        rp, cols, vals = full_rows(rng, n, int(rng.integers(1, 60)))
        x = rng.uniform(-1, 1, n)
        for v in (0,) + ABL:
            R = O.RefAblation(rp, v)
            with O.OracleLayout(rp, ablation=v) if v else O.OracleLayout(rp) as L:
                assert (L.layout.nwarps, L.layout.allocate_nz) == (R.nwarps, R.allocate_nz)
                for f, a in layout_arrays(L).items():
                    np.testing.assert_array_equal(a, R.arrays[f], err_msg=f"variant {v} {f}")
                if v & 2:
                    pv, pc = L.process(vals, cols)
                    rpv, rpc = R.process(vals, cols)
                    np.testing.assert_array_equal(pv, rpv)
                    y = L.run(pv, pc, x, fma=True)
                    yr = R.run_nocoalesced(rpv, rpc, x)
                    np.testing.assert_array_equal(y.view(np.int64), yr.view(np.int64))
            R.free()


def test_oracle_ablation_matches_golden(golden):
    checked = 0
    for name, rp, cols, vals, x, layouts in golden_cases(golden):
        for v in ABL:
            tag = f"{name}/abl{v}"
            if f"{tag}/info" not in golden:
                continue
            with O.OracleLayout(rp, ablation=v) as L:
                info = golden[f"{tag}/info"]
                assert (L.layout.nwarps, L.layout.allocate_nz) == tuple(int(i) for i in info)
                for f, a in layout_arrays(L).items():
                    np.testing.assert_array_equal(a, golden[f"{tag}/{f}"], err_msg=f"{tag} {f}")
                if f"{tag}/y" in golden:
                    pv, pc = L.process(vals, cols)
                    y = L.run(pv, pc, x, fma=True)
                    np.testing.assert_array_equal(y.view(np.int64), golden[f"{tag}/y"].view(np.int64))
                checked += 1
    assert checked >= 12


def test_ablation_layouts_with_empty_rows_drop_them():
    rng = np.random.default_rng(9)
    rp, cols, vals = random_csr(rng, 300, 30, p_empty=0.3)
    x = rng.uniform(-1, 1, 300)
    ref = O.csr_spmv(rp, cols, vals, x)
    for v in ABL:
        with O.OracleLayout(rp, ablation=v) as L:
            lay = L.layout
            nzr = int(np.count_nonzero(np.diff(rp)))
            assert lay.nznrows == nzr and lay.nwarps == (nzr + 31) // 32
            rm = lay.arrays["row_map"]
            assert np.all(np.diff(rp)[rm[nzr:]] == 0)  # empty rows last
            if v & 1:  # CSR order kept among the rows with entries
                assert np.all(np.diff(rm[:nzr]) > 0)
            pv, pc = L.process(vals, cols)
            y = L.run(pv, pc, x, fma=True)
            assert np.allclose(y, ref, rtol=1e-12, atol=1e-12)
