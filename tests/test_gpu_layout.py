"""Device-built WPK1/WPK2 layouts are bit-identical to the reference's host
scan (golden fixtures from the reference's own code) and to the oracle."""
import numpy as np
import pytest

from conftest import golden_cases, random_csr
from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu

FIELDS1 = ("row_map", "row_map_inv", "reorder_rows", "warp_offsets", "max_nz_rows")
FIELDS2 = FIELDS1 + ("threads_per_row", "row_offset_warp")


def wk():
    import warpkernel_gb300
    return warpkernel_gb300


def scan(kind, rp, nz, th=0, device=False):
    import torch
    rows = torch.from_numpy(rp).cuda() if device else rp
    k = wk().structure() if kind == 1 else wk().structure2()
    if kind == 1:
        k.scan(nz, len(rp) - 1, None, rows)
    else:
        k.scan(nz, len(rp) - 1, None, rows, None, th)
    return k


def assert_layout_equal(k, L, kind, tag=""):
    assert (k.nrows, k.nznrows, k.nz, k.allocate_nz, k.nwarps) == \
        (L.nrows, L.nznrows, L.nz, L.allocate_nz, L.nwarps), tag
    for f in (FIELDS1 if kind == 1 else FIELDS2):
        a, b = getattr(k, f), L.arrays[f] if hasattr(L, "arrays") else L[f]
        assert a.dtype == b.dtype and np.array_equal(a, b), (tag, f)
    if kind == 2:
        assert (k.min_nz, k.max_nz, k.nmax_per_thread) == (L.min_nz, L.max_nz, L.nmax_per_thread), tag


def test_layout_matches_reference_golden(golden):
    for name, rp, cols, vals, x, layouts in golden_cases(golden):
        for kind, th in layouts:
            tag = f"{name}/k{kind}_t{th}"
            k = scan(kind, rp, len(cols), th)
            info = golden[f"{tag}/info"]
            assert [k.nrows, k.nznrows, k.nz, k.allocate_nz, k.nwarps] == list(info[:5]), tag
            if kind == 2:
                assert [k.min_nz, k.max_nz, k.nmax_per_thread] == list(info[5:]), tag
            for f in (FIELDS1 if kind == 1 else FIELDS2):
                np.testing.assert_array_equal(getattr(k, f), golden[f"{tag}/{f}"], err_msg=f"{tag} {f}")
            if len(cols) == 0:
                continue
            eng = wk().engine(k, vals, cols)
            np.testing.assert_array_equal(eng.device_values, golden[f"{tag}/pvals"])
            np.testing.assert_array_equal(eng.device_colinds, golden[f"{tag}/pcols"])
            np.testing.assert_array_equal(k.reorder_columns_coalesced(cols), golden[f"{tag}/pcols_renum"])
            np.testing.assert_array_equal(k.reorder_x(x).cpu().numpy(), golden[f"{tag}/x_reordered"])


def test_layout_random_matrices_vs_oracle():
    rng = np.random.default_rng(3)
    for trial in range(40):
        n = int(rng.integers(1, 3000))
        rp, cols, vals = random_csr(rng, n, int(rng.choice([1, 5, 27, 81, 400])),
                                    float(rng.choice([0, 0.05, 0.5])))
        for kind, th in [(1, 0), (2, int(rng.integers(-1, 100))), (2, 0), (2, 1)]:
            k = scan(kind, rp, len(cols), th, device=bool(trial % 2))
            with O.OracleLayout(rp, kind=kind, threshold=th) as o:
                assert_layout_equal(k, o.layout, kind, (trial, kind, th))
                if len(cols):
                    eng = wk().engine(k, vals, cols)
                    pv, pc = o.process(vals, cols)
                    assert np.array_equal(eng.device_values, pv)
                    assert np.array_equal(eng.device_colinds, pc)
                    assert np.array_equal(k.reorder_columns(cols), o.reorder_columns(cols))


def test_radix_sort_multiple_passes():
    # row lengths above 255 and above 65535 force 2 and 3 digit passes
    rng = np.random.default_rng(9)
    for big in (700, 70000):
        n = big + 500
        lens = rng.integers(0, 40, n)
        lens[rng.integers(0, n, 5)] = rng.integers(256, big, 5)
        lens[3] = big
        rp = np.zeros(n + 1, np.int32)
        rp[1:] = np.cumsum(lens)
        for kind, th in ((1, 0), (2, 16)):
            k = scan(kind, rp, int(rp[-1]), th)
            with O.OracleLayout(rp, kind=kind, threshold=th) as o:
                assert_layout_equal(k, o.layout, kind, big)


def test_fe_matrices_vs_oracle():
    for dim, e, dof, ths in ((2, 128, 1, (1, 4, 9)), (3, 24, 3, (6, 27, 81))):
        rp, cols, vals = O.fe_matrix(dim, e, e, e if dim == 3 else 0, dof, value_mode=1, seed=1)
        for kind, th in [(1, 0)] + [(2, t) for t in ths]:
            k = scan(kind, rp, len(cols), th, device=True)
            with O.OracleLayout(rp, kind=kind, threshold=th) as o:
                assert_layout_equal(k, o.layout, kind, (dim, kind, th))


def test_empty_and_tiny():
    for rp in (np.zeros(1, np.int32), np.zeros(5, np.int32), np.array([0, 1], np.int32),
               np.array([0, 0, 1, 1], np.int32)):
        for kind, th in ((1, 0), (2, 0), (2, 1)):
            k = scan(kind, rp, int(rp[-1]), th)
            with O.OracleLayout(rp, kind=kind, threshold=th) as o:
                assert_layout_equal(k, o.layout, kind, (list(rp), kind, th))


def test_device_rowptr_validation():
    import torch
    for rp, nz in (([1, 2, 3], 3), ([0, 2, 1], 1), ([0, 1, 2], 3)):
        k = wk().structure()
        with pytest.raises(wk().WKError) as ei:
            k.scan(nz, len(rp) - 1, None, torch.tensor(rp, dtype=torch.int32, device="cuda"))
        assert ei.value.status == 1


def test_engine_rejects_out_of_range_columns():
    rp = np.array([0, 2, 3], np.int32)
    k = scan(1, rp, 3)
    with pytest.raises(wk().WKError, match="outside"):
        wk().engine(k, np.ones(3), np.array([0, 2, 1], np.int32))
    eng = wk().engine(k, np.ones(3), np.array([0, 1, 1], np.int32))
    bad = np.zeros(k.allocate_nz, np.int32)
    bad[5] = 7
    with pytest.raises(wk().WKError, match="outside"):
        eng.device_colinds = bad


def test_process_into_caller_buffers_matches_oracle():
    """wk_process (structure::reorder / process, reorder_values_coalesced)
    with host and device arrays, values and columns separately."""
    import torch

    import warpkernel_gb300 as wk
    from conftest import random_csr
    rng = np.random.default_rng(17)
    rp, cols, vals = random_csr(rng, 1500, 45, p_empty=0.1)
    for kind, th in ((1, 0), (2, 7)):
        k = wk.structure() if kind == 1 else wk.structure2()
        if kind == 1:
            k.scan(len(cols), len(rp) - 1, None, rp)
        else:
            k.scan(len(cols), len(rp) - 1, None, rp, None, th)
        with O.OracleLayout(rp, kind=kind, threshold=th) as L:
            ov, oc = L.process(vals, cols)
            pv, pc = k.process(vals, cols)
            np.testing.assert_array_equal(pv, ov)
            np.testing.assert_array_equal(pc, oc)
            dv, dc = k.process(torch.from_numpy(vals).cuda(), torch.from_numpy(cols).cuda())
            np.testing.assert_array_equal(dv.cpu().numpy(), ov)
            np.testing.assert_array_equal(dc.cpu().numpy(), oc)
            np.testing.assert_array_equal(k.reorder_values_coalesced(vals), ov)
            assert k.process(None, cols)[0] is None
            f32 = k.process(vals.astype(np.float32), None, dtype="f32")[0]
            np.testing.assert_array_equal(f32, ov.astype(np.float32))
