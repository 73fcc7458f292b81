"""The CPU oracle against the reference: known answers, committed golden
fixtures produced by the reference's own code, and (where the reference
sources are present) a live byte-for-byte cross-check on random matrices."""
import numpy as np
import pytest

from conftest import golden_cases, random_csr
from oracle import wk_oracle as O


def lap2d(m):
    rows, cols = [0], []
    for i in range(m):
        for j in range(m):
            for di, dj in ((-1, 0), (0, -1), (0, 0), (0, 1), (1, 0)):
                a, b = i + di, j + dj
                if 0 <= a < m and 0 <= b < m:
                    cols.append(a * m + b)
            rows.append(len(cols))
    return np.array(rows, np.int32), np.array(cols, np.int32)


def test_known_answers_6x6_laplacian():
    # 5-point Laplacian on a 6x6 grid: 4 corners (3 nnz), 16 edges (4), 16 interior (5).
    rp, _ = lap2d(6)
    with O.OracleLayout(rp, kind=1) as o:
        L = o.layout
        assert (L.nwarps, L.allocate_nz) == (2, 256)
        assert list(L.row_map[:4]) == [7, 8, 9, 10]  # first interior rows, ascending
        assert list(L.max_nz_rows) == [5, 3]  # 16 interior + 16 edge rows, then 4 corners
    with O.OracleLayout(rp, kind=2, threshold=2) as o:
        L = o.layout
        assert (L.nwarps, L.allocate_nz) == (5, 320)
        assert L.threads_per_row[0] == 4 and L.max_nz_rows[0] == 2
        assert (L.min_nz, L.max_nz) == (3, 5)
        assert L.row_offset_warp[-1] == 36


def test_oracle_matches_golden(golden):
    for name, rp, cols, vals, x, layouts in golden_cases(golden):
        for kind, th in layouts:
            tag = f"{name}/k{kind}_t{th}"
            with O.OracleLayout(rp, kind=kind, threshold=th) as o:
                L = o.layout
                info = golden[f"{tag}/info"]
                got = [L.nrows, L.nznrows, L.nz, L.allocate_nz, L.nwarps]
                if kind == 2:
                    got += [L.min_nz, L.max_nz, L.nmax_per_thread]
                assert got == list(info[:len(got)]), tag
                for f in O.FIELDS:
                    if kind == 1 and f in ("threads_per_row", "row_offset_warp"):
                        continue
                    np.testing.assert_array_equal(L.arrays[f], golden[f"{tag}/{f}"], err_msg=f"{tag} {f}")
                pv, pc = o.process(vals, cols)
                np.testing.assert_array_equal(pv, golden[f"{tag}/pvals"])
                np.testing.assert_array_equal(pc, golden[f"{tag}/pcols"])
                pcr = o.reorder_columns_coalesced(cols)
                xr = o.reorder_x(x)
                np.testing.assert_array_equal(pcr, golden[f"{tag}/pcols_renum"])
                np.testing.assert_array_equal(xr, golden[f"{tag}/x_reordered"])
                if f"{tag}/y_run_fma" in golden:
                    for mode, fma in (("fma", True), ("mul_add", False)):
                        y = o.run(pv, pc, x, fma=fma)
                        np.testing.assert_array_equal(y.view(np.int64), golden[f"{tag}/y_run_{mode}"].view(np.int64))
                        y = o.run_x(pv, pcr, xr, fma=fma)
                        np.testing.assert_array_equal(y.view(np.int64), golden[f"{tag}/y_runx_{mode}"].view(np.int64))


@pytest.mark.skipif(not O.RefLib.available(), reason="reference sources not built here")
def test_oracle_matches_reference_scan_random():
    R = O.RefLib("mul_add")
    RF = O.RefLib("fma")
    rng = np.random.default_rng(11)
    for trial in range(120):
        n = int(rng.integers(1, 900))
        rp, cols, vals = random_csr(rng, n, int(rng.choice([1, 4, 9, 33, 81, 300])),
                                    float(rng.choice([0, 0.1, 0.6])))
        x = rng.standard_normal(n)
        ths = [int(t) for t in rng.integers(-1, 90, 3)] + [0]
        for kind, th in [(1, 0)] + [(2, t) for t in ths]:
            with O.OracleLayout(rp, kind=kind, threshold=th) as o:
                r = R.scan(rp, kind, th)
                L = o.layout
                for f in O.FIELDS:
                    if kind == 1 and f in ("threads_per_row", "row_offset_warp"):
                        continue
                    assert np.array_equal(L.arrays[f], r.arrays[f]), (trial, kind, th, f)
                assert (L.nznrows, L.allocate_nz, L.nwarps) == (r.nznrows, r.allocate_nz, r.nwarps)
                if kind == 2:
                    assert (L.min_nz, L.max_nz) == (r.min_nz, r.max_nz)
                pv, pc = o.process(vals, cols)
                rv, rc = r.process(vals, cols)
                assert np.array_equal(pv, rv) and np.array_equal(pc, rc)
                if kind == 1 and L.nwarps:
                    for RL, fma in ((R, False), (RF, True)):
                        r2 = RL.scan(rp, 1, 0)
                        y1 = o.run(pv, pc, x, fma=fma)
                        y2 = r2.run_wpk1(pv, pc, x, mapped=True, wpb=int(rng.integers(1, 17)))
                        assert np.array_equal(y1.view(np.int64), y2.view(np.int64))
                        r2.free()
                r.free()


def test_wpk2_tree_order_is_pairwise():
    """Leader sums of a split row follow ((s0+s1)+(s2+s3)); check against a
    direct restatement on values where association matters."""
    rp = np.array([0, 8, 9], np.int32)  # row 0: 8 entries, row 1: 1
    cols = np.zeros(9, np.int32)
    vals = np.array([1e16, 1.0, -1e16, 1.0, 3.0, 1e-3, 5.0, 7.0, 1.0])
    x = np.array([1.0, 1.0])
    with O.OracleLayout(rp, kind=2, threshold=1) as o:
        L = o.layout
        assert L.threads_per_row[0] > 1
        pv, pc = o.process(vals, cols)
        y = o.run(pv, pc, x, fma=True)
        T, A = int(L.threads_per_row[0]), int(L.max_nz_rows[0])
        lanes = [0.0] * T
        for t in range(T):  # x = 1: products are exact, so fma(v, 1, s) == s + v
            s = float(pv[L.warp_offsets[0] + t])
            for i in range(1, A):
                s = s + float(pv[L.warp_offsets[0] + t + 32 * i])
            lanes[t] = s
        k = 1
        while k < T:
            lanes = [lanes[i] + lanes[i + k] if i % (2 * k) == 0 and i + k < T else lanes[i] for i in range(T)]
            k *= 2
        assert y[L.row_map[0]] == lanes[0]


def test_csr_checks_reject_malformed():
    for rp, nz in (([1, 2, 3], 3), ([0, 2, 1], 1), ([0, 1, 2], 3)):
        with pytest.raises(ValueError):
            O.OracleLayout(np.array(rp, np.int32), nz=nz)


def test_fe_generator_shapes_and_symmetry():
    n, z = O.fe_size(2, 128, 128, 0, 1)
    assert (n, z) == (16641, 148225)
    n, z = O.fe_size(3, 128, 128, 128, 3)
    assert (n, z) == (6440067, 513599625)
    assert O.fe_size(3, 96, 96, 96, 3) == (2738019, 217238121)
    assert O.fe_size(3, 64, 64, 64, 3) == (823875, 64701513)
    for dim, ex, dof, mode in ((2, 6, 1, 0), (3, 3, 3, 1), (2, 5, 2, 1)):
        rp, cols, vals = O.fe_matrix(dim, ex, ex, ex if dim == 3 else 0, dof, value_mode=mode, seed=3)
        n = len(rp) - 1
        A = np.zeros((n, n))
        for r in range(n):
            A[r, cols[rp[r]:rp[r + 1]]] = vals[rp[r]:rp[r + 1]]
            assert np.all(np.diff(cols[rp[r]:rp[r + 1]]) > 0)
        np.testing.assert_array_equal(A, A.T)
        assert np.linalg.eigvalsh(A).min() > 0  # SPD
    # stencil mode: diagonal = 1.01 x absolute off-diagonal row sum
    rp, cols, vals = O.fe_matrix(2, 4, 4, 0, 1, value_mode=0, seed=0)
    for r in range(len(rp) - 1):
        seg = slice(rp[r], rp[r + 1])
        off = vals[seg][cols[seg] != r]
        assert np.all((off > -1) & (off < 0))
        s = 0.0
        for v in off:  # sequential, ascending column, as the generator sums
            s = s + abs(float(v))
        assert vals[seg][cols[seg] == r][0] == 1.01 * s


def test_csr_baselines_agree():
    rng = np.random.default_rng(5)
    rp, cols, vals = random_csr(rng, 500, 30, 0.1)
    x = rng.standard_normal(500)
    y = O.csr_spmv(rp, cols, vals, x)
    A = np.zeros((500, 500))
    for r in range(500):
        np.add.at(A[r], cols[rp[r]:rp[r + 1]], vals[rp[r]:rp[r + 1]])
    np.testing.assert_allclose(y, A @ x, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(O.csr_spmv_t(rp, cols, vals, x, 500), A.T @ x, rtol=1e-12, atol=1e-12)


# ---- reduced-precision storage: the oracle's FP32 restatement --------------

def _round_to(q, sig, emin):
    """Fraction q rounded to `sig` significant bits, nearest-even, with the
    smallest quantum 2^emin (the subnormal step); inf at 2^128 and above."""
    from fractions import Fraction as F
    if q == 0:
        return 0.0
    a = abs(q)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    while F(2) ** e > a:
        e -= 1
    while F(2) ** (e + 1) <= a:
        e += 1
    qe = max(e - (sig - 1), emin)
    m = a / F(2) ** qe
    fl = m.numerator // m.denominator
    rem = m - fl
    if rem > F(1, 2) or (rem == F(1, 2) and fl % 2 == 1):
        fl += 1
    r = F(fl) * F(2) ** qe
    v = float("inf") if r >= F(2) ** 128 else float(r)
    return v if q > 0 else -v


def f32(q):
    return _round_to(q, 24, -149)


def test_bf16_rounding_is_one_step_nearest_even():
    """wko_round_bf16 against exact rational rounding to 8 significant bits
    (values whose rounding through FP32 would differ included)."""
    from fractions import Fraction as F
    rng = np.random.default_rng(8)
    a = rng.standard_normal(3000) * 10.0 ** rng.integers(-44, 38, 3000)
    # ties and near-ties of the bf16 grid, reached only by exact rounding
    a = np.concatenate([a, [1 + 2.0 ** -8, 1 + 2.0 ** -8 + 2.0 ** -40, 1 + 3 * 2.0 ** -8, 2.0 ** -134,
                            2.0 ** -134 * (1 + 2.0 ** -30), 3.3e38, -0.0]])
    got = O.bf16_to_f32(O.round_bf16(a)).astype(np.float64)
    for v, g in zip(a, got):
        want = _round_to(F(float(v)), 8, -133)
        assert g == want or (want == 0 and g == 0), (v, g, want)
    assert np.array_equal(O.round_f32(a), a.astype(np.float32))


def _lp_reference(o, pv, pc, x):
    """Per-lane first product then fused multiply-adds, then the WPK2 pairwise
    tree, every operation rounded to FP32 exactly (Fractions)."""
    from fractions import Fraction as F
    L = o.layout
    y = np.zeros(L.nrows, np.float32)
    for w in range(L.nwarps):
        T = int(L.threads_per_row[w]) if L.kind == 2 else 1
        first = int(L.row_offset_warp[w]) if L.kind == 2 else 32 * w
        s = [0.0] * 32
        for lane in range(32):
            if first + lane // T >= L.nznrows:
                continue
            off = int(L.warp_offsets[w]) + lane
            acc = f32(F(float(pv[off])) * F(float(x[pc[off]])))
            for i in range(1, int(L.max_nz_rows[w])):
                k = off + 32 * i
                acc = f32(F(float(pv[k])) * F(float(x[pc[k]])) + F(acc))
            s[lane] = acc
        for lead in range(0, 32, T):
            r = first + lead // T
            if r >= L.nznrows:
                continue
            t = s[lead:lead + T]
            i = 1
            while i < T:
                for k in range(0, T - i, 2 * i):
                    t[k] = f32(F(t[k]) + F(t[k + i]))
                i *= 2
            y[L.row_map[r]] = t[0]
    return y


def test_fp32_documented_order_against_exact_rounding():
    """wko_run_lp (FP32 and BF16 storage) against the same order evaluated
    with exact rational arithmetic and one FP32 rounding per operation, on a
    ragged matrix with empty rows, WPK1 and WPK2 (split rows)."""
    rng = np.random.default_rng(9)
    rp, cols, vals = random_csr(rng, 150, 70, p_empty=0.2)
    x = rng.uniform(-1, 1, len(rp) - 1)
    for kind, th in ((1, 0), (2, 3), (2, 40)):
        with O.OracleLayout(rp, kind=kind, threshold=th) as o:
            _, pc = o.process(vals, cols)
            for sv, sx in ((O.round_f32(vals), O.round_f32(x)), (O.round_bf16(vals), O.round_bf16(x))):
                pv = o.place(sv)
                y = o.run_lp(pv, pc, sx)
                fv = pv if pv.dtype == np.float32 else O.bf16_to_f32(pv)
                fx = sx if sx.dtype == np.float32 else O.bf16_to_f32(sx)
                ref = _lp_reference(o, fv, pc, fx)
                assert np.array_equal(y.view(np.uint32), ref.view(np.uint32)), (kind, th, pv.dtype)
                y1 = o.run_lp(pv, pc, sx, nthreads=1)
                assert np.array_equal(y1.view(np.uint32), y.view(np.uint32))
