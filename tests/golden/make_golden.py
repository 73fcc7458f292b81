"""Regenerates tests/golden/wpk_golden.npz from the reference itself.

The reference's host scan/process/reorder code (including
reorder_columns_rowsort) and its WPK1 SpMV and assembly kernels
(warpkernel.hpp), and the ablation scans and warpKernel_nocoalesced of
optimization.cu, are compiled for the CPU by `make -C oracle ref` (needs the
reference sources) and run here on a fixed set of small matrices.  The
fixture stores inputs and the reference's outputs, so tests on machines
without the reference sources can still check the oracle and the CUDA path
against the reference's own results.

    python tests/golden/make_golden.py
"""
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import wk_oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "wpk_golden.npz")


def lap2d(m):
    rows, cols = [0], []
    for i in range(m):
        for j in range(m):
            for di, dj in ((-1, 0), (0, -1), (0, 0), (0, 1), (1, 0)):
                a, b = i + di, j + dj
                if 0 <= a < m and 0 <= b < m:
                    cols.append(a * m + b)
            rows.append(len(cols))
    rp = np.array(rows, np.int32)
    c = np.array(cols, np.int32)
    v = np.where(c == np.repeat(np.arange(m * m), np.diff(rp)), 4.0, -1.0)
    return rp, c, v


def csr_from_lengths(lens, ncols, rng):
    rp = np.zeros(len(lens) + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    cols = rng.integers(0, ncols, rp[-1]).astype(np.int32)
    vals = rng.standard_normal(rp[-1])
    return rp, cols, vals


def cases():
    rng = np.random.default_rng(2024)
    out = []
    rp, c, v = lap2d(6)
    out.append(("lap2d_6", rp, c, v, [(1, 0), (2, 2)]))
    rp, c, v = O.fe_matrix(2, 8, 8, 0, 1, value_mode=0, seed=0)
    out.append(("q1_8x8", rp, c, v, [(1, 0), (2, 1), (2, 4), (2, 9)]))
    rp, c, v = O.fe_matrix(3, 3, 3, 3, 3, value_mode=1, seed=1)
    out.append(("hex_3", rp, c, v, [(1, 0), (2, 6), (2, 20), (2, 81)]))
    n = 300
    lens = rng.integers(0, 41, n)
    lens[rng.random(n) < 0.2] = 0
    rp, c, v = csr_from_lengths(lens, n, rng)
    out.append(("ragged_300", rp, c, v, [(1, 0), (2, 0), (2, 3), (2, 17), (2, -1)]))
    n = 200
    lens = rng.integers(1, 6, n)
    lens[rng.integers(0, n, 7)] = rng.integers(60, 200, 7)
    rp, c, v = csr_from_lengths(lens, n, rng)
    out.append(("longrows_200", rp, c, v, [(1, 0), (2, 2), (2, 50)]))
    rp = np.zeros(11, np.int32)
    out.append(("empty_10", rp, np.zeros(0, np.int32), np.zeros(0), [(1, 0), (2, 1)]))
    rp, c, v = csr_from_lengths(np.full(35, 20), 35, rng)  # last warp 3 rows: partial split
    out.append(("partial_35", rp, c, v, [(1, 0), (2, 4)]))
    rp, c, v = csr_from_lengths(np.full(37, 20), 37, rng)  # last warp 5 rows: full split
    out.append(("fullsplit_37", rp, c, v, [(1, 0), (2, 4)]))
    return out


def main():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    R = {"mul_add": O.RefLib("mul_add"), "fma": O.RefLib("fma")}
    rng = np.random.default_rng(7)
    data = {}
    names = []
    for name, rp, c, v, layouts in cases():
        names.append(name)
        n = len(rp) - 1
        x = rng.uniform(-1, 1, n)
        data[f"{name}/rowptr"], data[f"{name}/cols"], data[f"{name}/vals"], data[f"{name}/x"] = rp, c, v, x
        data[f"{name}/layouts"] = np.array(layouts, np.int64).reshape(-1, 2)
        for kind, th in layouts:
            tag = f"{name}/k{kind}_t{th}"
            s = R["mul_add"].scan(rp, kind, th)
            data[f"{tag}/info"] = np.array([s.nrows, s.nznrows, s.nz, s.allocate_nz, s.nwarps,
                                            s.min_nz, s.max_nz, s.nmax_per_thread], np.int64)
            for f in O.FIELDS:
                data[f"{tag}/{f}"] = s.arrays[f]
            pv, pc = s.process(v, c)
            data[f"{tag}/pvals"], data[f"{tag}/pcols"] = pv, pc
            pcr = s.reorder_columns_coalesced(c)
            xr = s.reorder_x(x)
            data[f"{tag}/pcols_renum"], data[f"{tag}/x_reordered"] = pcr, xr
            rs_cols, rs_src = s.reorder_columns_rowsort(rp, c)
            data[f"{tag}/cols_rowsort"], data[f"{tag}/reorder_A_rows"] = rs_cols, rs_src
            if kind == 1 and s.nwarps > 0:
                data[f"{tag}/y_assembly"] = s.assembly_wpk1(pv)
                for mode, RL in R.items():
                    s2 = RL.scan(rp, 1, 0)
                    data[f"{tag}/y_run_{mode}"] = s2.run_wpk1(pv, pc, x, mapped=True)
                    data[f"{tag}/y_runx_{mode}"] = s2.run_wpk1(pv, pcr, xr, mapped=False)
                    s2.free()
            s.free()
        # ablation layouts of optimization.cu, on matrices without empty rows
        if n and np.all(np.diff(rp) > 0):
            for va in (1, 2, 3):
                tag = f"{name}/abl{va}"
                A = O.RefAblation(rp, va)
                data[f"{tag}/info"] = np.array([A.nwarps, A.allocate_nz], np.int64)
                for f in O.FIELDS[:5]:
                    data[f"{tag}/{f}"] = A.arrays[f]
                if va & 2:
                    pv, pc = A.process(v, c)
                    data[f"{tag}/y"] = A.run_nocoalesced(pv, pc, x)
                A.free()
    data["names"] = np.array(names)
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes, {len(names)} matrices)")


if __name__ == "__main__":
    main()
