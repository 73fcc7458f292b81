"""Host-side pieces of the batched path (no GPU): the seeded 512-patch
workload description, the library's FE size formula against the oracle's
CPU generator, and the algorithmic byte count the bench reports."""
import numpy as np

from oracle import wk_oracle as O


def test_fe_matrix_set_is_seeded_and_in_range():
    from warpkernel_gb300 import batched
    a = batched.fe_matrix_set(512, seed=3)
    b = batched.fe_matrix_set(512, seed=3)
    assert a == b and len(a) == 512
    assert a != batched.fe_matrix_set(512, seed=4)
    for s in a:
        assert s["dim"] in (2, 3) and s["dof"] in (1, 3) and 1 <= s["nrhs"] <= 16 and s["ex"] >= 1
        # log-uniform targets in [1k, 200k]; rounding the mesh edge moves the
        # row count by less than a factor of two either way
        assert 400 <= s["nrows"] <= 420_000, s
    dims = {s["dim"] for s in a}
    dofs = {s["dof"] for s in a}
    ks = {s["nrhs"] for s in a}
    assert dims == {2, 3} and dofs == {1, 3} and ks == set(range(1, 17))


def test_fe_size_matches_the_oracle_generator():
    from warpkernel_gb300 import fe
    for dim, ex, dof in ((2, 1, 1), (2, 7, 3), (3, 1, 1), (3, 4, 3), (3, 6, 1)):
        n, z = fe.fe_size(dim, ex, ex, ex if dim == 3 else 0, dof)
        rp, cols, vals = O.fe_matrix(dim, ex, ex, ex if dim == 3 else 0, dof, value_mode=1, seed=1)
        assert (n, z) == (len(rp) - 1, len(cols)), (dim, ex, dof)


def test_algorithmic_bytes():
    from warpkernel_gb300 import batched
    specs = [dict(nnz=100, nrows=10, nrhs=3), dict(nnz=7, nrows=2, nrhs=16)]
    assert batched.algorithmic_bytes(specs) == (8 * 100 + 10 * 3 * 8) + (8 * 7 + 2 * 16 * 8)
    assert batched.algorithmic_bytes(specs, value_bytes=8, vec_bytes=8) == (12 * 100 + 10 * 3 * 16) + (12 * 7 + 2 * 16 * 16)
