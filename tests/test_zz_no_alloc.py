"""wk_residual_static: the residual entry point that allocates no device
memory, for callers that must not call cudaMalloc while they run (a host
application that owns the GPU's whole memory budget, or a latency-critical
loop that cannot afford cudaMalloc's implicit synchronisation).

Called through the C ABI and compared with wk_residual, the allocating entry
point, on two calls in a row.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # the tolerance of the other fp64 parity tests


def test_residual_static_matches_allocating_entry_point():
    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300._lib import check, load

    L = load()
    rp, cols, vals = O.fe_matrix(3, 12, 12, 12, 3, value_mode=1, seed=6)
    n = len(rp) - 1
    k = wk.structure2().scan(len(cols), n, None, rp, None, 27)
    eng = wk.engine(k, vals, cols)
    rng = np.random.default_rng(21)
    b = torch.from_numpy(rng.uniform(-1, 1, n)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # two calls in a row, different x each time
        x = torch.from_numpy(rng.uniform(-1, 1, n)).cuda()
        r_ref = torch.empty(n, dtype=torch.float64, device="cuda")
        n_ref = torch.zeros(1, dtype=torch.float64, device="cuda")
        check(L.wk_residual(eng.handle, x.data_ptr(), b.data_ptr(), r_ref.data_ptr(), n_ref.data_ptr(), stream))
        r = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        nrm = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        check(L.wk_residual_static(eng.handle, x.data_ptr(), b.data_ptr(), r.data_ptr(), nrm.data_ptr(), stream))
        torch.cuda.synchronize()
        rr, rs = r_ref.cpu().numpy(), r.cpu().numpy()
        assert np.linalg.norm(rs - rr) / np.linalg.norm(rr) <= REL_TOL, call
        assert abs(nrm.item() - n_ref.item()) <= REL_TOL * n_ref.item(), call
        assert np.array_equal(rs, rr) and nrm.item() == n_ref.item(), call  # same kernel, same order
    # after the set-up call, a call allocates nothing: with the library's next
    # device allocation armed to fail it still succeeds, and the device's free
    # memory is unchanged across it
    x = torch.from_numpy(rng.uniform(-1, 1, n)).cuda()
    r = torch.empty(n, dtype=torch.float64, device="cuda")
    nrm = torch.empty(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    L.wk_debug_fail_alloc(1)
    try:
        st = L.wk_residual_static(eng.handle, x.data_ptr(), b.data_ptr(), r.data_ptr(), nrm.data_ptr(), stream)
    finally:
        L.wk_debug_fail_alloc(0)
    assert st == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_residual_static_rejects_layouts_beyond_its_scratch():
    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300._lib import load

    # 300,000 rows of 64 entries split 32 ways: 300,000 layout warps > 262,144
    n = 300_000
    rp = np.arange(n + 1, dtype=np.int64) * 64
    rp = rp.astype(np.int32)
    cols = (np.arange(n * 64, dtype=np.int64) % n).astype(np.int32)
    k = wk.structure2().scan(len(cols), n, None, rp, None, 2)
    assert k.nwarps > 262_144
    eng = wk.engine(k, np.ones(len(cols)), cols)
    t = torch.zeros(n, dtype=torch.float64, device="cuda")
    L = load()
    st = L.wk_residual_static(eng.handle, t.data_ptr(), t.data_ptr(), t.data_ptr(), None, None)
    assert st == 1  # WK_ERR_INVALID
    from warpkernel_gb300._lib import last_error
    assert "static scratch" in last_error()
