"""Failure paths made on the host: injected allocation failures, layouts
that overflow the reference's int32 offsets, and wrong vector sizes.  No GPU
fault is provoked: every failure is a status code returned before or instead
of a kernel touching memory it should not."""
import numpy as np
import pytest

from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu


def test_injected_allocation_failures_leave_the_library_usable():
    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300._lib import load
    rp, cols, vals = O.fe_matrix(2, 40, 40, 0, 1, value_mode=0)
    n = len(rp) - 1
    x = torch.from_numpy(O.uniform_vec(1, 0, n)).cuda()
    ref = O.csr_spmv(rp, cols, vals, x.cpu().numpy())
    L = load()
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    for nth in range(1, 40):  # fail the nth device allocation of scan + engine build
        L.wk_debug_fail_alloc(nth)
        try:
            k = wk.structure2().scan(len(cols), n, None, rp, None, 4)
            eng = wk.engine(k, vals, cols)
        except wk.WKError as e:
            assert e.status == 3 and "injected" in str(e)
            failures += 1
            continue
        finally:
            L.wk_debug_fail_alloc(0)
        y = torch.zeros(n, dtype=torch.float64, device="cuda")
        eng.run(0, 128, x, y)
        assert np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref) < 1e-12
        del eng, k
    assert failures >= 10  # every allocation site of the build was exercised
    import gc
    gc.collect()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0 - (64 << 20)  # nothing large leaked


def test_allocate_nz_beyond_int32_is_rejected():
    import warpkernel_gb300 as wk
    # one warp: one row of 2^26 entries and 31 short rows -> 32 * 2^26 padded slots
    lens = np.ones(40, np.int64)
    lens[5] = 1 << 26
    rp = np.zeros(41, np.int64)
    rp[1:] = np.cumsum(lens)
    rp = rp.astype(np.int32)
    for kind in (1, 2):
        k = wk.structure() if kind == 1 else wk.structure2()
        with pytest.raises(wk.WKError) as ei:
            if kind == 1:
                k.scan(int(rp[-1]), 40, None, rp)
            else:
                k.scan(int(rp[-1]), 40, None, rp, None, 1 << 30)
        assert ei.value.status == 4 and "int32" in str(ei.value)


def test_vector_checks_in_the_binding():
    import torch

    import warpkernel_gb300 as wk
    rp, cols, vals = O.fe_matrix(2, 8, 8, 0, 1, value_mode=0)
    n = len(rp) - 1
    k = wk.structure().scan(len(cols), n, None, rp)
    eng = wk.engine(k, vals, cols)
    good = torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        eng.run(0, 128, torch.zeros(n - 1, dtype=torch.float64, device="cuda"), good)
    with pytest.raises(ValueError):
        eng.run(0, 128, good, torch.zeros(n, dtype=torch.float32, device="cuda"))
    with pytest.raises(ValueError):
        eng.run(0, 128, torch.zeros(n, dtype=torch.float64), good)
    eng.run(0, 128, good, good.clone())
