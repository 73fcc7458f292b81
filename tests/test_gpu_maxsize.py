"""The largest layouts the reference's int32 warp_offsets allow: allocate_nz
just below 2^31 slots.  Checked through size-independent properties (integer
x, exact FP32 sums) against a torch gather-sum of the same CSR on the GPU; the
oracle would take minutes at this size.  Needs ~50 GB of device memory."""
import pytest

pytestmark = pytest.mark.gpu

ROW_LEN = 64
NROWS = ((1 << 31) - (1 << 24)) // ROW_LEN  # allocate_nz = 2^31 - 2^24


def torch():
    import torch as t
    return t


@pytest.mark.parametrize("kind,th", [(1, 0), (2, 16)])
def test_allocate_nz_just_below_int32(kind, th):
    t = torch()
    if t.cuda.mem_get_info()[0] < (80 << 30):
        pytest.skip("needs ~50 GB of free device memory")
    import warpkernel_gb300 as wk
    n, L = NROWS, ROW_LEN
    nnz = n * L
    rp = t.arange(0, nnz + 1, L, dtype=t.int64, device="cuda").to(t.int32)
    # column i of row r: (r + 97 i) mod n (no int32 overflow: r + 97 i < 2^31)
    r = t.arange(n, dtype=t.int32, device="cuda").unsqueeze(1)
    i = t.arange(L, dtype=t.int32, device="cuda").unsqueeze(0)
    cols2d = (r + 97 * i) % n
    del r, i
    cols = cols2d.reshape(-1)
    vals = t.ones(nnz, dtype=t.float32, device="cuda")
    k = wk.structure() if kind == 1 else wk.structure2()
    if kind == 1:
        k.scan(nnz, n, None, rp)
    else:
        k.scan(nnz, n, None, rp, None, th)
    assert k.allocate_nz == nnz and nnz < (1 << 31)
    eng = wk.engine(k, vals, cols, dtype="f32")
    del vals
    x = (t.arange(n, dtype=t.int64, device="cuda") % 7).to(t.float32)
    ref = t.zeros(n, dtype=t.float32, device="cuda")
    for c0 in range(0, L, 8):  # gather-sum in column blocks (exact small integers)
        ref += x[cols2d[:, c0:c0 + 8].long()].sum(dim=1)
    for order in (0, 1):
        y = t.full((n,), -1.0, dtype=t.float32, device="cuda")
        eng.run(0, 0, x, y, order=order, timed=False)
        t.cuda.synchronize()
        assert t.equal(y, ref), f"order {order}"
    assert float(ref.max()) <= 6 * L and float(ref.min()) >= 0
    del eng, k, cols, cols2d, rp, x, y, ref
    t.cuda.empty_cache()
