"""SpMV on host vectors: wk_run_host (one vector, synchronous) and
wk_run_host_stream (a sequence, copies overlapped with the SpMVs) give the
same bits as the device-vector run / run_x."""
import numpy as np
import pytest

from conftest import random_csr
from oracle import wk_oracle as O

pytestmark = pytest.mark.gpu


def wk():
    import warpkernel_gb300
    return warpkernel_gb300


def torch():
    import torch as t
    return t


def engine(kind, rp, cols, vals, th=0, dtype="f64"):
    k = wk().structure() if kind == 1 else wk().structure2()
    if kind == 1:
        k.scan(len(cols), len(rp) - 1, None, rp)
    else:
        k.scan(len(cols), len(rp) - 1, None, rp, None, th)
    t = torch()
    v = t.from_numpy(vals).to({"f64": t.float64, "f32": t.float32, "bf16": t.bfloat16}[dtype])
    return k, wk().engine(k, v, cols, dtype=dtype)


def device_result(eng, x, mapped, order):
    t = torch()
    n = eng.kernel.nrows
    ydt = t.float64 if eng.dtype == 0 else t.float32
    dy = t.zeros(n, dtype=ydt, device="cuda")
    (eng.run if mapped else eng.run_x)(0, 128, x.cuda(), dy, order=order)
    return dy.cpu()


@pytest.mark.parametrize("dtype", ["f64", "f32", "bf16"])
@pytest.mark.parametrize("kind,th", [(1, 0), (2, 6)])
def test_run_host_and_stream_match_device_run(dtype, kind, th):
    t = torch()
    rng = np.random.default_rng(kind * 7 + th)
    rp, cols, vals = random_csr(rng, 3000, 50, p_empty=0.1)  # empty rows: y must be 0 there
    n = len(rp) - 1
    k, eng = engine(kind, rp, cols, vals, th, dtype)
    xdt = {"f64": t.float64, "f32": t.float32, "bf16": t.bfloat16}[dtype]
    ydt = t.float64 if dtype == "f64" else t.float32
    for mapped in (True, False):
        for order in (wk().WK_ORDER_FAST, wk().WK_ORDER_EXACT):
            xs = [t.from_numpy(O.uniform_vec(11, i, n)).to(xdt).pin_memory() for i in range(5)]
            refs = [device_result(eng, x, mapped, order) for x in xs]
            # one vector at a time (y pre-filled with garbage: empty rows must come back 0)
            y = t.full((n,), 3.0, dtype=ydt).pin_memory()
            eng.run_host(xs[0], y, mapped=mapped, order=order)
            assert t.equal(y, refs[0])
            # sequences of 1, 2 and 5 vectors, pinned and pageable
            for count in (1, 2, 5):
                for pin in (True, False):
                    ys = [t.full((n,), 3.0, dtype=ydt) for _ in range(count)]
                    xx = xs[:count] if pin else [x.clone() for x in xs[:count]]
                    if pin:
                        ys = [y.pin_memory() for y in ys]
                    sec = eng.run_host_stream(xx, ys, mapped=mapped, order=order)
                    assert sec > 0
                    for i in range(count):
                        assert t.equal(ys[i], refs[i]), (mapped, order, count, pin, i)


def test_run_host_stream_empty_and_bad_arguments():
    t = torch()
    rp, cols, vals = O.fe_matrix(2, 10, 10, 0, 1, value_mode=0)
    n = len(rp) - 1
    k, eng = engine(1, rp, cols, vals)
    assert eng.run_host_stream([], []) >= 0
    with pytest.raises(ValueError):
        eng.run_host_stream([t.zeros(n, dtype=t.float64)], [])
    L = wk().load()
    import ctypes as C
    arr = (C.c_void_p * 1)(None)
    assert L.wk_run_host_stream(eng.handle, 1, 0, 1, arr, arr, None, None) == 1  # NULL vector
