"""The C-ABI library without a GPU: it loads, exports every symbol the public
header declares, and rejects malformed input on the host."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "wk_capi.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wk_[a-z0-9_]+)\s*\(", text)))


def test_library_loads_and_exports_header_symbols():
    import warpkernel_gb300._lib as L
    lib = L.load()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    # and the ctypes binding covers all of them
    assert set(syms) <= set(L.SIGNATURES), set(syms) - set(L.SIGNATURES)
    assert b"sm_103a" in lib.wk_version()


def test_every_header_declares_only_exported_symbols():
    import warpkernel_gb300._lib as L
    lib = L.load()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", h)).read(), flags=re.S)
        for s in set(re.findall(r"\b(wk_[a-z0-9_]+)\s*\(", text)):
            assert hasattr(lib, s), (h, s)


def test_host_csr_validation_without_gpu():
    import warpkernel_gb300 as wk
    cases = [(np.array([1, 2, 3], np.int32), 3, r"rowptr\[0\]"),
             (np.array([0, 2, 1], np.int32), 1, "monotone"),
             (np.array([0, 1, 2], np.int32), 3, "does not equal nz")]
    for rp, nz, msg in cases:
        s = wk.structure()
        with pytest.raises(wk.WKError, match=msg) as ei:
            s.scan(nz, len(rp) - 1, rows=rp)
        assert ei.value.status == 1  # WK_ERR_INVALID


def test_null_arguments_are_rejected():
    import warpkernel_gb300._lib as L
    lib = L.load()
    h = C.c_void_p()
    assert lib.wk_scan1(None, 3, 0, None, C.byref(h)) == 1
    assert "NULL" in L.last_error()
    assert lib.wk_run(None, 0, 0, 1, 0, None, None, None, None) == 1
    assert lib.wk_engine_destroy(None) == 0
    assert lib.wk_layout_destroy(None) == 0
    n, z = C.c_int64(), C.c_int64()
    assert lib.wk_fe_size(4, 1, 1, 1, 1, C.byref(n), C.byref(z)) == 1
    assert lib.wk_fe_size(3, 128, 128, 128, 3, C.byref(n), C.byref(z)) == 0
    assert (n.value, z.value) == (6440067, 513599625)


def test_python_mirror_names_match_reference_surface():
    import warpkernel_gb300 as wk
    for name in ("scan", "reorder_columns_coalesced", "reorder_columns", "reorder_x", "row_map",
                 "row_map_inv", "reorder_rows", "warp_offsets", "max_nz_rows", "nrows", "nznrows", "nz",
                 "allocate_nz", "nwarps"):
        assert hasattr(wk.structure, name), name
    for name in ("row_offset_warp", "threads_per_row", "nmax_per_thread", "min_nz", "max_nz"):
        assert hasattr(wk.structure2, name), name
    for name in ("run", "run_x", "verify", "verify_x", "device_colinds", "device_values"):
        assert hasattr(wk.engine, name), name
    p = wk.profiler()
    p.add(1.0)
    p.add(3.0)
    assert p.avg() == 2.0 and p.count == 2
    s = wk.stats()
    s.add(2.0, "a")
    s.add(1.0, "b")
    s.add(5.0, "c")
    assert (s.Min(), s.Min_str(), s.Max(), s.Max_str()) == (1.0, "b", 5.0, "c")


def test_cpp_drop_in_header_compiles_and_links(tmp_path):
    """include/warpkernel.hpp and the driver written against it compile and
    link on a machine without a GPU (running it is a GPU test)."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not gxx or not os.path.exists(nvcc):
        pytest.skip("g++ or the CUDA toolkit is missing")
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    libdir = os.path.join(ROOT, "warpkernel_gb300")
    if not os.path.exists(os.path.join(libdir, "libwarpkernel_gb300.so")):
        pytest.skip("library not built")
    exe = str(tmp_path / "wpk_driver")
    cmd = [gxx, "-O1", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cpp", "wpk_driver.cpp"), "-o", exe,
           "-L", libdir, "-lwarpkernel_gb300", "-L", os.path.join(cuda, "lib64"), "-L", os.path.join(cuda, "lib"),
           "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
