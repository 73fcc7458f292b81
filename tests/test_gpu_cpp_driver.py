"""The C++ drop-in header (include/warpkernel.hpp) compiles and runs host
code shaped like the reference's wpk1.cu / wpk2.cu drivers."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def build_driver(tmp_path):
    libdir = os.path.join(ROOT, "warpkernel_gb300")
    exe = str(tmp_path / "wpk_driver")
    cuda = cuda_home()
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "cpp", "wpk_driver.cpp"), "-o", exe, "-L", libdir, "-lwarpkernel_gb300",
           "-L", os.path.join(cuda, "lib64"), "-L", os.path.join(cuda, "lib"), "-lcudart",
           f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_driver_wpk1_wpk2(tmp_path):
    exe = build_driver(tmp_path)
    for args in (["2", "64", "64", "0", "1"], ["3", "12", "12", "12", "3"]):
        r = subprocess.run([exe] + args + ["2"], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "driver passed: 0 failure(s)" in r.stdout


def test_cpp_driver_matrix_market_rowsort_assembly_layout_file(tmp_path):
    """The driver reading a Matrix Market file (wpk1.cu:43-48), then the
    rowsort variant, run_assembly and a layout file round trip."""
    from oracle import wk_oracle as O
    from test_formats import _write_mm
    exe = build_driver(tmp_path)
    rp, cols, vals = O.fe_matrix(3, 7, 6, 5, 2, value_mode=1, seed=3)
    n = len(rp) - 1
    ents = [(r + 1, int(cols[q]) + 1, float(vals[q])) for r in range(n) for q in range(rp[r], rp[r + 1])
            if cols[q] <= r]
    p = str(tmp_path / "fe.mtx")
    _write_mm(p, n, n, ents, sym="symmetric")
    r = subprocess.run([exe, "--mm", p, "2"], capture_output=True, text=True, timeout=180, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Finished Loading" in r.stdout and "driver passed: 0 failure(s)" in r.stdout
