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
