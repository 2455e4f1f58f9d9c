"""The C++ interface (grid2grid_gb300/include/grid2grid/*.hpp): the reference's
types and transform overloads over the C ABI. CPU: the test program in
tests/cpp/facade_test.cpp compiles against the headers and links the library.
GPU: it runs -- the reference's four scalapack2scalapack ctest cases and more,
with virtual ranks as threads calling transform collectively."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "grid2grid_gb300", "_lib")
EXE = os.path.join(ROOT, "grid2grid_gb300", "_build", "facade_test")


def _cuda_home():
    nv = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nv)))


def compile_driver():
    from grid2grid_gb300 import build
    build.build()
    cuda = _cuda_home()
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "grid2grid_gb300", "include"),
           "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "cpp", "facade_test.cpp"), "-o", EXE,
           "-L", LIB_DIR, "-lgrid2grid_gb300", f"-Wl,-rpath,{LIB_DIR}",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return EXE


def test_cpp_interface_compiles_and_links():
    assert os.path.exists(compile_driver())


@pytest.mark.gpu
def test_cpp_interface_runs_reference_style_driver():
    exe = compile_driver()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout
    assert r.stdout.count(": ok") >= 7
