"""The C++ host side (include/mhdvlct_method.hpp, the shape of a Cello glue
class) compiles against the C ABI and behaves like the reference's Method:
construction from the Method:mhd_vlct parameter text, the reference's
validation errors as exceptions (host only), and -- on a GPU -- one timestep
and compute that equal the plain C ABI's."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "method_example.cpp")
LIBDIR = os.path.join(ROOT, "enzo-e_gb300")


def _build(tmp_path):
    exe = os.path.join(str(tmp_path), "method_example")
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), SRC, "-o", exe,
           "-L", LIBDIR, "-lmhdvlct_gb300", "-L", os.path.join(cuda, "lib64"),
           "-lcudart", "-Wl,-rpath," + LIBDIR, "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_method_host(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libmhdvlct_gb300.so")):
        pytest.skip("library not built")
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "cpp method ok" in r.stdout


@pytest.mark.gpu
def test_cpp_method_gpu(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "--gpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    assert "cpp method ok (gpu)" in r.stdout
