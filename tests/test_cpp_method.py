"""The C++ host side (include/mhdvlct_method.hpp, the shape of a Cello glue
class) compiles against the C ABI and behaves like the reference's Method:
construction from the Method:mhd_vlct parameter text, the reference's
validation errors as exceptions (host only), and -- on a GPU -- one timestep
and compute that equal the plain C ABI's, and a two-level static mesh run
(refresh across levels, step with stored fluxes, flux correction) through the
class's mesh-level calls that conserves mass and energy to round-off."""
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


@pytest.mark.gpu
def test_cpp_smr_flux_correct(tmp_path):
    from mhdvlct import mesh as M
    exe = _build(tmp_path)
    n, g, root = 8, 4, 2
    mesh = M.Mesh((root,) * 3, refine=lambda lvl, c: c == (0, 0, 0))
    faces = mesh.face_ints()
    lines = [f"{len(mesh.leaves)} {n} {g} {root}"]
    for i, (lvl, _) in enumerate(mesh.leaves):
        lines.append(f"{lvl} " + " ".join(str(x) for x in mesh.origin(i, (n, n, n))))
    lines.append(str(len(faces)))
    lines += [" ".join(str(int(v)) for v in row) for row in faces]
    path = os.path.join(str(tmp_path), "mesh.txt")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    r = subprocess.run([exe, "--smr", path], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    words = r.stdout.split()
    mass, energy = float(words[words.index("mass") + 1]), float(words[words.index("energy") + 1])
    assert mass < 1e-15 and energy < 1e-15, r.stdout
