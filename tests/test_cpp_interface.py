"""The C++ mirror of the reference's simulator interface (include/CCUDAParticleSimulator.hpp)
compiles against the C ABI here, and runs its checks on the GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_simulator.cpp")


def build_binary(sphlib, tmp_path):
    exe = str(tmp_path / "test_simulator")
    libdir = os.path.dirname(sphlib.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", libdir, "-lsph_gb300", "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_mirror_compiles(sphlib, tmp_path):
    assert os.path.exists(build_binary(sphlib, tmp_path))


@pytest.mark.gpu
def test_cpp_mirror_runs(sphlib, tmp_path):
    exe = build_binary(sphlib, tmp_path)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
