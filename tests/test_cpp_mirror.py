"""The C++ mirror of gpuvmem's plugin surface (include/gpuvmem_gb300.hpp):
factory ids and error paths on the CPU, and on the GPU a main.cu-style run
through the mirror against the same run through the C ABI."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "gpuvmem_gb300")


def _build(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None or not os.path.exists(os.path.join(LIBDIR, "libgpuvmem_gb300.so")):
        pytest.skip("g++ or the built library is missing")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / "test_plugins")
    cmd = [cxx, "-std=c++17", "-O1", os.path.join(ROOT, "tests", "cpp", "test_plugins.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           "-L", LIBDIR, "-lgpuvmem_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{LIBDIR}", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_mirror_factory_and_errors(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_mirror_matches_c_abi_run(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
