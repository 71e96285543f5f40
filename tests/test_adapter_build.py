"""The gpuvmem plugin adapter (gpuvmem_gb300/adapter/gvgb_plugins.cu) built
against gpuvmem's own headers -- include/classes/fi.cuh,
objectivefunction.cuh, optimizer.cuh, include/factory.cuh -- and linked
with libgpuvmem_gb300: gpuvmem's factories must hand out the adapter's
classes under gpuvmem's ids.  CPU only (no kernel runs).  Needs the gpuvmem
sources, located by GV_REFERENCE, and nvcc; casacore, cfitsio and boost are
replaced by the stand-in headers of oracle/ref_harness/shim."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("GV_REFERENCE", "")
LIB = os.path.join(ROOT, "gpuvmem_gb300", "libgpuvmem_gb300.so")

pytestmark = pytest.mark.skipif(
    not (REF and os.path.exists(os.path.join(REF, "include", "classes", "fi.cuh"))
         and shutil.which("nvcc") and os.path.exists(LIB)),
    reason="needs GV_REFERENCE (gpuvmem sources), nvcc and the built library")


def test_adapter_registers_under_gpuvmem_ids(tmp_path):
    inc = ["-I", os.path.join(ROOT, "oracle", "ref_harness", "shim"),
           "-I", os.path.join(REF, "include"), "-I", os.path.join(REF, "include", "classes"),
           "-I", os.path.join(REF, "src"), "-I", os.path.join(ROOT, "include")]
    flags = ["-std=c++17", "-x", "cu", "-Xcompiler", "-fopenmp", "-w"]
    objs = []
    for src in (os.path.join(ROOT, "gpuvmem_gb300", "adapter", "gvgb_plugins.cu"),
                os.path.join(ROOT, "tests", "cpp", "adapter_main.cu")):
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        subprocess.run(["nvcc", *flags, *inc, "-c", src, "-o", obj], check=True)
        objs.append(obj)
    exe = str(tmp_path / "adapter_test")
    libdir = os.path.dirname(LIB)
    subprocess.run(["nvcc", "-o", exe, *objs, "-L", libdir, "-lgpuvmem_gb300", "-Xcompiler",
                    "-fopenmp", "-Xlinker", f"-rpath={libdir}"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "adapter factory wiring ok" in r.stdout
