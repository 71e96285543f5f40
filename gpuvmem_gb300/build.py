"""Build recipe of the in-tree CUDA library (nvcc, sm_103a only).

Compiles every translation unit of gpuvmem_gb300/csrc in parallel and links
gpuvmem_gb300/libgpuvmem_gb300.so.  Used by __graft_entry__.build() and by
`python -m gpuvmem_gb300.build`.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgpuvmem_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


# per-file flags (none at present: the line search rounds its operations
# separately through intrinsics, whatever the contraction setting)
FILE_FLAGS: dict = {}


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src, extra):
    obj = os.path.join(OBJ, src + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj, *FILE_FLAGS.get(src, []),
           *extra]
    if src.endswith(".cpp"):
        cmd += ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, extra=()):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        res = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [o for o, _ in res]
    if verbose:
        for _, err in res:
            if err.strip():
                print(err, file=sys.stderr)
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, extra=["-Xptxas", "-v"] if "-v" in sys.argv else []))
