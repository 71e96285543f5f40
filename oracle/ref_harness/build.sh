#!/bin/bash
# Compiles the reference's own kernels (src/functions.cu and
# src/complexOps.cu of the gpuvmem sources at $GV_REFERENCE, read in place)
# into oracle/_ref/ref_kernels.cubin for sm_103a.  The stand-in headers under
# shim/ replace casacore, cfitsio, boost and the CUDA samples helper, which
# the kernels do not use.  Outputs go to oracle/_ref/ only.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${GV_REFERENCE:?set GV_REFERENCE to the gpuvmem source tree}"
OUT="$HERE/../_ref"
mkdir -p "$OUT"
nvcc -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 \
  -I "$HERE/shim" -I "$REF/include" -I "$REF/include/classes" -I "$REF/src" \
  -Xcompiler -fopenmp -w -o "$OUT/ref_kernels.cubin" "$HERE/ref_kernels.cu"
