#!/bin/bash
# Builds oracle/_ref/ref_grid: the reference's convolutional gridding
# (do_gridding in src/functions.cu) and its convolution-kernel classes
# (src/pillBox2D.cu, src/gaussian2D.cu, src/sinc2D.cu, src/gaussianSinc2D.cu,
# src/pswf_12D.cu), read in place from the gpuvmem sources, linked with
# grid_main.cu.  Run on the host only; shim_host/ makes the kernel classes'
# CUDA calls non-fatal without a device, shim/ replaces casacore, cfitsio and
# boost.  Outputs go to oracle/_ref/ only.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${GV_REFERENCE:?set GV_REFERENCE to the gpuvmem source tree}"
OUT="$HERE/../_ref"
mkdir -p "$OUT/gobj"
FLAGS=(-std=c++17 -O2 -rdc=true -gencode arch=compute_103a,code=sm_103a
       -I "$HERE/shim_host" -I "$HERE/shim" -I "$REF/include" -I "$REF/include/classes"
       -I "$REF/src" -Xcompiler -fopenmp,-fpermissive -w)
pids=()
for s in functions complexOps pillBox2D gaussian2D sinc2D gaussianSinc2D pswf_12D; do
  nvcc "${FLAGS[@]}" -c "$REF/src/$s.cu" -o "$OUT/gobj/$s.o" & pids+=($!)
done
nvcc "${FLAGS[@]}" -c "$HERE/grid_main.cu" -o "$OUT/gobj/grid_main.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
nvcc -gencode arch=compute_103a,code=sm_103a -o "$OUT/ref_grid" "$OUT/gobj/"*.o -lcufft \
  -Xcompiler -fopenmp
