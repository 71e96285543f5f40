#!/bin/bash
# Builds oracle/_ref/ref_weights: the reference's weighting schemes
# (src/naturalweightingscheme.cu, src/uniformweightingscheme.cu,
# src/briggsweightingscheme.cu, read in place from the gpuvmem sources) linked
# with weights_main.cu.  Host code only; the stand-in headers under shim/
# replace casacore, cfitsio and boost.  Outputs go to oracle/_ref/ only.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${GV_REFERENCE:?set GV_REFERENCE to the gpuvmem source tree}"
OUT="$HERE/../_ref"
mkdir -p "$OUT/wobj"
FLAGS=(-std=c++17 -O2 -x cu -I "$HERE/shim" -I "$REF/include" -I "$REF/include/classes"
       -I "$REF/src" -Xcompiler -fopenmp -w)
for s in naturalweightingscheme uniformweightingscheme briggsweightingscheme; do
  nvcc "${FLAGS[@]}" -c "$REF/src/$s.cu" -o "$OUT/wobj/$s.o"
done
nvcc "${FLAGS[@]}" -c "$HERE/weights_main.cu" -o "$OUT/wobj/weights_main.o"
nvcc -o "$OUT/ref_weights" "$OUT/wobj/"*.o -Xcompiler -fopenmp
